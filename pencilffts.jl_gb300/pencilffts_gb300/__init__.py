"""GB300 (sm_103a) implementation of the PencilFFTs.jl transform path.

The API mirrors the reference's ``PencilFFTPlan`` / ``Transforms`` interface at
``proc_dims = (1, ..., 1)``; all transform arithmetic runs in the CUDA library
``libpencilfft_gb300.so`` behind the C ABI of ``include/pencilfft_gb300.h``.
"""
from . import transforms as Transforms
from ._lib import ArgumentError, LibraryError, load as load_library
from .plans import (FFTW_ESTIMATE, FFTW_EXHAUSTIVE, FFTW_MEASURE, FFTW_PATIENT, Batch,
                    ManyPencilArray, Pencil, PencilArray, PencilFFTPlan, Val,
                    allocate_input, allocate_output, bmul_, export_wisdom, forget_wisdom,
                    gather, import_wisdom, is_inplace, wisdom_stats,
                    ldiv, ldiv_, ldiv_curl_, ldiv_deriv_sum_, ldiv_divergence_, mul_,
                    plan_query, scale_factor)

__all__ = [
    "Transforms", "Batch", "ArgumentError", "LibraryError", "load_library", "ManyPencilArray",
    "Pencil", "PencilArray", "PencilFFTPlan", "Val", "allocate_input", "allocate_output",
    "bmul_", "gather", "is_inplace", "ldiv", "ldiv_", "ldiv_curl_", "ldiv_deriv_sum_",
    "ldiv_divergence_", "mul_", "plan_query", "scale_factor", "export_wisdom", "import_wisdom",
    "forget_wisdom", "wisdom_stats",
    "FFTW_ESTIMATE", "FFTW_MEASURE", "FFTW_PATIENT", "FFTW_EXHAUSTIVE",
]
