"""ctypes binding of the C ABI declared in include/pencilfft_gb300.h.

The library is the only compute path: if it cannot be loaded, every transform
call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

MAX_DIMS = 8
MAX_EXTRA = 4

OK = 0
ERR_ARGUMENT = -1
ERR_UNSUPPORTED = -2
ERR_CUDA = -3
ERR_ALLOC = -4

KIND_FFT, KIND_BFFT, KIND_RFFT, KIND_BRFFT, KIND_R2R, KIND_NOTRANSFORM = range(6)


class PlanDesc(ctypes.Structure):
    _fields_ = [
        ("ndims", ctypes.c_int32),
        ("dims", ctypes.c_int64 * MAX_DIMS),
        ("kind", ctypes.c_int32 * MAX_DIMS),
        ("inplace", ctypes.c_int32 * MAX_DIMS),
        ("r2r_kind", ctypes.c_int32 * MAX_DIMS),
        ("brfft_even", ctypes.c_int32 * MAX_DIMS),
        ("real_bytes", ctypes.c_int32),
        ("permute_dims", ctypes.c_int32),
        ("n_extra", ctypes.c_int32),
        ("extra_dims", ctypes.c_int64 * MAX_EXTRA),
        ("precision_mode", ctypes.c_int32),
        ("autotune", ctypes.c_int32),
    ]


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("ndims", ctypes.c_int32),
        ("dims_in", ctypes.c_int64 * MAX_DIMS),
        ("dims_out", ctypes.c_int64 * MAX_DIMS),
        ("perm_out", ctypes.c_int32 * MAX_DIMS),
        ("eltype_in_complex", ctypes.c_int32),
        ("eltype_out_complex", ctypes.c_int32),
        ("real_bytes", ctypes.c_int32),
        ("inplace", ctypes.c_int32),
        ("scale_factor", ctypes.c_double),
        ("input_bytes", ctypes.c_int64),
        ("output_bytes", ctypes.c_int64),
        ("inplace_bytes", ctypes.c_int64),
        ("scratch_bytes", ctypes.c_int64),
        ("n_passes_forward", ctypes.c_int32),
        ("n_passes_backward", ctypes.c_int32),
    ]


class PassTiming(ctypes.Structure):
    _fields_ = [
        ("direction", ctypes.c_int32),
        ("pass_", ctypes.c_int32),
        ("axis", ctypes.c_int32),
        ("op", ctypes.c_int32),
        ("launches", ctypes.c_int32),
        ("total_ms", ctypes.c_double),
        ("bytes_per_launch", ctypes.c_int64),
        ("kernel", ctypes.c_char * 48),
    ]


class BatchOp(ctypes.Structure):
    _fields_ = [
        ("plan", ctypes.c_void_p),
        ("direction", ctypes.c_int32),
        ("normalise", ctypes.c_int32),
        ("dst", ctypes.c_void_p),
        ("src", ctypes.c_void_p),
        ("deriv_dim", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("deriv_length", ctypes.c_double),
    ]


class BatchInfo(ctypes.Structure):
    _fields_ = [
        ("form", ctypes.c_int32),
        ("transforms", ctypes.c_int32),
        ("items", ctypes.c_int32),
        ("grid", ctypes.c_int32),
        ("tiles", ctypes.c_int64),
        ("smem", ctypes.c_int64),
        ("graph_ms", ctypes.c_double),
        ("persistent_ms", ctypes.c_double),
        ("wave_bytes", ctypes.c_int64),
    ]


BATCH_GRAPH, BATCH_PERSISTENT, BATCH_AUTO, BATCH_MEASURE = 0, 1, 2, 3

# Every symbol the header declares, with (restype, argtypes).
_vp = ctypes.c_void_p
SIGNATURES = {
    "pfgb_plan_create": (ctypes.c_int, [ctypes.POINTER(PlanDesc), ctypes.POINTER(_vp)]),
    "pfgb_plan_query": (ctypes.c_int, [ctypes.POINTER(PlanDesc), ctypes.POINTER(PlanInfo)]),
    "pfgb_plan_destroy": (ctypes.c_int, [_vp]),
    "pfgb_plan_info_get": (ctypes.c_int, [_vp, ctypes.POINTER(PlanInfo)]),
    "pfgb_forward": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "pfgb_backward": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int]),
    "pfgb_forward_deriv": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_double]),
    "pfgb_backward_deriv": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    "pfgb_backward_deriv_sum": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(_vp), ctypes.c_int,
                                               ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                               ctypes.POINTER(ctypes.c_double), _vp, ctypes.c_int]),
    "pfgb_execute_many": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp),
                                         ctypes.POINTER(_vp), ctypes.c_int, _vp]),
    "pfgb_batch_create": (ctypes.c_int, [ctypes.POINTER(_vp), ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_vp),
                                         ctypes.POINTER(_vp), ctypes.c_int, ctypes.POINTER(_vp)]),
    "pfgb_batch_launch": (ctypes.c_int, [_vp, _vp]),
    "pfgb_batch_destroy": (ctypes.c_int, [_vp]),
    "pfgb_batch_create_ex": (ctypes.c_int, [ctypes.POINTER(BatchOp), ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(_vp)]),
    "pfgb_batch_get_info": (ctypes.c_int, [_vp, ctypes.POINTER(BatchInfo)]),
    "pfgb_batch_status": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(ctypes.c_int32)]),
    "pfgb_batch_set_wait_test": (ctypes.c_int, [_vp, ctypes.c_int]),
    "pfgb_plan_set_timing": (ctypes.c_int, [_vp, ctypes.c_int]),
    "pfgb_plan_get_timing": (ctypes.c_int, [_vp, ctypes.POINTER(PassTiming), ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_int)]),
    "pfgb_fft1d_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _vp, _vp, _vp]),
    "pfgb_device_status": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(ctypes.c_int32)]),
    "pfgb_plan_set_wait_test": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "pfgb_wisdom_export": (ctypes.c_int, [ctypes.c_char_p]),
    "pfgb_wisdom_import": (ctypes.c_int, [ctypes.c_char_p]),
    "pfgb_wisdom_forget": (ctypes.c_int, []),
    "pfgb_wisdom_stats": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "pfgb_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "pfgb_version": (ctypes.c_char_p, []),
}

_LIB = None
_BUILD_ERROR = None


def lib_path() -> str:
    """The in-tree library, or the file named by PENCILFFT_GB300_LIB."""
    return os.environ.get("PENCILFFT_GB300_LIB") or _build.LIB


def load(build_if_missing: bool = True):
    """Loads the shared library (building it first if it is missing or stale)."""
    global _LIB, _BUILD_ERROR
    if _LIB is not None:
        return _LIB
    if _BUILD_ERROR is not None:
        raise RuntimeError(f"libpencilfft_gb300.so failed to build: {_BUILD_ERROR}")
    if build_if_missing and not os.environ.get("PENCILFFT_GB300_LIB") and not _build.up_to_date():
        try:
            _build.build()
        except Exception as e:  # keep the first failure; do not rebuild on every call
            _BUILD_ERROR = str(e)[:2000]
            raise
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError(f"libpencilfft_gb300.so not found at {path}; run the build first")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def last_error() -> str:
    L = load()
    buf = ctypes.create_string_buffer(4096)
    L.pfgb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class ArgumentError(ValueError):
    """Mirrors Julia's ArgumentError raised by the reference."""


class LibraryError(RuntimeError):
    pass


def check(rc: int, what: str = ""):
    if rc == OK:
        return
    msg = last_error()
    if rc == ERR_ARGUMENT:
        raise ArgumentError(msg)
    raise LibraryError(f"{what}: status {rc}: {msg}")
