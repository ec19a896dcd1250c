"""Lines longer than one register pass takes (c2c, more than 4096 points),
split in two passes (GPU): M = M1 * M2 with M2 a power of two; the first
pass transforms n2 and multiplies by W_M^(n1 k2), the second transforms n1
and writes X[k2 + M2 k1] (reference: FFTW plans of any length,
src/Transforms/c2c.jl:53-56).  Powers of two, 3 * 2^k and lengths whose
other factor goes through Bluestein; 1D with extra dimensions, along
strided axes, both output orders, in place, Float32 and double-float; each
against the oracle."""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T
from test_gpu_parity import check_plan

pytestmark = pytest.mark.gpu
F64, F32 = np.float64, np.float32


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("n", [8192, 16384, 24576, 5000, 1 << 20])
def test_long_c2c_lines(cuda, real, n):
    for tr in (T.FFT(), T.BFFT()):
        plan = P.PencilFFTPlan((n,), tr, real, extra_dims=(3,))
        assert plan.info.n_passes_forward == 2
        check_plan(plan, seed=n % 97)


@pytest.mark.parametrize("real", [F64, F32])
def test_long_lines_in_3d_layouts(cuda, real):
    for dims, tr in (((6, 16384), T.FFT()), ((8, 9000, 4), T.FFT()),
                     ((64, 12288), (T.RFFT(), T.FFT()))):
        for permute in (True, False):
            check_plan(P.PencilFFTPlan(dims, tr, real, permute_dims=permute), seed=5)


def test_long_line_in_place(cuda):
    check_plan(P.PencilFFTPlan((16384, 5), T.FFT_(), F64), seed=6)
