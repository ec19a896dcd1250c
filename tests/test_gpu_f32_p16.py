"""Float32 lines of 1024 points and more take 16 points per thread (radix-16
register stages: two shared-memory exchanges for a 1024-point line instead of
three) (GPU): c2c, r2c and c2r along contiguous and strided axes, both output
orders, partial tiles, in place, fused derivatives; against the oracle at the
Float32 tolerance."""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, TOL, input_array, oracle_plan, random_input, rel
from oracle import pencilfft_oracle as O
from test_gpu_parity import check_plan

pytestmark = pytest.mark.gpu
F32 = np.float32


@pytest.mark.parametrize("dims,tr", [((1024, 6, 5), T.RFFT()), ((6, 1024, 5), T.FFT()),
                                     ((5, 3, 2048), T.FFT()), ((2048, 9), T.RFFT()),
                                     ((4096, 5), T.BFFT()), ((1024, 1024), T.RFFT())],
                         ids=["x-r2c", "y-strided", "z-2048", "r2c-2048", "bfft-4096", "2d-1024"])
def test_p16_layouts(cuda, dims, tr):
    for permute in (True, False):
        check_plan(P.PencilFFTPlan(dims, tr, F32, permute_dims=permute), seed=7)


def test_p16_in_place(cuda):
    check_plan(P.PencilFFTPlan((1024, 10, 3), T.RFFT_(), F32), seed=8)
    check_plan(P.PencilFFTPlan((6, 2048), T.FFT_(), F32), seed=8)


def test_p16_fused_derivative(cuda):
    dims = (8, 6, 1024)
    plan = P.PencilFFTPlan(dims, T.FFT(), F32)
    orc = oracle_plan(plan)
    x = random_input(plan, 9)
    spec = orc.forward(x)
    B = plan.allocate_output()
    P.mul_(B, plan, input_array(plan, x), deriv=(3, 4.0))
    assert rel(B.to_logical(), O.wavenumbers(orc, 2, 4.0) * spec) <= TOL[np.dtype(F32)]
    S = plan.allocate_output()
    S.copy_from_logical(spec)
    U = plan.allocate_input()
    P.ldiv_(U, plan, S, deriv=(3, 4.0))
    assert rel(U.to_logical(), orc.ldiv(O.wavenumbers(orc, 2, 4.0) * spec)) <= TOL[np.dtype(F32)]
