"""Bluestein register pass (GPU): c2c, r2c and c2r lines of any length up
to 2048 that are neither powers of two nor 3 * 2^k / 5 * 2^k, as a chirp
convolution through two power-of-two register transforms.  Primes, odd and
even composite lengths, contiguous and strided axes, both output orders,
partial tiles, Float32 and double-float Float64; each case against the
oracle (reference FFTW plans of any length, src/Transforms/c2c.jl:53-56,
r2c.jl:83-96) and asserting that the Bluestein kernel ran."""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, input_array, oracle_plan, random_input, rel
from test_gpu_parity import check_plan

pytestmark = pytest.mark.gpu
F64, F32 = np.float64, np.float32


def kernels(plan):
    A = input_array(plan, random_input(plan, 1))
    plan.set_timing(True)
    B = plan * A
    plan.ldiv(B)
    rec = plan.get_timing()
    plan.set_timing(False)
    return {(e["direction"], e["axis"]): e["kernel"] for e in rec}


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("n", [2, 3, 7, 12, 17, 56, 97, 101, 127, 191, 1000, 1021, 2047])
def test_bs_1d_lines(cuda, real, n):
    """FFT and RFFT (odd and even lengths: the c2r extension of n // 2 + 1
    inputs) along one axis, 7 lines."""
    for tr in (T.FFT(), T.RFFT()):
        plan = P.PencilFFTPlan((n,), tr, real, extra_dims=(7,))
        check_plan(plan, seed=n)
        k = kernels(plan)
        assert k[(1, 0)].startswith("bs_pass") and k[(-1, 0)].startswith("bs_pass"), k


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("dims,tr", [((97, 20, 12), T.RFFT()), ((20, 101, 7), T.FFT()),
                                     ((12, 10, 131), T.FFT()), ((53, 47, 59), T.RFFT()),
                                     ((63, 64, 96), (T.RFFT(), T.FFT(), T.FFT()))],
                         ids=["x-r2c", "y-strided", "z-last", "all-bs", "bs-pow2-mr"])
def test_bs_3d_layouts(cuda, real, dims, tr):
    for permute in (True, False):
        plan = P.PencilFFTPlan(dims, tr, real, permute_dims=permute)
        check_plan(plan, seed=2)


def test_bs_float64_line_scales(cuda):
    """Per-line exponents of the double-float Bluestein pass: lines 1e+-150
    apart and an all-zero line, each checked against the oracle on its own."""
    n, h = 97, 6
    plan = P.PencilFFTPlan((n,), T.FFT(), F64, extra_dims=(h,))
    x = random_input(plan, 9) * np.array([1e150, 1.0, 1e-150, 3e-100, 0.0, 1e20])[None, :]
    out = (plan * input_array(plan, x)).to_logical()
    ref = oracle_plan(plan).forward(x)
    for j in range(h):
        if j == 4:
            assert np.all(out[:, j] == 0)
        else:
            assert rel(out[:, j], ref[:, j]) <= 1e-13, j


def test_bs_derivative_falls_back_to_generic(cuda):
    """A fused derivative on a Bluestein-eligible first backward pass runs on
    the generic kernel and stays correct."""
    from oracle import pencilfft_oracle as O
    dims = (16, 12, 97)
    plan = P.PencilFFTPlan(dims, T.FFT(), F32)
    orc = oracle_plan(plan)
    spec = orc.forward(random_input(plan, 4))
    S = plan.allocate_output()
    S.copy_from_logical(spec)
    U = plan.allocate_input()
    P.ldiv_(U, plan, S, deriv=(3, 2.0))
    assert rel(U.to_logical(), orc.ldiv(O.wavenumbers(orc, 2, 2.0) * spec)) <= 2e-6


@pytest.mark.parametrize("real", [F64, F32])
def test_bs_planner_measurement(cuda, real):
    """fftw_flags = FFTW.MEASURE times the Bluestein pass against the generic
    kernel for these lines and keeps the faster; the result matches the
    oracle whichever is kept."""
    plan = P.PencilFFTPlan((97, 40, 12), T.RFFT(), real, fftw_flags=P.FFTW_MEASURE)
    check_plan(plan, seed=12)
