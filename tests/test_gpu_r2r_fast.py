"""REDFT00 (DCT-I) and RODFT00 (DST-I) on the register Stockham kernel (GPU).

Lines of n = 2^k + 1 (REDFT00) and n = 2^k - 1 (RODFT00) points are complex
DFTs of their even / odd extensions, whose length 2(n - 1) or 2(n + 1) is a
power of two: the kernel loads through the extension and stores the first n
outputs (times i for RODFT00).  Complex lines chain with neighbouring passes
in double-float form (first, middle and last pass of a run); real lines are
packed two per complex line.  Every case is checked against the oracle
(reference src/Transforms/r2r.jl; FFTW's REDFT00 / RODFT00 definitions) and
asserts that the R2R pass ran on the register kernel.
"""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, input_array, random_input
from test_gpu_parity import check_plan

pytestmark = pytest.mark.gpu
F64, F32 = np.float64, np.float32


def pass_kernels(plan, x):
    """Kernel names of the forward passes, by logical axis."""
    A = input_array(plan, x)
    plan.set_timing(True)
    plan * A
    rec = plan.get_timing()
    plan.set_timing(False)
    return {e["axis"]: e["kernel"] for e in rec if e["direction"] > 0}


def assert_fast_on(plan, axis):
    k = pass_kernels(plan, random_input(plan, 1))
    assert k[axis].startswith("fast_pass"), k


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("kind,n", [(T.REDFT00, 9), (T.REDFT00, 65), (T.REDFT00, 257), (T.REDFT00, 2049),
                                    (T.RODFT00, 7), (T.RODFT00, 63), (T.RODFT00, 511), (T.RODFT00, 2047)])
def test_r2r00_real_lines(cuda, real, kind, n):
    """1D real lines, an odd number of them (the last packed pair is half
    empty), as extra dimensions."""
    plan = P.PencilFFTPlan((n,), T.R2R(kind), real, extra_dims=(7,))
    check_plan(plan)
    assert_fast_on(plan, 0)


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("kind,n", [(T.REDFT00, 17), (T.REDFT00, 129), (T.RODFT00, 31), (T.RODFT00, 255)])
@pytest.mark.parametrize("pos", ["first", "middle", "last"])
def test_r2r00_complex_in_runs(cuda, real, kind, n, pos):
    """R2R on complex data as the first, middle or last pass of a run of
    register-kernel passes (dd-form input / output, per-line rescaling of the
    second pass of a Float64 run)."""
    if pos == "first":
        dims, tr, ax = (n, 16, 12), (T.R2R(kind), T.FFT(), T.FFT()), 0
    elif pos == "middle":
        dims, tr, ax = (16, n, 12), (T.FFT(), T.R2R(kind), T.FFT()), 1
    else:
        dims, tr, ax = (16, 12, n), (T.FFT(), T.FFT(), T.R2R(kind)), 2
    for permute in (True, False):
        plan = P.PencilFFTPlan(dims, tr, real, permute_dims=permute)
        check_plan(plan, seed=3)
        assert_fast_on(plan, ax)


@pytest.mark.parametrize("real", [F64, F32])
def test_taylor_green_like_rfft_fft_redft00(cuda, real):
    """The C3 transform tuple on a small grid, with extra dimensions."""
    plan = P.PencilFFTPlan((32, 16, 33), (T.RFFT(), T.FFT(), T.R2R(T.REDFT00)), real, extra_dims=(2,))
    check_plan(plan, seed=4)
    assert_fast_on(plan, 2)


@pytest.mark.parametrize("real", [F64, F32])
def test_all_r2r00_real_3d(cuda, real):
    """Three packed-real passes (not chained in dd form), mixed kinds and a
    non-power-of-two normalisation through the generic DCT-II along y."""
    plan = P.PencilFFTPlan((33, 12, 15), (T.R2R(T.REDFT00), T.R2R(T.REDFT10), T.R2R(T.RODFT00)), real)
    check_plan(plan, seed=5)
    k = pass_kernels(plan, random_input(plan, 1))
    assert k[0].startswith("fast_pass") and k[2].startswith("fast_pass"), k


@pytest.mark.parametrize("kind,n", [(T.REDFT00, 65), (T.RODFT00, 31)])
def test_r2r00_inplace(cuda, kind, n):
    """In-place R2R! on real data: every tile rewrites the lines it read."""
    plan = P.PencilFFTPlan((n, 10, 6), T.R2R_(kind), F64)
    check_plan(plan, seed=6)


@pytest.mark.parametrize("scale", [1e-200, 1e250])
def test_r2r00_wide_dynamic_range(cuda, scale):
    """Float64 data far from unit scale: the double-float run exponent keeps
    any finite double range inside the float exponent range."""
    from helpers import oracle_plan, rel
    plan = P.PencilFFTPlan((16, 65), (T.FFT(), T.R2R(T.REDFT00)), F64)
    x = random_input(plan, 8) * scale
    out = (plan * input_array(plan, x)).to_logical()
    assert rel(out, oracle_plan(plan).forward(x)) <= 1e-13
