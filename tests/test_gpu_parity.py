"""GPU parity against the CPU oracle, over the cases of the reference's tests
(test/transforms.jl, test/rfft.jl, test/brfft.jl) and the configurations of the
benchmark.  Every call goes through the C ABI of libpencilfft_gb300.so."""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import TOL, T, input_array, oracle_plan, random_input, rel

pytestmark = pytest.mark.gpu

F64, F32 = np.float64, np.float32
R2R_KINDS = T.R2R_SUPPORTED_KINDS


def check_plan(plan, seed=0, tol=None):
    tol = TOL[np.dtype(plan.real_type)] if tol is None else tol
    orc = oracle_plan(plan)
    x = random_input(plan, seed)
    A = input_array(plan, x)
    ref_out = orc.forward(x)
    if plan.is_inplace():
        plan * A
        out = A.last().to_logical()
    else:
        B = plan * A
        out = B.to_logical()
        # out-of-place forward leaves its input untouched
        assert np.array_equal(A.to_logical(), x)
    e_fwd = rel(out, ref_out)
    assert e_fwd <= tol, f"forward rel L2 {e_fwd:.3e} > {tol}"
    # backward (ldiv!): round trip and against the oracle
    if plan.is_inplace():
        plan.ldiv(A)
        back = A.first().to_logical()
    else:
        Bin = B.to_logical()
        back_arr = plan.ldiv(B)
        back = back_arr.to_logical()
        assert np.array_equal(B.to_logical(), Bin), "backward clobbered its input"
    e_rt = rel(back, x)
    assert e_rt <= tol, f"round trip rel L2 {e_rt:.3e} > {tol}"
    e_bwd = rel(back, orc.ldiv(ref_out))
    assert e_bwd <= tol, f"backward rel L2 {e_bwd:.3e} > {tol}"
    return e_fwd, e_rt


# -- test/transforms.jl: DATA_DIMS = (16, 12, 6), every transform kind --------------
SIZE_IN = (16, 12, 6)
PAIRS = [
    T.FFT(), T.RFFT(), T.BFFT(), T.NoTransform(),
    *[T.R2R(k) for k in R2R_KINDS],
    (T.NoTransform(), T.RFFT(), T.FFT()),
    (T.FFT(), T.NoTransform(), T.FFT()),
    (T.FFT(), T.NoTransform(), T.NoTransform()),
    T.BRFFT(SIZE_IN),
]


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("edims", [(), (3,)])
@pytest.mark.parametrize("tr", PAIRS, ids=repr)
def test_transforms_16_12_6(cuda, tr, real, edims):
    plan = P.PencilFFTPlan(SIZE_IN, tr, real, extra_dims=edims)
    check_plan(plan)


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("edims", [(), (3,)])
def test_inplace_fft(cuda, real, edims):
    plan = P.PencilFFTPlan(SIZE_IN, T.FFT_(), real, extra_dims=edims)
    check_plan(plan)


def test_inplace_fft_notransform(cuda):
    plan = P.PencilFFTPlan(SIZE_IN, (T.FFT_(), T.FFT_(), T.NoTransform_()))
    check_plan(plan)


# -- test/transforms.jl:439-462: dimensionality, permute_dims ---------------------------
@pytest.mark.parametrize("dims", [(11, 15), (11, 7, 13), (9, 7, 5, 12)])
@pytest.mark.parametrize("permute", [True, False])
@pytest.mark.parametrize("tr", [T.RFFT(), T.FFT_(), T.FFT()], ids=repr)
def test_dimensionality(cuda, dims, permute, tr):
    plan = P.PencilFFTPlan(dims, tr, F64, permute_dims=permute)
    check_plan(plan)


# -- test/rfft.jl: even and odd sizes, in-place RFFT! ---------------------------------
@pytest.mark.parametrize("dims", [(42, 24, 16), (41, 23, 15)])
@pytest.mark.parametrize("tr", [T.RFFT(), T.RFFT_()], ids=repr)
def test_rfft_even_odd(cuda, dims, tr):
    plan = P.PencilFFTPlan(dims, tr, F64)
    check_plan(plan)


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("dims", [(1,), (2,), (3,), (5, 1), (1, 7), (2, 3, 1), (4, 16, 1), (1, 16, 4), (4, 1, 16)])
def test_small_and_unit_sizes(cuda, dims, real):
    """Transforms along dimensions of one point (identity lines, no stage)."""
    for tr in (T.FFT(), T.RFFT(), T.BFFT()):
        for permute in (True, False):
            check_plan(P.PencilFFTPlan(dims, tr, real, permute_dims=permute))


@pytest.mark.parametrize("precision", ["default", "fx", "native"])
@pytest.mark.parametrize("dims", [(16, 12, 6), (64, 32, 16), (8, 4096), (4096, 3), (512, 8, 2)])
@pytest.mark.parametrize("tr", [T.RFFT(), T.FFT(), T.BFFT(), T.RFFT_(), T.FFT_()], ids=repr)
def test_pow2_fast_path(cuda, dims, tr, precision):
    """Power-of-two lines (register Stockham kernel), every Float64 arithmetic
    (double-float, block floating point, native FP64)."""
    plan = P.PencilFFTPlan(dims, tr, F64, precision=precision)
    check_plan(plan)
    if precision == "default":
        check_plan(P.PencilFFTPlan(dims, tr, F32))


@pytest.mark.parametrize("permute", [True, False])
@pytest.mark.parametrize("edims", [(), (2,)])
def test_fast_path_layouts(cuda, permute, edims):
    for tr in (T.RFFT(), T.FFT(), T.BRFFT((32, 16, 64))):
        check_plan(P.PencilFFTPlan((32, 16, 33) if isinstance(tr, T.BRFFT) else (32, 16, 64), tr, F64,
                                   permute_dims=permute, extra_dims=edims))


@pytest.mark.parametrize("precision", ["default", "fx"])
def test_dd_wide_dynamic_range(cuda, precision):
    """Float64 data far outside the float exponent range keeps full accuracy."""
    plan = P.PencilFFTPlan((64, 32, 16), T.RFFT(), F64, precision=precision)
    orc = oracle_plan(plan)
    rng = np.random.default_rng(5)
    for scale in (1e-200, 1e250):
        x = rng.standard_normal((64, 32, 16)) * scale
        A = input_array(plan, x)
        B = plan * A
        assert rel(B.to_logical(), orc.forward(x)) <= 1e-13
        assert rel(plan.ldiv(B).to_logical(), x) <= 1e-13


@pytest.mark.parametrize("precision", ["default", "fx"])
@pytest.mark.parametrize("dims, tr", [((64, 32, 16), T.RFFT()), ((16, 8, 4, 6), T.FFT()),
                                      ((8, 64), (T.FFT(), T.FFT()))])
def test_dd_line_scales(cuda, dims, tr, precision):
    """Float64 runs scale each line by its own largest exponent (dd: the
    first pass's lines, rescaled to the run exponent in the next pass; fx:
    every pass's lines): lines whose magnitudes differ by up to 1e+-60 within
    one array, and all-zero lines, keep the 1e-13 bound (forward against the
    oracle and round trip), in both directions."""
    plan = P.PencilFFTPlan(dims, tr, F64, precision=precision)
    orc = oracle_plan(plan)
    rng = np.random.default_rng(11)
    x = random_input(plan, 11)
    line_scale = 10.0 ** rng.uniform(-60, 60, size=(1,) + tuple(dims[1:]))
    line_scale[..., 0] = 0.0  # some lines all zero
    x = x * line_scale
    B = plan * input_array(plan, x)
    assert rel(B.to_logical(), orc.forward(x)) <= 1e-13
    assert rel(plan.ldiv(B).to_logical(), x) <= 1e-13


@pytest.mark.parametrize("n", [7, 11, 13, 17, 23, 41, 53, 97, 191, 384, 1000, 1024, 2048])
@pytest.mark.parametrize("real", [F64, F32])
def test_1d_lengths(cuda, n, real):
    """Mixed radices, primes (Bluestein) and long lines along one axis, batched."""
    plan = P.PencilFFTPlan((n, 5), (T.FFT(), T.NoTransform()), real)
    check_plan(plan)
    plan = P.PencilFFTPlan((3, n), (T.FFT(), T.FFT()), real)
    check_plan(plan)
