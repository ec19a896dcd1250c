"""Spectral derivatives fused into the transform (GPU): the multiply by i k of
the reference's gradient / curl helpers (examples/gradient.jl,
test/include/FourierOperations.jl) done in the first backward or last forward
pass, against the oracle; and the Taylor-Green vorticity of
test/taylor_green.jl:125-150 computed with fused derivatives."""
import os

import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, TOL, input_array, oracle_plan, random_input, rel
from oracle import pencilfft_oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("real", [np.float64, np.float32])
@pytest.mark.parametrize("dims,tr", [((64, 32, 48), T.RFFT()), ((32, 24, 40), T.FFT()),
                                     ((30, 20, 12), T.RFFT()), ((16, 32, 64), T.RFFT())],
                         ids=["rfft-pow2", "fft", "rfft-generic", "rfft-c1"])
def test_fused_derivative_matches_oracle(cuda, dims, tr, real):
    plan = P.PencilFFTPlan(dims, tr, real)
    orc = oracle_plan(plan)
    rng = np.random.default_rng(9)
    shape = dims
    if plan.eltype_input().kind == "c":
        x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    else:
        x = rng.standard_normal(shape)
    x = x.astype(plan.eltype_input())
    L = (2 * np.pi, 3.0, 5.5)
    A = input_array(plan, x)
    for d in range(3):
        ik = O.wavenumbers(orc, d, L[d])
        B = plan.allocate_output()
        P.mul_(B, plan, A, deriv=(d + 1, L[d]))
        assert rel(B.to_logical(), ik * orc.forward(x)) <= TOL[np.dtype(real)]
        spec = orc.forward(x)
        S = plan.allocate_output()
        S.copy_from_logical(spec)
        before = S.to_logical()
        U = plan.allocate_input()
        P.ldiv_(U, plan, S, deriv=(d + 1, L[d]))
        assert np.array_equal(S.to_logical(), before)  # the spectrum is not modified
        assert rel(U.to_logical(), orc.ldiv(ik * spec)) <= TOL[np.dtype(real)]


@pytest.mark.parametrize("dims,tr", [((64, 32, 48), T.RFFT()), ((32, 24, 40), T.FFT())],
                         ids=["rfft", "fft-mixed"])
def test_fused_derivative_block_float_plan(cuda, dims, tr):
    """A Float64 plan in block floating point (precision="fx") runs a fused
    derivative with its double-float kernels; plain executions of the same
    plan before and after stay in fx, match the oracle and repeat bit for
    bit."""
    plan = P.PencilFFTPlan(dims, tr, np.float64, precision="fx")
    orc = oracle_plan(plan)
    x = random_input(plan, 13)
    A = input_array(plan, x)
    spec = orc.forward(x)
    B0 = plan * A
    assert rel(B0.to_logical(), spec) <= 1e-13
    L = (2 * np.pi, 3.0)
    B = plan.allocate_output()
    P.mul_(B, plan, A, deriv=(1, L[0]))
    assert rel(B.to_logical(), O.wavenumbers(orc, 0, L[0]) * spec) <= 1e-13
    U = plan.allocate_input()
    P.ldiv_(U, plan, B0, deriv=(2, L[1]))
    assert rel(U.to_logical(), orc.ldiv(O.wavenumbers(orc, 1, L[1]) * spec)) <= 1e-13
    assert np.array_equal((plan * A).to_logical(), B0.to_logical())
    assert rel(plan.ldiv(B0).to_logical(), x) <= 1e-13


def test_taylor_green_vorticity_fused(cuda):
    g = np.load(os.path.join(GOLD, "taylor_green_16_8_16.npz"))
    dims = (16, 8, 16)
    Ls = tuple(float(v) for v in g["L"])
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float64)
    u = plan.allocate_input(P.Val(3))
    for c, x in zip(u, g["u"]):
        c.copy_from_logical(x)
    uF = plan * u
    tmp = plan.allocate_input()

    def d(comp, dim):  # physical derivative of component comp along dim (1-based)
        P.ldiv_(tmp, plan, uF[comp], deriv=(dim, Ls[dim - 1]))
        return tmp.to_logical()
    w = [d(2, 2) - d(1, 3), d(0, 3) - d(2, 1), d(1, 1) - d(0, 2)]
    err = sum(np.sum((wi - wr) ** 2) for wi, wr in zip(w, g["w"]))
    assert err < 1e-16 * 1e3   # reference test/taylor_green.jl:148-149 (summed squared error)
    # divergence is zero
    div = d(0, 1) + d(1, 2) + d(2, 3)
    assert np.max(np.abs(div)) < 1e-12


def test_derivative_errors(cuda):
    plan = P.PencilFFTPlan((16, 12), (T.R2R(T.REDFT10), T.FFT()), np.float64)
    A = plan.allocate_input()
    B = plan.allocate_output()
    with pytest.raises(P.ArgumentError, match="FFT, BFFT, RFFT or BRFFT"):
        P.mul_(B, plan, A, deriv=(1, 1.0))
    with pytest.raises(P.ArgumentError):
        P.mul_(B, plan, A, deriv=(3, 1.0))
    # the multiply needs a complex-to-complex pass at that end of the plan
    plan1 = P.PencilFFTPlan((32,), T.RFFT(), np.float64)
    with pytest.raises(P.LibraryError, match="complex-to-complex"):
        P.mul_(plan1.allocate_output(), plan1, plan1.allocate_input(), deriv=(1, 1.0))
    planb = P.PencilFFTPlan((16, 12, 9), T.BRFFT(16), np.float64)
    with pytest.raises(P.LibraryError, match="complex-to-complex"):
        P.mul_(planb.allocate_output(), planb, planb.allocate_input(), deriv=(1, 1.0))


# -- fused sums of derivatives: divergence and curl in one backward transform each --
@pytest.mark.parametrize("real", [np.float64, np.float32])
@pytest.mark.parametrize("dims,tr", [((64, 32, 48), T.RFFT()), ((32, 24, 40), T.FFT()),
                                     ((30, 20, 12), T.RFFT()), ((16, 64, 8), T.RFFT())],
                         ids=["rfft-pow2", "fft", "rfft-generic", "rfft-tiles"])
def test_fused_divergence_and_curl_match_oracle(cuda, dims, tr, real):
    """dst = plan \\ sum_t c_t i k_t uF_t against the oracle, for the
    divergence (three terms) and the three curl components (two terms each),
    on power-of-two (register kernel) and generic first backward passes."""
    plan = P.PencilFFTPlan(dims, tr, real)
    orc = oracle_plan(plan)
    rng = np.random.default_rng(21)
    L = (2 * np.pi, 3.0, 5.5)
    specs = [orc.forward(random_input(plan, 30 + c)) for c in range(3)]
    uF = []
    for s in specs:
        S = plan.allocate_output()
        S.copy_from_logical(s)
        uF.append(S)
    before = [S.to_logical() for S in uF]
    ik = [O.wavenumbers(orc, d, L[d]) for d in range(3)]
    tol = TOL[np.dtype(real)]
    div = plan.allocate_input()
    P.ldiv_divergence_(div, plan, uF, L)
    ref = orc.ldiv(ik[0] * specs[0] + ik[1] * specs[1] + ik[2] * specs[2])
    assert rel(div.to_logical(), ref) <= tol
    om = plan.allocate_input(P.Val(3))
    P.ldiv_curl_(om, plan, uF, L)
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        ref = orc.ldiv(ik[b] * specs[c] - ik[c] * specs[b])
        assert rel(om[a].to_logical(), ref) <= tol, a
    for S, b0 in zip(uF, before):
        assert np.array_equal(S.to_logical(), b0)  # sources untouched
    # bmul! form and a single term with a coefficient
    U = plan.allocate_input()
    P.ldiv_deriv_sum_(U, plan, [(uF[1], 2, -2.5, L[1])], normalise=False)
    assert rel(U.to_logical(), orc.bmul(-2.5 * ik[1] * specs[1])) <= tol


def test_taylor_green_fused_divergence_and_curl(cuda):
    """reference test/taylor_green.jl:125-150: zero divergence and the exact
    vorticity, each from one fused backward transform."""
    g = np.load(os.path.join(GOLD, "taylor_green_16_8_16.npz"))
    dims = (16, 8, 16)
    Ls = tuple(float(v) for v in g["L"])
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float64)
    u = plan.allocate_input(P.Val(3))
    for c, x in zip(u, g["u"]):
        c.copy_from_logical(x)
    uF = plan * u
    div = plan.allocate_input()
    P.ldiv_divergence_(div, plan, uF, Ls)
    assert np.max(np.abs(div.to_logical())) < 1e-12
    om = plan.allocate_input(P.Val(3))
    P.ldiv_curl_(om, plan, uF, Ls)
    err = sum(np.sum((o.to_logical() - wr) ** 2) for o, wr in zip(om, g["w"]))
    assert err < 1e-16 * 1e3  # reference test/taylor_green.jl:148-149


def test_derivative_sum_errors(cuda):
    plan = P.PencilFFTPlan((16, 12, 8), T.RFFT(), np.float64)
    A = plan.allocate_input()
    B = plan.allocate_output()
    with pytest.raises(P.ArgumentError, match="1 to 3 terms"):
        P.ldiv_deriv_sum_(A, plan, [(B, 1, 1.0, 1.0)] * 4)
    with pytest.raises(P.ArgumentError):
        P.ldiv_deriv_sum_(A, plan, [(B, 4, 1.0, 1.0)])
    pip = P.PencilFFTPlan((16, 12, 8), T.FFT_(), np.float64)
    M = pip.allocate_input()
    with pytest.raises(P.ArgumentError):
        P.ldiv_deriv_sum_(M, pip, [(M, 1, 1.0, 1.0)])
