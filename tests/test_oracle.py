"""Pins the CPU oracle: against the direct long-double definitions of
oracle/dft_direct.c, and against the analytic known answers of the reference's
tests (golden fixtures in tests/golden).  CPU only."""
import os

import numpy as np
import pytest

from oracle import direct as D
from oracle import pencilfft_oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SIZES = [1, 2, 3, 4, 5, 7, 8, 11, 12, 13, 16, 17, 23, 32, 41]


@pytest.mark.parametrize("n", SIZES)
def test_c2c_matches_definition(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    for tr, sign in ((O.FFT(), -1), (O.BFFT(), 1)):
        got = O.transform_1d(tr, x, 0)
        assert O.rel_l2(got, D.dft(x, sign)) < 1e-14


@pytest.mark.parametrize("n", SIZES)
def test_r2c_c2r_match_definition(n):
    rng = np.random.default_rng(100 + n)
    x = rng.standard_normal(n)
    assert O.rel_l2(O.transform_1d(O.RFFT(), x, 0), D.rfft(x)) < 1e-14
    X = rng.standard_normal(n // 2 + 1) + 1j * rng.standard_normal(n // 2 + 1)
    got = O.transform_1d(O.BRFFT(n), X, 0, n_out=n)
    # imaginary parts of DC / Nyquist do not contribute (both sides)
    assert O.rel_l2(got, D.brfft(X, n)) < 1e-14


@pytest.mark.parametrize("kind", O.R2R_SUPPORTED_KINDS)
@pytest.mark.parametrize("n", [n for n in SIZES if n >= 2])
def test_r2r_matches_definition(kind, n):
    rng = np.random.default_rng(1000 * kind + n)
    x = rng.standard_normal(n)
    got = O.transform_1d(O.R2R(kind), x, 0)
    assert O.rel_l2(got, D.r2r(x, kind)) < 1e-14
    # complex data: real and imaginary parts independently (reference r2r.jl:83-84)
    z = x + 1j * rng.standard_normal(n)
    gz = O.transform_1d(O.R2R(kind), z, 0)
    assert O.rel_l2(gz, D.r2r(z.real, kind) + 1j * D.r2r(z.imag, kind)) < 1e-14


@pytest.mark.parametrize("kind", O.R2R_SUPPORTED_KINDS)
def test_r2r_inverse_pairs(kind):
    """binv pairs and scale factors (reference r2r.jl:96-131)."""
    n = 9
    x = np.random.default_rng(kind).standard_normal(n)
    y = O.transform_1d(O.R2R(kind), x, 0)
    xb = O.transform_1d(O.binv(O.R2R(kind), n), y, 0)
    s = O.scale_factor_1d(O.binv(O.R2R(kind), n), n)
    assert O.rel_l2(xb / s, x) < 1e-14


def test_unsupported_r2r_kinds():
    for k in (O.R2HC, O.HC2R):
        with pytest.raises(ValueError):
            O.R2R(k)


@pytest.mark.parametrize("nz", [16, 17])
def test_brfft_single_mode_known_answer(nz):
    """reference test/brfft.jl:17-45."""
    g = np.load(os.path.join(GOLD, f"brfft_single_mode_{nz}.npz"))
    plan = O.OraclePlan((12, 13, 9), O.BRFFT((12, 13, nz)))
    assert plan.dims_out == (12, 13, nz)
    ur = plan.forward(g["uc"])
    assert O.rel_l2(ur, g["ur"]) < 1e-14
    back = plan.ldiv(ur)
    assert np.max(np.abs(back - g["uc"])) < 1e-8


@pytest.mark.parametrize("n0", [42, 41])
def test_rfft_known_answer(n0):
    """reference test/rfft.jl:213-231: x[1:3] == [1, 2, 0] after a round trip."""
    g = np.load(os.path.join(GOLD, f"rfft_known_answer_{n0}.npz"))
    dims = tuple(int(d) for d in g["dims"])
    x = np.zeros(dims)
    for idx, v in zip(g["nonzero"], g["values"]):
        x[tuple(idx)] = v
    plan = O.OraclePlan(dims, O.RFFT())
    back = plan.ldiv(plan.forward(x))
    assert np.allclose(back[:3, 0, 0], g["expect_first3"], atol=1e-8)


def _curl_spectral(uF, dims, L):
    kx = 2 * np.pi / L[0] * np.arange(dims[0] // 2 + 1)
    ky = 2 * np.pi / L[1] * np.fft.fftfreq(dims[1], 1.0 / dims[1])
    kz = 2 * np.pi / L[2] * np.fft.fftfreq(dims[2], 1.0 / dims[2])
    KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing="ij")
    return np.stack([1j * (KY * uF[2] - KZ * uF[1]),
                     1j * (KZ * uF[0] - KX * uF[2]),
                     1j * (KX * uF[1] - KY * uF[0])]), (KX, KY, KZ)


def test_taylor_green_known_answer():
    """reference test/taylor_green.jl:125-150: exact spectrum, zero divergence,
    exact vorticity after plan \\ curl(uF)."""
    g = np.load(os.path.join(GOLD, "taylor_green_16_8_16.npz"))
    dims = (16, 8, 16)
    plan = O.OraclePlan(dims, O.RFFT())
    uF = np.stack([plan.forward(c) for c in g["u"]])
    assert O.max_abs(uF, g["uF"]) < 1e-12
    wF, (KX, KY, KZ) = _curl_spectral(uF, dims, g["L"])
    div = KX * uF[0] + KY * uF[1] + KZ * uF[2]
    assert np.sum(np.abs(div) ** 2) / np.prod(dims) < 1e-16
    w = np.stack([plan.ldiv(c) for c in wF])
    assert np.sum((w - g["w"]) ** 2) < 1e-16 * 1e3  # summed squared error


@pytest.mark.parametrize("dims", [(42, 24, 16), (41, 23, 15)])
def test_parseval(dims):
    """reference test/rfft.jl:21-43 with scale == Ngrid."""
    u = np.random.default_rng(7).standard_normal(dims)
    plan = O.OraclePlan(dims, O.RFFT())
    assert plan.scale == np.prod(dims)
    uF = plan.forward(u)
    w = np.full(uF.shape[0], 2.0)
    w[0] = 1.0
    if dims[0] % 2 == 0:
        w[-1] = 1.0
    s_phys = np.sum(u ** 2) / np.prod(dims)
    s_spec = np.sum(w[:, None, None] * np.abs(uF) ** 2) / (np.prod(dims) * plan.scale)
    assert abs(s_phys - s_spec) < 1e-12 * s_phys


def test_oracle_memory_layout_roundtrip():
    plan = O.OraclePlan((4, 5, 6), O.FFT(), extra_dims=(2,))
    x = np.arange(4 * 5 * 6 * 2).reshape(4, 5, 6, 2)
    for out in (False, True):
        assert np.array_equal(plan.from_memory(plan.to_memory(x, out), out), x)
    # natural memory: dimension 1 fastest; output: dimension N fastest
    assert plan.to_memory(x, False).shape == (2, 6, 5, 4)
    assert plan.to_memory(x, True).shape == (2, 4, 5, 6)


def test_longdouble_oracle_agrees():
    dims = (12, 10, 6)
    u = np.random.default_rng(3).standard_normal(dims)
    a = O.OraclePlan(dims, O.RFFT()).forward(u)
    b = O.OraclePlan(dims, O.RFFT(), longdouble=True).forward(u)
    assert O.rel_l2(a, b) < 1e-15
