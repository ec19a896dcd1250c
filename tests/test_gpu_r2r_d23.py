"""REDFT10 / REDFT01 (DCT-II / DCT-III), RODFT10 / RODFT01 (DST-II /
DST-III), the DHT and REDFT11 / RODFT11 (DCT-IV / DST-IV) of power-of-two
length on the register Stockham kernel (GPU).  The DHT is the DCT-II's
post-processing with w = (1 + i) / 2 on the DFT of the line in order; the
DCT-IV / DST-IV are one 2n-point DFT of the pre-twiddled, zero-padded line
with a paired post-twiddle.

A line of n points is one n-point complex DFT: DCT-II of the reordered line
v[m] = x[2m], v[n-1-m] = x[2m+1] followed by Y[k] = w_k V[k] + conj(w_k)
V[n-k] (w_k = exp(-i pi k / 2n)); DCT-III by the transposed steps; the DST
kinds alternate signs and reverse.  Complex lines chain with neighbouring
passes in double-float form; real lines are packed two per complex line.
Every case is checked against the oracle (reference src/Transforms/r2r.jl,
FFTW's definitions; the backward transforms are the inverse kinds, so every
round trip exercises both directions) and asserts that the pass ran on the
register kernel.
"""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, input_array, oracle_plan, random_input, rel
from test_gpu_parity import check_plan
from test_gpu_r2r_fast import assert_fast_on

pytestmark = pytest.mark.gpu
F64, F32 = np.float64, np.float32
KINDS = [T.REDFT10, T.REDFT01, T.RODFT10, T.RODFT01, T.DHT, T.REDFT11, T.RODFT11]


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("kind", KINDS, ids=["REDFT10", "REDFT01", "RODFT10", "RODFT01", "DHT", "REDFT11", "RODFT11"])
@pytest.mark.parametrize("n", [8, 16, 64, 512, 4096])
def test_d23_real_lines(cuda, real, kind, n):
    """1D real lines, an odd number of them (the last packed pair is half
    empty), as extra dimensions."""
    if kind in (T.REDFT11, T.RODFT11) and n == 4096:
        n = 2048  # (a 2n-point DFT: up to 2048 points on the register pass)
    plan = P.PencilFFTPlan((n,), T.R2R(kind), real, extra_dims=(5,))
    check_plan(plan)
    assert_fast_on(plan, 0)


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("kind", KINDS, ids=["REDFT10", "REDFT01", "RODFT10", "RODFT01", "DHT", "REDFT11", "RODFT11"])
@pytest.mark.parametrize("pos", ["first", "middle", "last"])
def test_d23_complex_in_runs(cuda, real, kind, pos):
    """R2R on complex data as the first, middle or last pass of a run of
    register-kernel passes (dd-form input / output, per-line rescaling of the
    second pass of a Float64 run), with both output orders."""
    n = 32
    if pos == "first":
        dims, tr, ax = (n, 16, 12), (T.R2R(kind), T.FFT(), T.FFT()), 0
    elif pos == "middle":
        dims, tr, ax = (16, n, 12), (T.FFT(), T.R2R(kind), T.FFT()), 1
    else:
        dims, tr, ax = (16, 12, n), (T.FFT(), T.FFT(), T.R2R(kind)), 2
    for permute in (True, False):
        plan = P.PencilFFTPlan(dims, tr, real, permute_dims=permute)
        check_plan(plan, seed=5)
        assert_fast_on(plan, ax)


@pytest.mark.parametrize("real", [F64, F32])
def test_d23_mixed_real_3d(cuda, real):
    """Three packed-real passes of different kinds on a 3D grid, with extra
    dimensions, both output orders."""
    tr = (T.R2R(T.REDFT11), T.R2R(T.RODFT01), T.R2R(T.DHT))
    for permute in (True, False):
        plan = P.PencilFFTPlan((16, 64, 8), tr, real, permute_dims=permute, extra_dims=(3,))
        check_plan(plan, seed=6)
        for ax in range(3):
            assert_fast_on(plan, ax)


def test_d23_rfft_fft_dct2_float64(cuda):
    """RFFT, FFT and DCT-II on a larger Float64 grid (a Taylor-Green style
    tuple with a DCT-II along z)."""
    plan = P.PencilFFTPlan((64, 48, 128), (T.RFFT(), T.FFT(), T.R2R(T.REDFT10)), F64)
    check_plan(plan, seed=7)
    assert_fast_on(plan, 2)


@pytest.mark.parametrize("kind", [T.REDFT10, T.RODFT01, T.REDFT11], ids=["REDFT10", "RODFT01", "REDFT11"])
def test_d23_float64_line_scales(cuda, kind):
    """Double-float runs through a DCT-II / DST-III pass: lines whose
    magnitudes differ by up to 1e+-60 within one array, and all-zero lines,
    keep the 1e-13 bound over the array (forward against the oracle and round
    trip), as for the c2c runs (test_dd_line_scales)."""
    dims = (16, 64, 12)
    plan = P.PencilFFTPlan(dims, (T.FFT(), T.R2R(kind), T.FFT()), F64)
    orc = oracle_plan(plan)
    rng = np.random.default_rng(12)
    x = random_input(plan, 12) * (10.0 ** rng.uniform(-60, 60, size=(1,) + dims[1:]))
    x[..., 0] = 0.0
    B = plan * input_array(plan, x)
    assert rel(B.to_logical(), orc.forward(x)) <= 1e-13
    assert rel(plan.ldiv(B).to_logical(), x) <= 1e-13
