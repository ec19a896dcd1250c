"""Lines longer than one register pass takes (c2c, more than 4096 points),
split in two passes (GPU): M = M1 * M2 with M2 a power of two; the first
pass transforms n2 and multiplies by W_M^(n1 k2), the second transforms n1
and writes X[k2 + M2 k1] (reference: FFTW plans of any length,
src/Transforms/c2c.jl:53-56).  Powers of two, 3 * 2^k and lengths whose
other factor goes through Bluestein; 1D with extra dimensions, along
strided axes, both output orders, in place, Float32 and double-float; each
against the oracle.

Real lines longer than 4096 points (r2c / c2r): two real lines packed as one
complex line z = x1 + i x2 (r2c) or Z = X1 + i X2 over both Hermitian
extensions (c2r), the n-point c2c transform of the packed line in two
passes, and a separating map; an odd number of lines (the last pair has no
second line), a single line, strided and permuted axes, in place
(reference src/Transforms/r2c.jl:83-101, src/multiarrays_r2c.jl:69-79).

Lengths without a split (no power-of-two factor of at least 8 with a
one-pass cofactor) beyond the generic kernel's core run as a Bluestein
convolution through two split power-of-two transforms; R2R lines whose
extension is beyond that core gather the extension into packed complex lines
around one long c2c transform (reference src/Transforms/r2r.jl:5-131)."""
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
                     ((64, 12288), (T.RFFT(), T.FFT())),
                     ((6, 16384), (T.NoTransform(), T.FFT()))):
        for permute in (True, False):
            check_plan(P.PencilFFTPlan(dims, tr, real, permute_dims=permute), seed=5)


def test_long_line_in_place(cuda):
    check_plan(P.PencilFFTPlan((16384, 5), T.FFT_(), F64), seed=6)


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("n", [8192, 16384, 5000, 24576, 1 << 20])
def test_long_real_lines(cuda, real, n):
    """RFFT lines with an odd number of them (3, extra dimension), a single
    line, and the BRFFT of n outputs as the forward transform."""
    for dims, edims in (((n,), (3,)), ((n,), ())):
        plan = P.PencilFFTPlan(dims, T.RFFT(), real, extra_dims=edims)
        assert plan.info.n_passes_forward == 4
        check_plan(plan, seed=n % 89)
    plan = P.PencilFFTPlan((n // 2 + 1,), T.BRFFT(n), real, extra_dims=(2,))
    assert plan.info.n_passes_forward == 4
    check_plan(plan, seed=n % 83)


@pytest.mark.parametrize("real", [F64, F32])
def test_long_real_lines_in_layouts(cuda, real):
    """Long r2c lines in 2D / 3D plans with both output orders (the
    separating map writes the permuted output), along a strided axis after a
    NoTransform, and an even, odd and single count of pairs."""
    for dims, tr in (((16384, 6), T.RFFT()), ((9000, 5, 3), T.RFFT()),
                     ((12288, 1, 4), T.RFFT()), ((6, 16384), (T.NoTransform(), T.RFFT())),
                     ((5, 8192, 3), (T.NoTransform(), T.RFFT(), T.FFT()))):
        for permute in (True, False):
            check_plan(P.PencilFFTPlan(dims, tr, real, permute_dims=permute), seed=7)


@pytest.mark.parametrize("real", [F64, F32])
def test_long_real_lines_in_place(cuda, real):
    """RFFT! on the padded in-place buffer (ManyPencilArray) with long lines."""
    for dims in ((16384, 5), (8192, 4, 3)):
        check_plan(P.PencilFFTPlan(dims, T.RFFT_(), real), seed=8)


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("n", [4097, 8209, 100003])
def test_long_c2c_bluestein(cuda, real, n):
    """Prime and two-prime lengths: chirp map, split forward transform,
    filter product, split inverse transform, chirp map."""
    for tr in (T.FFT(), T.BFFT()):
        plan = P.PencilFFTPlan((n,), tr, real, extra_dims=(2,))
        assert plan.info.n_passes_forward == 7
        check_plan(plan, seed=n % 79)


@pytest.mark.parametrize("real", [F64, F32])
def test_long_real_bluestein(cuda, real):
    """r2c / c2r lines whose packed c2c line takes the Bluestein form, in 1D
    (odd number of lines), 2D with both output orders, and the BRFFT of an
    odd output length."""
    check_plan(P.PencilFFTPlan((8209,), T.RFFT(), real, extra_dims=(3,)), seed=3)
    for permute in (True, False):
        check_plan(P.PencilFFTPlan((8209, 4), T.RFFT(), real, permute_dims=permute), seed=4)
    check_plan(P.PencilFFTPlan((4105,), T.BRFFT(8209), real, extra_dims=(2,)), seed=5)


# per kind: (extension with a split, extension through Bluestein)
R2R_LONG = {T.DHT: (9000, 8209), T.REDFT00: (8193, 8194), T.RODFT00: (8191, 8190),
            T.REDFT10: (5000, 4099), T.REDFT01: (5000, 4099), T.REDFT11: (5000, 4099),
            T.RODFT10: (5000, 4099), T.RODFT01: (5000, 4099), T.RODFT11: (5000, 4099)}


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("kind", list(R2R_LONG), ids=lambda k: repr(T.R2R(k)))
def test_long_r2r_lines(cuda, real, kind):
    """R2R lines with an extension beyond one pass: real lines (packed in
    pairs, an odd count) and complex lines after an FFT, one output order per
    length (both orders per kind)."""
    for n, permute in zip(R2R_LONG[kind], (True, False)):
        check_plan(P.PencilFFTPlan((n,), T.R2R(kind), real, extra_dims=(3,)), seed=n % 71)
        check_plan(P.PencilFFTPlan((4, n), (T.FFT(), T.R2R(kind)), real, permute_dims=permute), seed=n % 67)


@pytest.mark.parametrize("real", [F64, F32])
def test_many_pass_plan_and_in_place_r2r(cuda, real):
    """A plan of more than 12 passes (Bluestein lines along both axes: the
    scratch buffers alternate) with both output orders, and in-place R2R!
    lines whose extension is beyond one pass."""
    for permute in (True, False):
        plan = P.PencilFFTPlan((4097, 4099), T.FFT(), real, permute_dims=permute)
        assert plan.info.n_passes_forward == 14
        check_plan(plan, seed=9)
    check_plan(P.PencilFFTPlan((8193, 3), T.R2R_(T.REDFT00), real), seed=10)
    check_plan(P.PencilFFTPlan((5000, 4), T.R2R_(T.RODFT10), real), seed=11)


def test_long_lines_in_a_batch(cuda):
    """Long-line plans recorded into a batch: the graph form replays the
    element maps with the passes; the persistent form has no tile for them
    (LibraryError), and "auto" falls back to the graph form."""
    import torch
    from helpers import oracle_plan, rel
    plans = [P.PencilFFTPlan((16384, 3), T.RFFT(), F32), P.PencilFFTPlan((8209,), T.FFT(), F32, extra_dims=(2,))]
    rng = np.random.default_rng(12)
    us = [p.allocate_input() for p in plans]
    vs = [p.allocate_output() for p in plans]
    ws = [p.allocate_input() for p in plans]
    xs = []
    for p, u in zip(plans, us):
        x = rng.standard_normal(tuple(p.size_global_in) + tuple(p.extra_dims))
        if np.dtype(p.eltype_input()).kind == "c":
            x = x + 1j * rng.standard_normal(x.shape)
        u.copy_from_logical(x)
        xs.append(x)
    ops = [(P.mul_, v, p, u) for p, u, v in zip(plans, us, vs)] + \
          [(P.ldiv_, w, p, v) for p, v, w in zip(plans, vs, ws)]
    with pytest.raises(P.LibraryError):
        P.Batch(ops, form="persistent")
    for form in ("graph", "auto"):
        b = P.Batch(ops, form=form)
        assert b.form == "graph"
        b.launch()
        torch.cuda.synchronize()
        for p, x, v, w in zip(plans, xs, vs, ws):
            assert rel(v.to_logical(), oracle_plan(p).forward(x)) <= 1e-5
            assert rel(w.to_logical(), x) <= 1e-5
        assert b.status() == 0
