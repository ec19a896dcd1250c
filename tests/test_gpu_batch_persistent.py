"""Persistent batch form (GPU): every tile of every pass of every transform of
a batch in one launch of a work-list kernel, with bounded dependency waits.
The batches follow the reference's collections of fields (mul!/ldiv! over
tuples and arrays, src/operations.jl:129-152) and the spectral-derivative
example (examples/gradient.jl): each output against the FP64 oracle, and the
form that ran asserted."""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, input_array, oracle_plan, rel

pytestmark = pytest.mark.gpu
F32 = np.float32
TOL = 2e-6


def _sync():
    import torch
    torch.cuda.synchronize()


def _round_trips(sizes, form, seed=5):
    rng = np.random.default_rng(seed)
    plans = [P.PencilFFTPlan(d, T.RFFT(), F32) for d in sizes]
    xs = [rng.standard_normal(d).astype(F32) for d in sizes]
    us = [input_array(p, x) for p, x in zip(plans, xs)]
    vs = [p.allocate_output() for p in plans]
    ws = [p.allocate_input() for p in plans]
    ops = []
    for p, u, v, w in zip(plans, us, vs, ws):
        ops += [(P.mul_, v, p, u), (P.ldiv_, w, p, v)]
    return plans, xs, vs, ws, P.Batch(ops, form=form)


# lengths of every tile form: powers of two (register tile), 3 * 2^k with
# 2^k >= 128 (mixed-radix tile), 3 * 2^k and 5 * 2^k below that, primes and
# other composites (Bluestein tile)
SIZES = [(64, 48, 53), (96, 128, 80), (384, 20, 18), (97, 100, 36), (191, 12, 160), (50, 72, 127),
         (8, 9, 10), (2, 3, 256)]


@pytest.mark.parametrize("form", ["persistent", "graph"])
def test_uneven_round_trips(cuda, form):
    plans, xs, vs, ws, batch = _round_trips(SIZES, form)
    info = batch.info()
    assert info["form"] == form
    if form == "persistent":
        assert info["items"] == 6 * len(SIZES) and info["tiles"] >= info["items"] and info["grid"] > 0
    batch.launch()
    _sync()
    for p, x, v, w in zip(plans, xs, vs, ws):
        assert rel(v.to_logical(), oracle_plan(p).forward(x)) <= TOL
        assert rel(w.to_logical(), x) <= TOL
    assert batch.status() == 0


def test_replay_with_new_contents(cuda):
    rng = np.random.default_rng(3)
    sizes = [(48, 64, 50), (96, 60, 72), (64, 64, 64), (53, 128, 40)]
    plans = [P.PencilFFTPlan(d, T.RFFT(), F32) for d in sizes]
    us = [p.allocate_input() for p in plans]
    vs = [p.allocate_output() for p in plans]
    ws = [p.allocate_input() for p in plans]
    ops = [(P.mul_, v, p, u) for p, u, v in zip(plans, us, vs)] + \
          [(P.ldiv_, w, p, v) for p, v, w in zip(plans, vs, ws)]
    batch = P.Batch(ops, form="persistent")
    for _ in range(2):
        xs = [rng.standard_normal(d).astype(F32) for d in sizes]
        for u, x in zip(us, xs):
            u.copy_from_logical(x)
        batch.launch()
        _sync()
        for p, v, w, x in zip(plans, vs, ws, xs):
            assert rel(v.to_logical(), oracle_plan(p).forward(x)) <= TOL
            assert rel(w.to_logical(), x) <= TOL


def test_vector_gradient_with_fused_derivatives(cuda):
    """The spectral gradient of examples/gradient.jl as one batch: per
    component c, r2c then c2r of i k_c times the spectrum (the multiply fused
    into the first backward pass), on a grid with a 3 * 2^7 axis (mixed-radix
    tile), a power-of-two axis and a prime axis (Bluestein tile)."""
    from oracle import pencilfft_oracle as O
    dims = (384, 32, 29)
    plan = P.PencilFFTPlan(dims, T.RFFT(), F32)
    rng = np.random.default_rng(8)
    xs = [rng.standard_normal(dims).astype(F32) for _ in range(3)]
    us = [input_array(plan, x) for x in xs]
    vs = [plan.allocate_output() for _ in range(3)]
    ds = [plan.allocate_input() for _ in range(3)]
    L = 2 * np.pi
    ops = []
    for c in range(3):
        ops += [(P.mul_, vs[c], plan, us[c]), (P.ldiv_, ds[c], plan, vs[c], (c + 1, L))]
    batch = P.Batch(ops, form="persistent")
    batch.launch()
    _sync()
    orc = oracle_plan(plan)
    for c in range(3):
        ref = orc.ldiv(orc.forward(xs[c]) * O.wavenumbers(orc, c, L))
        assert rel(ds[c].to_logical(), ref) <= TOL, c


def test_complex_fields_and_forward_derivative(cuda):
    """c2c forward with the derivative fused into the last forward pass, then
    the plain backward; lengths on all three tile forms."""
    from oracle import pencilfft_oracle as O
    dims = (768, 24, 31)
    plan = P.PencilFFTPlan(dims, T.FFT(), F32)
    rng = np.random.default_rng(4)
    x = (rng.standard_normal(dims) + 1j * rng.standard_normal(dims)).astype(np.complex64)
    u = input_array(plan, x)
    v, w = plan.allocate_output(), plan.allocate_input()
    batch = P.Batch([(P.mul_, v, plan, u, (3, 5.0)), (P.ldiv_, w, plan, v)], form="persistent")
    batch.launch()
    _sync()
    orc = oracle_plan(plan)
    ref = orc.forward(x) * O.wavenumbers(orc, 2, 5.0)
    assert rel(v.to_logical(), ref) <= TOL
    assert rel(w.to_logical(), orc.ldiv(ref)) <= TOL


def test_order_across_plans_through_buffers(cuda):
    """Transforms of different plans that share buffers run in dependency
    order inside the one launch: B = F(A), then C = F(B) on a second plan (read
    after write), and A overwritten by F(D) on a third plan only after F(A)
    read it (write after read)."""
    dims = (32, 24, 20)
    p1 = P.PencilFFTPlan(dims, T.FFT(), F32)
    p2 = P.PencilFFTPlan(tuple(reversed(dims)), T.FFT(), F32, permute_dims=False)
    p3 = P.PencilFFTPlan(dims, T.FFT(), F32)
    rng = np.random.default_rng(17)
    xa = (rng.standard_normal(dims) + 1j * rng.standard_normal(dims)).astype(np.complex64)
    xd = (rng.standard_normal(dims) + 1j * rng.standard_normal(dims)).astype(np.complex64)
    A, D = input_array(p1, xa), input_array(p1, xd)
    B, C = p1.allocate_output(), p1.allocate_output()
    Bv = P.PencilArray(p2.pencil_input(), B.data, B.dtype)
    Cv = P.PencilArray(p2.pencil_output(), C.data, C.dtype)
    Av = P.PencilArray(p3.pencil_output(), A.data.view(p3.pencil_output().memory_shape()), A.dtype)
    batch = P.Batch([(P.mul_, B, p1, A), (P.mul_, Cv, p2, Bv), (P.mul_, Av, p3, D)], form="persistent")
    batch.launch()
    _sync()
    o1 = oracle_plan(p1)
    fa = o1.forward(xa)
    assert rel(B.to_logical(), fa) <= TOL
    # C holds the 3D FFT of F(A) taken in memory order (reversed dimensions)
    assert rel(Cv.to_logical(), np.fft.fftn(fa.transpose(2, 1, 0))) <= TOL
    assert rel(Av.to_logical(), o1.forward(xd)) <= TOL


def test_forms_agree(cuda):
    """The graph and persistent forms of the same batch give the same
    results to Float32 rounding."""
    a = _round_trips(SIZES[:4], "graph", seed=9)
    b = _round_trips(SIZES[:4], "persistent", seed=9)
    for r in (a, b):
        r[4].launch()
    _sync()
    for va, vb in zip(a[2], b[2]):
        assert rel(vb.to_logical(), va.to_logical()) <= TOL
    for wa, wb in zip(a[3], b[3]):
        assert rel(wb.to_logical(), wa.to_logical()) <= TOL


def test_unsupported_plans_fall_back(cuda):
    """Float64 plans and Float32 passes without a tile form (R2R, lines above
    1024 points) have no persistent form: "persistent" raises, "auto" records
    the graph form."""
    cases = [((24, 20, 16), T.FFT(), np.float64), ((16, 12, 10), T.R2R(T.REDFT10), F32),
             ((2048, 4, 4), T.FFT(), F32)]
    for dims, tr, real in cases:
        p = P.PencilFFTPlan(dims, tr, real)
        u, v = p.allocate_input(), p.allocate_output()
        with pytest.raises(P.LibraryError):
            P.Batch([(P.mul_, v, p, u)], form="persistent")
        b = P.Batch([(P.mul_, v, p, u)], form="auto")
        assert b.form == "graph"
        with pytest.raises(P.ArgumentError):
            b.set_wait_test(1)


def test_dependency_wait_gives_up_and_recovers(cuda):
    """A dependency wait bounded at one poll gives up: status bit 8, the
    launch stops early and returns; with the default bound the next launch
    is complete and correct, and the status is clear."""
    plans, xs, vs, ws, batch = _round_trips(SIZES[:3], "persistent", seed=21)
    batch.set_wait_test(1)
    batch.launch()
    assert batch.status() == 8
    batch.set_wait_test(0)
    batch.launch()
    _sync()
    assert batch.status() == 0
    for p, x, v, w in zip(plans, xs, vs, ws):
        assert rel(v.to_logical(), oracle_plan(p).forward(x)) <= TOL
        assert rel(w.to_logical(), x) <= TOL


def test_measured_form(cuda):
    """form="measure" times both forms at creation and keeps the faster; the
    kept form's results match the oracle."""
    plans, xs, vs, ws, batch = _round_trips(SIZES[:4], "measure", seed=2)
    info = batch.info()
    assert info["graph_ms"] > 0 and info["persistent_ms"] > 0
    assert info["form"] == ("persistent" if info["persistent_ms"] <= info["graph_ms"] else "graph")
    batch.launch()
    _sync()
    for p, x, v, w in zip(plans, xs, vs, ws):
        assert rel(v.to_logical(), oracle_plan(p).forward(x)) <= TOL
        assert rel(w.to_logical(), x) <= TOL


def test_auto_form(cuda):
    """form="auto" records the persistent form when every pass has a tile
    form; the default form is the graph form."""
    plans, xs, vs, ws, batch = _round_trips([(12, 20, 16), (24, 9, 30)], "auto", seed=1)
    assert batch.form == "persistent"
    batch.launch()
    _sync()
    for p, x, v, w in zip(plans, xs, vs, ws):
        assert rel(v.to_logical(), oracle_plan(p).forward(x)) <= TOL
        assert rel(w.to_logical(), x) <= TOL
    p = plans[0]
    assert P.Batch([(P.mul_, vs[0], p, p.allocate_input())]).form == "graph"


def test_single_transform_and_inplace_plans(cuda):
    """A batch of one transform, and an in-place FFT! plan's forward and
    backward on one ManyPencilArray (reference test/transforms.jl:177-256),
    each in the forms it records under "auto"; results against the oracle."""
    plan = P.PencilFFTPlan((24, 20, 9), T.RFFT(), F32)
    rng = np.random.default_rng(6)
    x = rng.standard_normal((24, 20, 9)).astype(F32)
    u, v = input_array(plan, x), plan.allocate_output()
    one = P.Batch([(P.mul_, v, plan, u)], form="persistent")
    one.launch()
    _sync()
    assert rel(v.to_logical(), oracle_plan(plan).forward(x)) <= TOL

    ip = P.PencilFFTPlan((16, 12, 6), T.FFT_(), F32)
    vi = ip.allocate_input()
    xi = (rng.standard_normal((16, 12, 6)) + 1j * rng.standard_normal((16, 12, 6))).astype(np.complex64)
    vi.first().copy_from_logical(xi)
    b = P.Batch([(P.mul_, vi, ip, vi), (P.ldiv_, vi, ip, vi)], form="auto")
    assert b.form in ("graph", "persistent")
    b.launch()
    _sync()
    assert rel(vi.first().to_logical(), xi) <= TOL
    f = P.Batch([(P.mul_, vi, ip, vi)], form="auto")
    vi.first().copy_from_logical(xi)
    f.launch()
    _sync()
    assert rel(vi.last().to_logical(), oracle_plan(ip).forward(xi)) <= TOL


def test_empty_and_malformed_batches(cuda):
    plan = P.PencilFFTPlan((8, 8, 8), T.RFFT(), F32)
    u, v = plan.allocate_input(), plan.allocate_output()
    with pytest.raises(P.ArgumentError):
        P.Batch([])
    with pytest.raises(P.ArgumentError):
        P.Batch([(P.mul_, v, plan, u)], form="fastest")
    with pytest.raises(P.ArgumentError):
        P.Batch([(P.mul_, v, plan)])
    with pytest.raises(P.ArgumentError):
        P.Batch([(P.ldiv_, u, plan, v, (4, 1.0))])
