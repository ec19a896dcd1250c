"""API behaviour on the GPU, following the reference's tests:
test/transforms.jl:145-256 (in-place plans, collections, errors) and
:465-509 (incompatibility between plans and arrays), test/rfft.jl:194-256
(RFFT! vs RFFT, known answer), plus the batched (CUDA graph) form."""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, input_array, oracle_plan, random_input, rel

pytestmark = pytest.mark.gpu


def test_incompatibility(cuda):
    """reference test/transforms.jl:465-509 (ArgumentError cases)."""
    dims, dims_other = (10, 8), (6, 8)
    plan = P.PencilFFTPlan(dims, T.FFT())
    plan_ = P.PencilFFTPlan(dims, T.FFT_())
    u = plan.allocate_input()
    v = plan.allocate_output()
    with pytest.raises(P.ArgumentError, match="incompatible with in-place plans"):
        plan_ * u
    M_ = plan_.allocate_input()
    assert isinstance(M_, P.ManyPencilArray)
    with pytest.raises(P.ArgumentError, match="incompatible with out-of-place plans"):
        plan * M_
    with pytest.raises(P.ArgumentError, match="incompatible with in-place plans"):
        P.mul_(v, plan_, u)
    with pytest.raises(P.ArgumentError, match="incompatible with out-of-place plans"):
        P.mul_(M_, plan, M_)
    with pytest.raises(P.ArgumentError, match="aliased"):
        P.mul_(u, plan, u)
    u3 = plan.allocate_input(P.Val(3))
    v2 = plan.allocate_output(P.Val(2))
    with pytest.raises(P.ArgumentError, match="collections have different lengths: 2 ≠ 3"):  # length(dst) first, as check_compatible(dst, src) formats it
        P.mul_(v2, plan, u3)
    plan_other = P.PencilFFTPlan(dims_other, T.FFT())
    with pytest.raises(P.ArgumentError, match="unexpected dimensions of input data"):
        plan_other * u
    v_other = plan_other.allocate_output()
    with pytest.raises(P.ArgumentError, match="unexpected dimensions of output data"):
        P.mul_(v_other, plan, u)


def test_inplace_manypencilarray(cuda):
    """reference test/transforms.jl:177-256."""
    plan = P.PencilFFTPlan((16, 12, 6), T.FFT_())
    plan_oop = P.PencilFFTPlan((16, 12, 6), T.FFT())
    vi = plan.allocate_input()
    u, v = vi.first(), vi.last()
    x = random_input(plan, 3)
    u.copy_from_logical(x)
    with pytest.raises(P.ArgumentError):
        plan_oop * vi
    with pytest.raises(P.ArgumentError):
        P.mul_(v, plan_oop, u)
    with pytest.raises(P.ArgumentError, match="must be the same"):
        P.mul_(plan.allocate_input(), plan, vi)
    with pytest.raises(P.ArgumentError):
        plan * u
    plan * vi
    assert not np.allclose(u.to_logical(), x)  # u was modified
    assert rel(v.to_logical(), oracle_plan(plan).forward(x)) <= 1e-13
    plan.ldiv(vi)
    assert rel(u.to_logical(), x) <= 1e-13
    # components: Val(3) and (3, 2)
    for comp in ((P.Val(3),), (3, 2)):
        vs = plan.allocate_input(*comp)
        flat = vs if isinstance(vs, tuple) else [a for row in vs for a in row]
        xs = [random_input(plan, 10 + i) for i in range(len(flat))]
        for a, xx in zip(flat, xs):
            a.first().copy_from_logical(xx)
        plan * vs
        plan.ldiv(vs)
        for a, xx in zip(flat, xs):
            assert rel(a.first().to_logical(), xx) <= 1e-13


@pytest.mark.parametrize("dims", [(42, 24, 16), (41, 23, 15)])
def test_rfft_inplace_vs_outofplace_known_answer(cuda, dims):
    """reference test/rfft.jl:194-256."""
    ip = P.PencilFFTPlan(dims, T.RFFT_())
    oop = P.PencilFFTPlan(dims, T.RFFT())
    u = ip.allocate_input()
    x, xh = u.first(), u.last()
    v = oop.allocate_input()
    vh = oop.allocate_output()
    z = np.zeros(dims)
    z[0, 0, 0], z[1, 0, 0] = 1.0, 2.0
    x.copy_from_logical(z)
    v.copy_from_logical(z)
    P.mul_(u, ip, u)
    P.mul_(vh, oop, v)
    assert np.allclose(xh.to_logical(), vh.to_logical(), atol=1e-8)
    P.ldiv_(u, ip, u)
    P.ldiv_(v, oop, vh)
    assert np.allclose(x.to_logical(), v.to_logical(), atol=1e-8)
    assert np.allclose(x.to_logical()[:3, 0, 0], [1.0, 2.0, 0.0], atol=1e-8)
    # bmul! of a random Hermitian-consistent spectrum, then mul! again
    spec = oracle_plan(oop).forward(np.random.default_rng(42).standard_normal(dims))
    xh.copy_from_logical(spec)
    vh.copy_from_logical(spec)
    P.bmul_(u, ip, u)
    P.bmul_(v, oop, vh)
    assert np.allclose(x.to_logical(), v.to_logical(), atol=1e-8)
    P.mul_(u, ip, u)
    P.mul_(vh, oop, v)
    assert np.allclose(xh.to_logical(), vh.to_logical(), atol=1e-6)


def test_notransform_bit_exact(cuda):
    plan = P.PencilFFTPlan((7, 5, 3), T.NoTransform(), np.float64, extra_dims=(2,))
    x = np.random.default_rng(1).standard_normal((7, 5, 3, 2))
    A = input_array(plan, x)
    B = plan * A
    assert np.array_equal(B.to_logical(), x)  # output permuted in memory, same logical values
    assert B.data.shape == (2, 7, 5, 3)       # memory order (z, y, x) reversed: x slowest
    assert np.array_equal(plan.ldiv(B).to_logical(), x)


def test_batch_graph_replay(cuda):
    """Batched form: forward + backward of uneven fields in one CUDA graph."""
    import torch
    rng = np.random.default_rng(2024)
    sizes = [(48, 64, 50), (96, 60, 72), (64, 64, 64), (53, 128, 40)]
    plans = [P.PencilFFTPlan(d, T.RFFT(), np.float32) for d in sizes]
    us = [input_array(p, rng.standard_normal(d).astype(np.float32)) for p, d in zip(plans, sizes)]
    vs = [p.allocate_output() for p in plans]
    ws = [p.allocate_input() for p in plans]
    ops = [(P.mul_, v, p, u) for p, u, v in zip(plans, us, vs)]
    ops += [(P.ldiv_, w, p, v) for p, v, w in zip(plans, vs, ws)]
    batch = P.Batch(ops, form="graph")
    assert batch.form == "graph"
    for trial in range(2):  # replay twice with new input contents
        xs = [rng.standard_normal(d).astype(np.float32) for d in sizes]
        for u, x in zip(us, xs):
            u.copy_from_logical(x)
        batch.launch()
        torch.cuda.synchronize()
        for p, v, w, x in zip(plans, vs, ws, xs):
            assert rel(v.to_logical(), oracle_plan(p).forward(x)) <= 2e-6
            assert rel(w.to_logical(), x) <= 2e-6


@pytest.mark.parametrize("real", [np.float64, np.float32])
def test_autotune_measure(cuda, real):
    """fftw_flags = FFTW.MEASURE (or autotune=True) times the alternative
    kernels of each pass at plan creation; the results are those of the
    default plan (both kernels run the same arithmetic)."""
    dims = (64, 48, 32)
    plan = P.PencilFFTPlan(dims, T.RFFT(), real, fftw_flags=P.FFTW_MEASURE)
    assert plan.autotune == 1
    assert P.PencilFFTPlan(dims, T.RFFT(), real, fftw_flags=P.FFTW_ESTIMATE).autotune == 0
    ref = P.PencilFFTPlan(dims, T.RFFT(), real)
    x = np.random.default_rng(3).standard_normal(dims).astype(real)
    v, vref = plan * input_array(plan, x), ref * input_array(ref, x)
    assert np.array_equal(v.to_logical(), vref.to_logical())
    w, wref = plan.ldiv(v), ref.ldiv(vref)
    assert np.array_equal(w.to_logical(), wref.to_logical())
    assert plan.device_status() == 0


def test_batch_branches_respect_buffer_order(cuda):
    """A batch records one graph branch per plan; operations of different
    plans that share buffers are ordered: B = F(A) then C = F(B) (read after
    write) and A overwritten by F(D) only after F(A) read it (write after
    read)."""
    dims = (32, 24, 20)
    p1 = P.PencilFFTPlan(dims, T.FFT(), np.float64)
    p2 = P.PencilFFTPlan(dims, T.FFT(), np.float64)
    p3 = P.PencilFFTPlan(dims, T.FFT(), np.float64)
    rng = np.random.default_rng(17)
    xa = rng.standard_normal(dims) + 1j * rng.standard_normal(dims)
    xd = rng.standard_normal(dims) + 1j * rng.standard_normal(dims)
    A, D = input_array(p1, xa), input_array(p1, xd)
    B, C = p1.allocate_output(), p1.allocate_output()
    # C = F(B) needs B in the input layout of p2: the output of p1 is the
    # reversed layout, so p2 reads it as a plan on the reversed dimensions
    p2 = P.PencilFFTPlan(tuple(reversed(dims)), T.FFT(), np.float64, permute_dims=False)
    Bv = P.PencilArray(p2.pencil_input(), B.data, B.dtype)
    Cv = P.PencilArray(p2.pencil_output(), C.data, C.dtype)
    # F(D) written over A's buffer, in p3's output layout
    Av = P.PencilArray(p3.pencil_output(), A.data.view(p3.pencil_output().memory_shape()), A.dtype)
    batch = P.Batch([(P.mul_, B, p1, A), (P.mul_, Cv, p2, Bv), (P.mul_, Av, p3, D)])
    batch.launch()
    import torch
    torch.cuda.synchronize()
    o1 = oracle_plan(p1)
    fa = o1.forward(xa)
    assert rel(B.to_logical(), fa) <= 1e-13
    # C holds the 3D FFT of F(A) taken in memory order (reversed dimensions)
    fb_mem = np.fft.fftn(fa.transpose(2, 1, 0))
    assert rel(Cv.to_logical(), fb_mem) <= 1e-13
    assert rel(Av.to_logical(), o1.forward(xd)) <= 1e-13
