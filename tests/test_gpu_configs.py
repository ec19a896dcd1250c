"""Parity on the benchmark configurations (GPU).

C1  3D RFFT Float64 (16, 32, 64), uniform [0, 1), seed 42.
C2  3D FFT/BFFT ComplexF64 256^3, N(0,1) seed 0;  RFFT Float32 512^3 U[-1,1) seed 1.
C3  (RFFT, FFT, R2R{REDFT00}) Float64 Taylor-Green on 512 x 512 x 257 with
    Chebyshev-Gauss-Lobatto points along z.
C4  RFFT Float32 1024^3: N(0,1) plus 8 Fourier modes; checked through
    size-independent properties (round trip, exact spectral peaks of the
    modes, Parseval, linearity) because a full-size CPU oracle is too slow.
C5  vector field 3 x 384^3 Float32 spectral gradient, and 64 independent r2c
    round trips with sizes drawn from 48..192 per axis (mixed radices and
    primes through Bluestein), seed 2024.
"""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, input_array, oracle_plan, rel
from oracle import pencilfft_oracle as O

pytestmark = pytest.mark.gpu


def run_fwd_bwd(plan, x):
    A = input_array(plan, x)
    B = plan * A
    out = B.to_logical()
    back = plan.ldiv(B).to_logical()
    return out, back


def rel_chunked(a, b, chunk=1 << 24):
    """Relative L2 |a - b| / |b| in float64 over chunks (arrays of 10^8
    elements and more; a float64 sum of squares is exact to ~1e-16 relative,
    far below the tolerances checked here)."""
    a = a.reshape(-1)
    b = b.reshape(-1)
    num = den = 0.0
    for i in range(0, a.size, chunk):
        x, y = a[i:i + chunk], b[i:i + chunk]
        num += float(np.sum(np.abs(x - y) ** 2))
        den += float(np.sum(np.abs(y) ** 2))
    return (num / den) ** 0.5


def test_headline_rfft_512_f64_vs_oracle(cuda):
    """The benchmark workload itself: 512^3 Float64 RFFT, out-of-place,
    permute_dims=true, input uniform [-1, 1) from the benchmark's device
    generator (seed 1).  Forward spectrum and ldiv! against the FP64 oracle
    at the Float64 tolerance, computed in the default double-float arithmetic."""
    import torch
    dims = (512, 512, 512)
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float64)
    u = plan.allocate_input()
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    u.data.uniform_(-1.0, 1.0, generator=g)
    x = u.to_logical()
    v = plan * u
    got = v.to_logical()
    orc = oracle_plan(plan)
    ref = orc.forward(x)
    assert rel_chunked(got, ref) <= 1e-13
    del ref
    back = plan.ldiv(v).to_logical()
    assert rel_chunked(back, orc.ldiv(got)) <= 1e-13
    assert rel_chunked(back, x) <= 1e-13


def test_c1_rfft_16_32_64(cuda):
    dims = (16, 32, 64)
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float64)
    u = np.random.default_rng(42).random(dims)
    out, back = run_fwd_bwd(plan, u)
    orc = oracle_plan(plan)
    assert rel(out, orc.forward(u)) <= 1e-13
    assert rel(back, u) <= 1e-13


@pytest.mark.parametrize("tr", [T.FFT(), T.BFFT()], ids=repr)
def test_c2_c2c_256_f64(cuda, tr):
    dims = (256, 256, 256)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(dims) + 1j * rng.standard_normal(dims)
    plan = P.PencilFFTPlan(dims, tr, np.float64)
    out, back = run_fwd_bwd(plan, x)
    assert rel(out, oracle_plan(plan).forward(x)) <= 1e-13
    assert rel(back, x) <= 1e-13


def test_c2_rfft_512_f32(cuda):
    dims = (512, 512, 512)
    x = np.random.default_rng(1).uniform(-1, 1, dims).astype(np.float32)
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float32)
    out, back = run_fwd_bwd(plan, x)
    assert rel(out, oracle_plan(plan).forward(x)) <= 2e-6
    assert rel(back, x) <= 2e-6


def test_c3_taylor_green_mixed_512_512_257(cuda):
    nx, ny, nz = 512, 512, 257
    x = 2 * np.pi * np.arange(nx) / nx
    y = 2 * np.pi * np.arange(ny) / ny
    z = np.cos(np.pi * np.arange(nz) / (nz - 1))  # Chebyshev-Gauss-Lobatto
    u = np.sin(x)[:, None, None] * np.cos(y)[None, :, None] * np.cos(z)[None, None, :]
    plan = P.PencilFFTPlan((nx, ny, nz), (T.RFFT(), T.FFT(), T.R2R(T.REDFT00)), np.float64)
    assert plan.scale_factor == 512.0 ** 3
    out, back = run_fwd_bwd(plan, u)
    assert rel(out, oracle_plan(plan).forward(u)) <= 1e-13
    assert rel(back, u) <= 1e-13


@pytest.mark.parametrize("precision", ["default", "tc"])
def test_c4_rfft_1024_f32_properties(cuda, precision):
    """C4 with the plain kernels and with the tensor-core split form (the
    1024-point y and z lines as tcgen05 DFT-matrix products)."""
    import torch
    n = 1024
    dims = (n, n, n)
    rng = np.random.default_rng(1234)
    amps = rng.uniform(1, 10, 8)
    phis = rng.uniform(0, 2 * np.pi, 8)
    ks = rng.integers(0, 64, size=(8, 3))
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float32, precision=precision)
    A = plan.allocate_input()
    g = torch.Generator(device="cuda").manual_seed(1234)
    noise = torch.randn(A.data.shape, generator=g, device="cuda", dtype=torch.float32)
    # modes on the device: u = noise + sum a cos(k.x + phi), x_j = 2 pi j / n
    lin = torch.arange(n, device="cuda", dtype=torch.float64) * (2 * np.pi / n)
    field = noise.double()
    for a, phi, k in zip(amps, phis, ks):
        # memory order (z, y, x): broadcast k_x x + k_y y + k_z z
        ph = (k[2] * lin)[:, None, None] + (k[1] * lin)[None, :, None] + (k[0] * lin)[None, None, :]
        field += a * torch.cos(ph + phi)
    A.data.copy_(field.float())
    u_host = A.data.clone()
    B = plan * A
    # exact spectral peaks: a cos(k.x + phi) contributes (a N/2) e^{i phi} at k
    N = float(n) ** 3
    for a, phi, k in zip(amps, phis, ks):
        # output memory order (x, y, z) logical; negative k_y, k_z wrap
        val = B.data[k[0], k[1], k[2]].item()
        assert abs(val - a * N / 2 * np.exp(1j * phi)) <= 1e-3 * a * N / 2 + 5 * np.sqrt(N)
    # Parseval (reference test/rfft.jl:21-43)
    w = torch.full((n // 2 + 1,), 2.0, device="cuda", dtype=torch.float64)
    w[0] = 1.0
    w[-1] = 1.0
    s_phys = (A.data.double() ** 2).sum().item() / N
    s_spec = (w[:, None, None] * B.data.abs().double() ** 2).sum().item() / (N * N)
    assert abs(s_phys - s_spec) <= 1e-5 * s_phys
    # round trip
    U = plan.ldiv(B)
    d = (U.data.double() - u_host.double()).norm().item() / u_host.double().norm().item()
    assert d <= 2e-6
    # linearity: F(2u + 3 * 1) = 2 F(u) + 3 F(1)  (F(1) is N at the origin)
    A.data.copy_(2 * u_host + 3)
    B2 = plan * A
    B2.data[0, 0, 0] -= 3 * N
    diff = (B2.data - 2 * B.data).abs().double().norm().item() / (2 * B.data.abs().double().norm().item())
    assert diff <= 2e-6
    assert plan.device_status() == 0


def test_c5_vector_gradient_384(cuda):
    """3-component Float32 field 384^3 (384 = 3 * 128, the mixed-radix pass):
    forward, then the derivative of component c along dimension c fused into
    the first backward pass (ldiv_ with deriv), and the divergence of the
    field as one fused backward transform; against the oracle."""
    n = 384
    dims = (n, n, n)
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float32)
    rng = np.random.default_rng(2024)
    comps = [rng.standard_normal(dims).astype(np.float32) for _ in range(3)]
    u = plan.allocate_input(P.Val(3))
    for c, x in zip(u, comps):
        c.copy_from_logical(x)
    uF = plan * u
    L = 2 * np.pi
    du = plan.allocate_input(P.Val(3))
    for c in range(3):
        P.ldiv_(du[c], plan, uF[c], deriv=(c + 1, L))
    orc = oracle_plan(plan)
    specs = [orc.forward(x) for x in comps]
    for c in range(3):
        ref = orc.ldiv(specs[c] * O.wavenumbers(orc, c, L))
        assert rel(du[c].to_logical(), ref) <= 2e-6
    div = plan.allocate_input()
    P.ldiv_divergence_(div, plan, uF, (L, L, L))
    ref = orc.ldiv(sum(specs[c] * O.wavenumbers(orc, c, L) for c in range(3)))
    assert rel(div.to_logical(), ref) <= 2e-6


@pytest.mark.parametrize("form", ["graph", "persistent"])
def test_c5_batch_of_64_uneven(cuda, form):
    """64 independent Float32 r2c + c2r round trips of sizes drawn from
    48..192 per axis (mixed radices, primes through Bluestein), recorded into
    one batch (one CUDA graph with one branch per field, or one persistent
    launch walking every tile of every pass) and launched once; every field
    against the oracle."""
    import torch
    rng = np.random.default_rng(2024)
    sizes = [tuple(int(s) for s in rng.integers(48, 193, 3)) for _ in range(64)]
    plans, arrays, xs = [], [], []
    for dims in sizes:
        plan = P.PencilFFTPlan(dims, T.RFFT(), np.float32)
        x = rng.standard_normal(dims).astype(np.float32)
        u, v, w = input_array(plan, x), plan.allocate_output(), plan.allocate_input()
        plans.append(plan)
        arrays.append((u, v, w))
        xs.append(x)
    ops = []
    for plan, (u, v, w) in zip(plans, arrays):
        ops += [(P.mul_, v, plan, u), (P.ldiv_, w, plan, v)]
    batch = P.Batch(ops, form=form)
    assert batch.form == form
    batch.launch()
    torch.cuda.synchronize()
    for plan, (u, v, w), x, dims in zip(plans, arrays, xs, sizes):
        assert rel(v.to_logical(), oracle_plan(plan).forward(x)) <= 2e-6, dims
        assert rel(w.to_logical(), x) <= 2e-6, dims
