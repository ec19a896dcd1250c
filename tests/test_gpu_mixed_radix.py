"""Mixed-radix register pass (GPU): lines of 3 * 2^k and 5 * 2^k points
(8 <= 2^k <= 512) as R0-point DFTs in registers, twiddles and 2^k-point
register stages.  c2c, r2c and c2r lines along contiguous and strided axes,
both output orders, partial tiles, extra dimensions, fused derivatives and
derivative sums, in Float32 and in double-float for Float64; each case
against the oracle at the type's tolerance (reference FFTW plans of any
length, src/Transforms/c2c.jl:53-56, r2c.jl:83-96) and asserting that the
mixed-radix kernel ran."""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, TOL, input_array, oracle_plan, random_input, rel
from oracle import pencilfft_oracle as O
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
@pytest.mark.parametrize("n", [24, 48, 96, 384, 1536, 40, 160, 640, 2560])
def test_mr_1d_lines(cuda, real, n):
    """FFT and RFFT of one axis, 7 lines (partial tiles, odd pair count)."""
    for tr in (T.FFT(), T.RFFT()):
        plan = P.PencilFFTPlan((n,), tr, real, extra_dims=(7,))
        check_plan(plan, seed=n)
        k = kernels(plan)
        assert k[(1, 0)].startswith("mr_pass") and k[(-1, 0)].startswith("mr_pass"), k


@pytest.mark.parametrize("real", [F64, F32])
@pytest.mark.parametrize("dims,tr", [((48, 20, 12), T.RFFT()), ((20, 96, 7), T.FFT()),
                                     ((12, 10, 80), T.FFT()), ((96, 48, 40), T.RFFT()),
                                     ((64, 24, 96), (T.RFFT(), T.FFT(), T.FFT()))],
                         ids=["x-r2c", "y-strided", "z-last", "all-mr", "mix-pow2"])
def test_mr_3d_layouts(cuda, real, dims, tr):
    for permute in (True, False):
        plan = P.PencilFFTPlan(dims, tr, real, permute_dims=permute)
        check_plan(plan, seed=2)


def test_mr_c5_like_gradient_and_divergence(cuda):
    """384-point lines as in the vector-field configuration (on a 384 x 24 x 48
    grid): fused derivative in the first backward pass and a fused
    divergence, against the oracle."""
    dims = (384, 24, 48)
    plan = P.PencilFFTPlan(dims, T.RFFT(), F32)
    orc = oracle_plan(plan)
    L = (2 * np.pi, 3.0, 5.0)
    xs = [random_input(plan, 40 + c) for c in range(3)]
    specs = [orc.forward(x) for x in xs]
    uF = []
    for s in specs:
        S = plan.allocate_output()
        S.copy_from_logical(s)
        uF.append(S)
    for d in range(3):
        U = plan.allocate_input()
        P.ldiv_(U, plan, uF[d], deriv=(d + 1, L[d]))
        assert rel(U.to_logical(), orc.ldiv(O.wavenumbers(orc, d, L[d]) * specs[d])) <= TOL[np.dtype(F32)]
    div = plan.allocate_input()
    P.ldiv_divergence_(div, plan, uF, L)
    ref = orc.ldiv(sum(O.wavenumbers(orc, d, L[d]) * specs[d] for d in range(3)))
    assert rel(div.to_logical(), ref) <= TOL[np.dtype(F32)]
    k = kernels(plan)
    assert k[(-1, 2)].startswith("mr_pass"), k  # 48 = 3 * 16 along z: the first backward pass


@pytest.mark.parametrize("real", [F64, F32])
def test_mr_forward_derivative(cuda, real):
    """i k multiply fused into the last forward pass, on a mixed-radix line."""
    dims = (16, 12, 96)
    plan = P.PencilFFTPlan(dims, T.FFT(), real)
    orc = oracle_plan(plan)
    x = random_input(plan, 3)
    B = plan.allocate_output()
    P.mul_(B, plan, input_array(plan, x), deriv=(3, 2.5))
    assert rel(B.to_logical(), O.wavenumbers(orc, 2, 2.5) * orc.forward(x)) <= TOL[np.dtype(real)]


def test_mr_float64_wide_dynamic_range(cuda):
    """Per-line exponents of the double-float mixed-radix pass: lines 1e+-150
    apart, each checked against the oracle on its own."""
    n, h = 192, 6
    plan = P.PencilFFTPlan((n,), T.FFT(), F64, extra_dims=(h,))
    x = random_input(plan, 9) * np.array([1e150, 1.0, 1e-150, 3e-100, 0.0, 1e20])[None, :]
    out = (plan * input_array(plan, x)).to_logical()
    ref = oracle_plan(plan).forward(x)
    for j in range(h):
        if j == 4:
            assert np.all(out[:, j] == 0)
        else:
            assert rel(out[:, j], ref[:, j]) <= 1e-13, j
