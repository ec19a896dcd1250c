"""Tensor-core split form (precision="tc", Float32): c2c lines of 256, 512
and 1024 points as tcgen05 tf32 DFT-matrix products with a hi/lo split,
checked against the oracle at the Float32 tolerance (rel. L2 <= 2e-6),
forward, backward and round trip, in the axis-contiguous and strided
layouts, with partial tiles, spectral derivatives and the device status."""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, input_array, oracle_plan, random_input, rel

pytestmark = pytest.mark.gpu
TOL = 2e-6


def roundtrip_case(dims, tr):
    plan = P.PencilFFTPlan(dims, tr, np.float32, precision="tc")
    x = random_input(plan, 7)
    u = input_array(plan, x)
    v = plan * u
    e_fwd = rel(v.to_logical(), oracle_plan(plan).forward(x))
    w = plan.ldiv(v)
    e_rt = rel(w.to_logical(), x)
    assert plan.device_status() == 0
    return plan, e_fwd, e_rt


@pytest.mark.parametrize("dims", [(256, 6, 5), (512, 3, 4), (1024, 5, 2)])
def test_tc_c2c_contiguous_lines(cuda, dims):
    """First axis of length 256/512/1024 (stride 1), line counts not a
    multiple of the tile's 4 or 8 lines."""
    _, e_fwd, e_rt = roundtrip_case(dims, (T.FFT(), T.NoTransform(), T.NoTransform()))
    assert e_fwd <= TOL and e_rt <= TOL, (e_fwd, e_rt)


@pytest.mark.parametrize("dims", [(9, 512, 6), (4, 1024, 3), (13, 256, 2)])
def test_tc_c2c_strided_lines(cuda, dims):
    """Middle axis (strided), lines adjacent along the tile dimension."""
    _, e_fwd, e_rt = roundtrip_case(dims, (T.NoTransform(), T.FFT(), T.NoTransform()))
    assert e_fwd <= TOL and e_rt <= TOL, (e_fwd, e_rt)


def test_tc_rfft_3d(cuda):
    """RFFT plan: the y and z passes are c2c on the tensor cores, the x pass
    (r2c / c2r) stays on the plain kernel; agrees with the plain plan."""
    plan, e_fwd, e_rt = roundtrip_case((64, 512, 256), T.RFFT())
    assert e_fwd <= TOL and e_rt <= TOL, (e_fwd, e_rt)
    plain = P.PencilFFTPlan((64, 512, 256), T.RFFT(), np.float32)
    x = random_input(plain, 7)
    a = (plain * input_array(plain, x)).to_logical()
    b = (plan * input_array(plan, x)).to_logical()
    assert rel(b, a) <= 2 * TOL


def test_tc_bfft_sign(cuda):
    """Backward (sign +1) transform as a forward plan, no normalisation."""
    plan = P.PencilFFTPlan((16, 512), (T.NoTransform(), T.BFFT()), np.float32, precision="tc")
    x = random_input(plan, 3)
    v = plan * input_array(plan, x)
    assert rel(v.to_logical(), oracle_plan(plan).forward(x)) <= TOL


def test_tc_spectral_derivative(cuda):
    """i k multiply fused into the first backward (tensor-core) pass."""
    dims = (32, 512, 256)
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float32, precision="tc")
    L = 2 * np.pi
    y = np.arange(dims[1]) * L / dims[1]
    x = np.broadcast_to((np.sin(3 * y) + 0.5 * np.cos(5 * y))[None, :, None], dims).astype(np.float32)
    uF = plan * input_array(plan, x)
    d = plan.allocate_input()
    P.ldiv_(d, plan, uF, deriv=(2, L))
    expect = np.broadcast_to((3 * np.cos(3 * y) - 2.5 * np.sin(5 * y))[None, :, None], dims)
    assert rel(d.to_logical(), expect) <= 1e-5
    assert plan.device_status() == 0
