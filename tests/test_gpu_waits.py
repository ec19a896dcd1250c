"""Give-up path of the bounded device waits (GPU).

The persistent kernels (the TMA-fed c2r form fast_pass_tma and the
tensor-core form tc_pass) wait on mbarriers for their bulk copies and
products with a poll limit; a wait that runs out sets a bit in the plan's
device status, the CTA waits (bounded, normal limit) for what it issued and
returns.  pfgb_plan_set_wait_test makes the first data wait of every CTA poll
an mbarrier that nothing signals, with a short limit: no wait here can hang
and nothing traps.  Each case checks that the status reports the bit, that a
second status read is clean, and that the next normal execution matches the
oracle.
"""
import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, input_array, oracle_plan, random_input, rel

pytestmark = pytest.mark.gpu


def test_tma_copy_wait_gives_up_then_recovers(cuda):
    """Float64 RFFT plan: the backward c2r pass along x (contiguous 33-point
    half spectra, 528-byte lines) runs in the TMA-fed form."""
    dims = (64, 24, 10)
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float64)
    x = random_input(plan, 5)
    v = plan * input_array(plan, x)
    plan.set_wait_test(16, tma=True)
    plan.ldiv(v)
    st = plan.device_status()
    assert st & 1, st
    assert not st & 4, st  # the copies in flight completed before the CTAs left
    assert plan.device_status() == 0  # read and cleared
    plan.set_wait_test(0, tma=True)  # same TMA-fed kernels, normal waits
    w = plan.ldiv(v)
    assert plan.device_status() == 0
    assert rel(w.to_logical(), x) <= 1e-13
    plan.set_wait_test(0, tma=False)
    w = plan.ldiv(v)
    assert rel(w.to_logical(), x) <= 1e-13
    assert plan.device_status() == 0


def test_tc_product_wait_gives_up_then_recovers(cuda):
    """Float32 tensor-core plan: 256-point c2c lines along x."""
    dims = (256, 6, 5)
    plan = P.PencilFFTPlan(dims, (T.FFT(), T.NoTransform(), T.NoTransform()), np.float32,
                           precision="tc")
    x = random_input(plan, 9)
    u = input_array(plan, x)
    plan.set_wait_test(16)
    plan * u
    st = plan.device_status()
    assert st & 2, st
    assert not st & 4, st  # the product completed before tensor memory was released
    assert plan.device_status() == 0
    plan.set_wait_test(0)
    v = plan * u
    assert plan.device_status() == 0
    assert rel(v.to_logical(), oracle_plan(plan).forward(x)) <= 2e-6
