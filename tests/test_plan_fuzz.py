"""Host-only plan analysis over seeded random plans (no device): every
descriptor either plans or fails with the library's error, never a crash (a
transform along a one-point dimension once divided by zero in the planner,
which traps on x86 hosts only), and lines of any length up to 2^23 points
plan.  Mirrors the reference's transform tuples (src/Transforms/*.jl): c2c,
r2c first, R2R kinds, NoTransform, in-place variants, extra dimensions and
both output orders."""
import random

import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T

SIZES = [1, 2, 3, 5, 8, 16, 17, 64, 100, 4097, 5000, 8192, 8209, 16384]


def _random_plan(rng):
    N = rng.randint(1, 4)
    dims = tuple(rng.choice(SIZES) if rng.random() < 0.3 else rng.choice([1, 2, 4, 6, 8, 12])
                 for _ in range(N))
    inplace = rng.random() < 0.25
    kinds = []
    for d in range(N):
        r = rng.random()
        if r < 0.15:
            kinds.append(T.NoTransform_() if inplace else T.NoTransform())
        elif r < 0.3 and d == 0:
            kinds.append(T.RFFT_() if inplace else T.RFFT())
        elif r < 0.45:
            k = rng.choice([T.REDFT10, T.DHT, T.RODFT11, T.REDFT00, T.RODFT01])
            kinds.append(T.R2R_(k) if inplace else T.R2R(k))
        else:
            kinds.append(T.FFT_() if inplace else T.FFT())
    real = rng.choice([np.float32, np.float64])
    edims = tuple(rng.choice([1, 2, 3]) for _ in range(rng.randint(0, 2)))
    return dims, tuple(kinds), real, rng.random() < 0.5, edims


@pytest.mark.parametrize("seed", [11, 12])
def test_random_plans_analyse_cleanly(seed):
    rng = random.Random(seed)
    planned = 0
    for _ in range(300):
        dims, kinds, real, permute, edims = _random_plan(rng)
        if np.prod(dims) > 2 ** 26:
            continue
        try:
            info = P.plan_query(dims, kinds, real, permute_dims=permute, extra_dims=edims)
        except P.ArgumentError as e:
            # the reference's own argument errors (REDFT00 needs two points)
            assert "REDFT00" in str(e), (dims, kinds, str(e))
            continue
        planned += 1
        transforms = sum(not isinstance(k, T.NoTransform) for k in kinds)
        assert info.n_passes_forward >= min(1, transforms) and info.scratch_bytes >= 0
    assert planned >= 250


def test_any_length_plans():
    """Primes and lengths without a power-of-two factor plan up to 2^23
    points (Bluestein through split transforms), for every kind of line."""
    for n in (4099, 8209, 65537, (1 << 23) - 15):
        P.plan_query((n,), T.FFT(), np.float64)
    for n in (8209, 65537):
        P.plan_query((n,), T.RFFT(), np.float32)
        P.plan_query((n,), T.R2R(T.REDFT01), np.float64)
