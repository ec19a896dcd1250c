"""Shared helpers: map the host API's transforms to the oracle's, run a plan on
the GPU and compare it with the oracle."""
from __future__ import annotations

import numpy as np

import pencilffts_gb300 as P
from oracle import pencilfft_oracle as O

T = P.Transforms

# tolerances (relative L2 against the FP64 oracle)
TOL = {np.dtype(np.float64): 1e-13, np.dtype(np.float32): 2e-6}


def to_oracle(tr) -> O.Tr:
    ip = tr.inplace
    if isinstance(tr, T.FFT):
        return O.Tr("FFT", ip)
    if isinstance(tr, T.BFFT):
        return O.Tr("BFFT", ip)
    if isinstance(tr, T.RFFT):
        return O.Tr("RFFT", ip)
    if isinstance(tr, T.BRFFT):
        return O.Tr("BRFFT", ip, even=tr.even_output)
    if isinstance(tr, T.R2R):
        return O.Tr("R2R", ip, kind=tr.kind)
    return O.Tr("NoTransform", ip)


def oracle_plan(plan: P.PencilFFTPlan) -> O.OraclePlan:
    return O.OraclePlan(plan.size_global_in, tuple(to_oracle(t) for t in plan.transforms),
                        plan.real_type, plan.permute_dims, plan.extra_dims)


def random_input(plan: P.PencilFFTPlan, seed=0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    shape = tuple(plan.size_global_in) + tuple(plan.extra_dims)
    dt = plan.eltype_input()
    if dt.kind == "c":
        x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    else:
        x = rng.standard_normal(shape)
    if isinstance(plan.transforms[-1], T.BRFFT):
        # Hermitian-consistent input: u = plan \ v for a real v (reference test/transforms.jl:267-273)
        orc = oracle_plan(plan)
        vshape = tuple(plan.size_global_out) + tuple(plan.extra_dims)
        v = rng.standard_normal(vshape)
        x = orc.ldiv(v)
    return x.astype(dt)


def input_array(plan, x):
    A = plan.allocate_input()
    if isinstance(A, P.ManyPencilArray):
        A.first().copy_from_logical(x)
    else:
        A.copy_from_logical(x)
    return A


def rel(a, b):
    return O.rel_l2(a, b)
