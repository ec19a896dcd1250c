"""The allocation-free entry point pfgb_fft1d_noalloc, called through the C ABI.

It is meant for callers that cannot call cudaMalloc (their device memory is
owned by a pool or reserved up front, or they run where an allocation's
implicit synchronisation or the allocation call itself is not allowed).  Its
output must match the FP64 oracle (scipy.fft on the host) within the Float64
tolerance of the other tests, and the regular plan path
(pfgb_plan_create + pfgb_forward on a 1D plan with the batch as an extra
dimension), on two calls in a row that share its fixed scratch.  A batch
whose lines differ in magnitude by 1e120 keeps every line's accuracy (each
line is scaled by its own exponent).

This file is collected last so that a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

import pencilffts_gb300 as P
from helpers import T, rel
from oracle import pencilfft_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-13


def _oracle(sign, x):
    """x: (n, howmany) logical, lines along axis 0."""
    return O.transform_1d(O.FFT() if sign < 0 else O.BFFT(), x, axis=0)


def _regular(n, howmany, tr, x):
    plan = P.PencilFFTPlan((n,), tr, np.float64, extra_dims=(howmany,))
    A = plan.allocate_input()
    A.copy_from_logical(x)
    return (plan * A).to_logical()


def _noalloc(sign, n, howmany, x, inplace=False):
    import torch
    L = P.load_library()
    src = torch.from_numpy(np.ascontiguousarray(x.T)).to("cuda")  # memory: lines contiguous
    dst = src if inplace else torch.empty_like(src)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.pfgb_fft1d_noalloc(sign, n, howmany, ctypes.c_void_p(dst.data_ptr()),
                              ctypes.c_void_p(src.data_ptr()), stream)
    assert rc == 0, P._lib.last_error()
    torch.cuda.synchronize()
    return dst.cpu().numpy().T


def test_noalloc_matches_oracle_two_calls(cuda):
    rng = np.random.default_rng(11)
    # two calls in a row with different lengths, data and directions
    for (sign, tr, n, howmany, scale) in ((-1, T.FFT(), 512, 300, 1.0),
                                          (1, T.BFFT(), 64, 1000, 1e-7)):
        x = scale * (rng.standard_normal((n, howmany)) + 1j * rng.standard_normal((n, howmany)))
        got = _noalloc(sign, n, howmany, x)
        assert rel(got, _oracle(sign, x)) <= TOL
        assert rel(got, _regular(n, howmany, tr, x)) <= TOL


def test_noalloc_lines_of_very_different_magnitude(cuda):
    """Lines 1e+60, 1, 1e-60 and all-zero lines in one batch: each line is
    checked on its own against the oracle."""
    rng = np.random.default_rng(13)
    n, howmany = 256, 40
    x = rng.standard_normal((n, howmany)) + 1j * rng.standard_normal((n, howmany))
    scales = np.array([1e60, 1.0, 1e-60, 0.0] * (howmany // 4))
    x = x * scales[None, :]
    for sign in (-1, 1):
        got = _noalloc(sign, n, howmany, x)
        ref = _oracle(sign, x)
        for j in range(howmany):
            if scales[j] == 0.0:
                assert np.all(got[:, j] == 0)
            else:
                assert rel(got[:, j], ref[:, j]) <= TOL, (j, scales[j])


def test_noalloc_inplace_and_limits(cuda):
    rng = np.random.default_rng(12)
    n, howmany = 4096, 17
    x = rng.standard_normal((n, howmany)) + 1j * rng.standard_normal((n, howmany))
    assert rel(_noalloc(-1, n, howmany, x, inplace=True), _oracle(-1, x)) <= TOL
    import torch
    L = P.load_library()
    buf = torch.zeros(2 * 8192, dtype=torch.float64, device="cuda")
    for bad_n in (8192, 100, 16):
        rc = L.pfgb_fft1d_noalloc(-1, bad_n, 1, ctypes.c_void_p(buf.data_ptr()),
                                  ctypes.c_void_p(buf.data_ptr()), None)
        assert rc == P._lib.ERR_ARGUMENT
        assert "power of two in [32, 4096]" in P._lib.last_error()
