"""ctypes loader for oracle/dft_direct.c (test infrastructure only).

Builds the shared object with ``make -C oracle`` on first use.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libdft_direct.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(
                os.path.join(_HERE, "dft_direct.c")):
            build()
        L = ctypes.CDLL(_SO)
        dp = ctypes.POINTER(ctypes.c_double)
        L.pfo_dft.argtypes = [ctypes.c_int64, ctypes.c_int, dp, dp]
        L.pfo_rfft.argtypes = [ctypes.c_int64, dp, dp]
        L.pfo_brfft.argtypes = [ctypes.c_int64, dp, dp]
        L.pfo_r2r.argtypes = [ctypes.c_int, ctypes.c_int64, dp, dp]
        L.pfo_r2r.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def dft(x: np.ndarray, sign: int) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.complex128)
    y = np.empty_like(x)
    lib().pfo_dft(x.size, sign, _p(x.view(np.float64)), _p(y.view(np.float64)))
    return y


def rfft(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(x.size // 2 + 1, dtype=np.complex128)
    lib().pfo_rfft(x.size, _p(x), _p(y.view(np.float64)))
    return y


def brfft(x: np.ndarray, n: int) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.complex128)
    assert x.size == n // 2 + 1
    y = np.empty(n, dtype=np.float64)
    lib().pfo_brfft(n, _p(x.view(np.float64)), _p(y))
    return y


def r2r(x: np.ndarray, kind: int) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    rc = lib().pfo_r2r(kind, x.size, _p(x), _p(y))
    if rc != 0:
        raise ValueError(f"r2r kind {kind} undefined for n={x.size}")
    return y
