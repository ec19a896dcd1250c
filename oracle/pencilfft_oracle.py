"""CPU oracle for the PencilFFTs transform path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: tests, the smoke check and
the CPU-baseline leg of the benchmark import it.  The product path (the CUDA
library) never calls it and has no CPU fallback.

What it restates
----------------
* The multidimensional transform chain of PencilFFTs (reference
  ``src/plans.jl:241-293,406-449`` and ``src/operations.jl:24-70,161-172,
  227-257``): one 1D transform per dimension, applied left to right for the
  forward transform and right to left (with the inverse 1D transforms) for the
  backward one; ``ldiv!`` divides by the product of the per-dimension scale
  factors; the output is stored with its memory order reversed when
  ``permute_dims`` is true (``src/plans.jl:503-521``).
* The transform descriptors of ``src/Transforms/*.jl``: ``expand_dims``,
  ``binv``, ``length_output``, ``scale_factor``, element types.
* The 1D transforms themselves.  In the reference they are FFTW 3.3 plans
  (FFTW.jl, compat 1.6; the benchmark manifest pins FFTW.jl 1.4.3 with
  FFTW_jll 3.3.9), which is not part of the reference tree.  FFTW's published
  definitions are restated here through ``scipy.fft`` (pocketfft), float64 or
  long double:

  - FFT  (sign -1, unnormalised)      ``Y_k = sum_j X_j exp(-2 pi i jk/n)``
  - BFFT (sign +1, unnormalised)
  - RFFT: n reals -> n//2+1 complex; BRFFT: the unnormalised c2r inverse, which
    uses only the real parts of the DC and (even n) Nyquist terms
  - R2R kinds with FFTW's numeric codes: DHT (``Re F - Im F``), REDFT00..11
    (DCT-I..IV: 00=I, 10=II, 01=III, 11=IV), RODFT00..11 (DST-I..IV), all
    unnormalised; on complex data they act on real and imaginary parts
    separately (reference ``src/Transforms/r2r.jl:83-84``).

  ``oracle/dft_direct.c`` evaluates the same definitions directly (O(n^2), long
  double) and the tests check this module against it on small sizes, and against
  the analytic known answers of the reference's tests.

Array conventions
-----------------
A *logical* array has numpy shape ``(n1, ..., nN, e1, ..., eK)`` indexed like
the Julia array ``u[i1, ..., iN, j1, ..., jK]``.  Its *memory* buffer in
Julia's column-major order (dimension 1 fastest) is the C-order array
``logical.transpose(reversed axes)``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np
import scipy.fft as sfft

# FFTW's r2r kind codes (fftw3.h); PencilFFTs passes them through unchanged
# (reference src/Transforms/r2r.jl:5-15).
R2HC, HC2R, DHT = 0, 1, 2
REDFT00, REDFT01, REDFT10, REDFT11 = 3, 4, 5, 6
RODFT00, RODFT01, RODFT10, RODFT11 = 7, 8, 9, 10
R2R_SUPPORTED_KINDS = (DHT, REDFT00, REDFT01, REDFT10, REDFT11,
                       RODFT00, RODFT01, RODFT10, RODFT11)
KIND_NAMES = {R2HC: "R2HC", HC2R: "HC2R", DHT: "DHT", REDFT00: "REDFT00",
              REDFT01: "REDFT01", REDFT10: "REDFT10", REDFT11: "REDFT11",
              RODFT00: "RODFT00", RODFT01: "RODFT01", RODFT10: "RODFT10",
              RODFT11: "RODFT11"}

# DCT/DST kind -> (family, scipy type).  FFTW: REDFT00=DCT-I, REDFT10=DCT-II,
# REDFT01=DCT-III, REDFT11=DCT-IV, and RODFT likewise for the DSTs.
_R2R_SCIPY = {
    REDFT00: ("dct", 1), REDFT10: ("dct", 2), REDFT01: ("dct", 3), REDFT11: ("dct", 4),
    RODFT00: ("dst", 1), RODFT10: ("dst", 2), RODFT01: ("dst", 3), RODFT11: ("dst", 4),
}


# ---------------------------------------------------------------------------
# Transform descriptors (reference src/Transforms/*.jl)
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Tr:
    """One 1D transform descriptor.

    ``name`` is one of FFT, BFFT, RFFT, BRFFT, R2R, NoTransform; ``inplace``
    marks the ``!`` variants; ``even`` is BRFFT's ``even_output``;
    ``kind`` the FFTW r2r kind.
    """
    name: str
    inplace: bool = False
    even: bool = True
    kind: int = -1

    def __repr__(self):  # mirrors Base.show in the reference
        s = self.name + ("!" if self.inplace else "")
        if self.name == "BRFFT":
            s += "{even}" if self.even else "{odd}"
        if self.name == "R2R":
            s += "{" + KIND_NAMES[self.kind] + "}"
        return s


def FFT(inplace=False): return Tr("FFT", inplace)
def BFFT(inplace=False): return Tr("BFFT", inplace)
def RFFT(inplace=False): return Tr("RFFT", inplace)
def NoTransform(inplace=False): return Tr("NoTransform", inplace)


def BRFFT(d, inplace=False):
    """reference r2c.jl:66-69: BRFFT(d) stores iseven(d); a tuple uses its last entry."""
    if isinstance(d, (tuple, list)):
        d = d[-1]
    return Tr("BRFFT", inplace, even=(int(d) % 2 == 0))


def R2R(kind, inplace=False):
    """reference r2r.jl:38-57: unsupported kinds raise ArgumentError."""
    if kind not in R2R_SUPPORTED_KINDS:
        raise ValueError(f"unsupported r2r transform kind: {KIND_NAMES.get(kind, kind)}")
    return Tr("R2R", inplace, kind=kind)


_R2R_INV = {REDFT00: REDFT00, REDFT01: REDFT10, REDFT10: REDFT01, REDFT11: REDFT11,
            RODFT00: RODFT00, RODFT01: RODFT10, RODFT10: RODFT01, RODFT11: RODFT11,
            DHT: DHT}


def binv(tr: Tr, d: int) -> Tr:
    """reference c2c.jl:58-61, r2c.jl:98-101, r2r.jl:103-131, no_transform.jl:23."""
    if tr.name == "FFT":
        return Tr("BFFT", tr.inplace)
    if tr.name == "BFFT":
        return Tr("FFT", tr.inplace)
    if tr.name == "RFFT":
        return BRFFT(d, tr.inplace)
    if tr.name == "BRFFT":
        return Tr("RFFT", tr.inplace)
    if tr.name == "R2R":
        return Tr("R2R", tr.inplace, kind=_R2R_INV[tr.kind])
    return tr


def length_output(tr: Tr, n: int) -> int:
    """reference c2c.jl:47, r2c.jl:74-75, r2r.jl:78, no_transform.jl:24."""
    if tr.name == "RFFT":
        return n // 2 + 1
    if tr.name == "BRFFT":
        return 2 * n - 1 - int(tr.even)
    return n


def scale_factor_1d(tr: Tr, n_in: int) -> int:
    """Scale factor of ``tr`` applied to an input of length ``n_in`` along one dim.

    reference c2c.jl:71, r2c.jl:103-111, r2r.jl:96-101, no_transform.jl:26.
    """
    if tr.name in ("FFT", "BFFT", "RFFT"):
        return n_in
    if tr.name == "BRFFT":
        return length_output(tr, n_in)
    if tr.name == "R2R":
        if tr.kind == REDFT00:
            return 2 * (n_in - 1)
        if tr.kind == RODFT00:
            return 2 * (n_in + 1)
        if tr.kind == DHT:
            return n_in
        return 2 * n_in
    return 1


def expand_dims(tr: Tr, N: int) -> tuple:
    """reference Transforms.jl:285-291 and r2c.jl:114-124."""
    if N == 0:
        return ()
    if tr.name == "RFFT":
        return (tr,) + tuple(Tr("FFT", tr.inplace) for _ in range(N - 1))
    if tr.name == "BRFFT":
        return tuple(Tr("BFFT", tr.inplace) for _ in range(N - 1)) + (tr,)
    return tuple(tr for _ in range(N))


def is_inplace(*trs: Tr):
    """reference Transforms.jl:141-147: None for a mix of in/out-of-place."""
    flags = {t.inplace for t in trs}
    return flags.pop() if len(flags) == 1 else None


def eltype_input(tr: Tr, real):
    """reference c2c.jl:49, r2c.jl:80-81, r2r.jl:79, no_transform.jl:25.

    Returns None when the transform accepts both real and complex data.
    """
    real = np.dtype(real)
    cplx = np.result_type(real, np.complex64)
    if tr.name in ("FFT", "BFFT", "BRFFT"):
        return cplx
    if tr.name == "RFFT":
        return real
    return None


def eltype_output(tr: Tr, t):
    """reference Transforms.jl:235-236, c2c.jl:48, r2c.jl:77-78."""
    t = np.dtype(t)
    if tr.name in ("FFT", "BFFT"):
        if t.kind != "c":
            raise ValueError(f"invalid input data type for {tr.name}: {t}")
        return t
    if tr.name == "RFFT":
        if t.kind != "f":
            raise ValueError(f"invalid input data type for {tr.name}: {t}")
        return np.result_type(t, np.complex64)
    if tr.name == "BRFFT":
        if t.kind != "c":
            raise ValueError(f"invalid input data type for {tr.name}: {t}")
        return np.dtype(np.float32) if t == np.complex64 else np.dtype(np.float64)
    return t


def input_data_type(real, transforms) -> np.dtype:
    """reference global_params.jl:81-95: first transform with a fixed input type."""
    for t in transforms:
        ti = eltype_input(t, real)
        if ti is not None:
            return ti
    return np.dtype(real)


# ---------------------------------------------------------------------------
# 1D transforms (FFTW definitions, via scipy.fft)
# ---------------------------------------------------------------------------
# all host threads for the large test arrays
_W = -1


def _r2r_real(x: np.ndarray, kind: int, axis: int) -> np.ndarray:
    if kind == DHT:
        F = sfft.fft(x, axis=axis, workers=_W)
        return F.real - F.imag
    fam, typ = _R2R_SCIPY[kind]
    f = sfft.dct if fam == "dct" else sfft.dst
    return f(x, type=typ, axis=axis, norm=None, workers=_W)


def transform_1d(tr: Tr, x: np.ndarray, axis: int, n_out: int | None = None,
                 forward_sign: bool = True) -> np.ndarray:
    """Apply one 1D transform along ``axis`` (unnormalised, FFTW semantics)."""
    if tr.name == "FFT":
        return sfft.fft(x, axis=axis, workers=_W)
    if tr.name == "BFFT":
        return sfft.ifft(x, axis=axis, norm="forward", workers=_W)
    if tr.name == "RFFT":
        if np.iscomplexobj(x):
            raise ValueError("RFFT needs real input")
        return sfft.rfft(x, axis=axis, workers=_W)
    if tr.name == "BRFFT":
        n = length_output(tr, x.shape[axis]) if n_out is None else n_out
        return sfft.irfft(x, n=n, axis=axis, norm="forward", workers=_W)
    if tr.name == "R2R":
        if np.iscomplexobj(x):
            return _r2r_real(x.real, tr.kind, axis) + 1j * _r2r_real(x.imag, tr.kind, axis)
        return _r2r_real(x, tr.kind, axis)
    return x.copy()


# ---------------------------------------------------------------------------
# Multidimensional plan (reference src/plans.jl, src/operations.jl)
# ---------------------------------------------------------------------------
@dataclass
class OraclePlan:
    """CPU restatement of ``PencilFFTPlan`` at ``proc_dims = (1, ..., 1)``."""
    dims: tuple
    transforms: tuple
    real_type: np.dtype = field(default_factory=lambda: np.dtype(np.float64))
    permute_dims: bool = True
    extra_dims: tuple = ()
    longdouble: bool = False

    def __post_init__(self):
        self.dims = tuple(int(d) for d in self.dims)
        if isinstance(self.transforms, Tr):
            self.transforms = expand_dims(self.transforms, len(self.dims))
        self.transforms = tuple(self.transforms)
        if len(self.transforms) != len(self.dims):
            raise ValueError("number of transforms must equal the number of dimensions")
        self.real_type = np.dtype(self.real_type)
        if is_inplace(*self.transforms) is None:
            raise ValueError(f"cannot combine in-place and out-of-place transforms: {self.transforms}")
        # reference global_params.jl:50-62
        self.dims_out = tuple(length_output(t, n) for t, n in zip(self.transforms, self.dims))
        self.eltype_in = input_data_type(self.real_type, self.transforms)
        t = self.eltype_in
        for tr in self.transforms:
            t = eltype_output(tr, t)
        self.eltype_out = t
        # reference plans.jl:268 and 540-546: product of per-dim backward scales
        # (the backward transform maps the forward output back, so its scale is
        # evaluated on the forward output length along that dimension).
        scale = 1.0
        for tr, n_in, n_out in zip(self.transforms, self.dims, self.dims_out):
            scale *= float(scale_factor_1d(binv(tr, n_in), n_out))
        self.scale = scale

    # -- layouts ---------------------------------------------------------
    @property
    def ndims(self):
        return len(self.dims)

    def to_memory(self, logical: np.ndarray, output: bool) -> np.ndarray:
        """Logical array -> C-order memory buffer of the input or output pencil."""
        N, K = self.ndims, len(self.extra_dims)
        if output and self.permute_dims:
            # memory order (N, ..., 1, e1, ..., eK): C-order shape (eK..e1, n1..nN)
            perm = tuple(range(N + K - 1, N - 1, -1)) + tuple(range(N))
        else:
            perm = tuple(range(N + K - 1, -1, -1))
        return np.ascontiguousarray(logical.transpose(perm))

    def from_memory(self, mem: np.ndarray, output: bool) -> np.ndarray:
        N, K = self.ndims, len(self.extra_dims)
        if output and self.permute_dims:
            perm = tuple(range(N + K - 1, N - 1, -1)) + tuple(range(N))
        else:
            perm = tuple(range(N + K - 1, -1, -1))
        inv = np.argsort(perm)
        return np.ascontiguousarray(mem.transpose(inv))

    # -- execution (logical arrays) ---------------------------------------
    def _work(self, x):
        if self.longdouble:
            return x.astype(np.clongdouble if np.iscomplexobj(x) else np.longdouble)
        return x.astype(np.complex128 if np.iscomplexobj(x) else np.float64)

    def forward(self, u: np.ndarray) -> np.ndarray:
        """``mul!(v, plan, u)``: reference operations.jl:24-31, 227-254."""
        x = self._work(u)
        for n, tr in enumerate(self.transforms):
            x = transform_1d(tr, x, axis=n)
        return x

    def bmul(self, v: np.ndarray) -> np.ndarray:
        """``bmul!``: backward transforms in reverse order, unscaled (operations.jl:34-41, 164-167)."""
        x = self._work(v)
        for n in range(self.ndims - 1, -1, -1):
            tr_b = binv(self.transforms[n], self.dims[n])
            x = transform_1d(tr_b, x, axis=n, n_out=self.dims[n])
        return x

    def ldiv(self, v: np.ndarray) -> np.ndarray:
        """``ldiv!``: ``bmul!`` followed by division by ``scale_factor`` (operations.jl:44-52, 64-70)."""
        return self.bmul(v) / self.scale


def wavenumbers(plan: "OraclePlan", dim: int, length: float) -> np.ndarray:
    """i k along 0-based ``dim`` of the plan's spectral (output) array,
    broadcastable to its logical shape: k = 2 pi f / length with f the
    AbstractFFTs frequencies (``rfftfreq`` along an r2c / c2r dimension,
    ``fftfreq`` otherwise), as the reference's test helpers use them
    (test/include/Grids.jl:38-59)."""
    tr = plan.transforms[dim]
    if tr.name == "RFFT":
        f = np.arange(plan.dims_out[dim])
    elif tr.name == "BRFFT":
        f = np.arange(plan.dims[dim])
    else:
        n = plan.dims[dim]
        f = np.fft.fftfreq(n, 1.0 / n)
    k = 2 * np.pi * f / length
    shape = [1] * (plan.ndims + len(plan.extra_dims))
    shape[dim] = -1
    return (1j * k).reshape(shape)


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """Relative L2 error ``|a - b| / |b|`` computed in long double."""
    a = np.asarray(a).astype(np.clongdouble)
    b = np.asarray(b).astype(np.clongdouble)
    den = np.sum(np.abs(b) ** 2)
    num = np.sum(np.abs(a - b) ** 2)
    if den > 0:
        return math.sqrt(float(num / den))
    return math.sqrt(float(num))


def max_abs(a, b) -> float:
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) if np.size(a) else 0.0
