"""Transform descriptors: the host-side mirror of PencilFFTs' ``Transforms``.

Each class corresponds to one transform type of the reference
(``src/Transforms/{c2c,r2c,r2r,no_transform}.jl``).  Julia's in-place names
ending in ``!`` are spelled with a trailing underscore (``FFT_`` for ``FFT!``).
The descriptors only describe; the arithmetic runs in the CUDA library.
"""
from __future__ import annotations

import numpy as np

from ._lib import ArgumentError

# FFTW r2r kind codes (fftw3.h), used unchanged by the reference and the C ABI.
R2HC, HC2R, DHT = 0, 1, 2
REDFT00, REDFT01, REDFT10, REDFT11 = 3, 4, 5, 6
RODFT00, RODFT01, RODFT10, RODFT11 = 7, 8, 9, 10
R2R_SUPPORTED_KINDS = (DHT, REDFT00, REDFT01, REDFT10, REDFT11,
                       RODFT00, RODFT01, RODFT10, RODFT11)
_KIND_NAMES = {R2HC: "R2HC", HC2R: "HC2R", DHT: "DHT", REDFT00: "REDFT00",
               REDFT01: "REDFT01", REDFT10: "REDFT10", REDFT11: "REDFT11",
               RODFT00: "RODFT00", RODFT01: "RODFT01", RODFT10: "RODFT10",
               RODFT11: "RODFT11"}


def kind2string(k: int) -> str:
    return _KIND_NAMES.get(k, str(k))


class AbstractTransform:
    """reference Transforms.jl:31."""
    inplace = False
    _abi_kind = -1

    def __eq__(self, other):
        return type(self) is type(other) and self.__dict__ == other.__dict__

    def __hash__(self):
        return hash((type(self).__name__, tuple(sorted(self.__dict__.items()))))

    def __repr__(self):
        return type(self).__name__.replace("_", "!")


# -- c2c (reference src/Transforms/c2c.jl) --------------------------------------
class FFT(AbstractTransform):
    _abi_kind = 0


class FFT_(FFT):
    inplace = True


class BFFT(AbstractTransform):
    _abi_kind = 1


class BFFT_(BFFT):
    inplace = True


# -- r2c / c2r (reference src/Transforms/r2c.jl) ------------------------------
class RFFT(AbstractTransform):
    _abi_kind = 2


class RFFT_(RFFT):
    inplace = True


class BRFFT(AbstractTransform):
    """reference r2c.jl:45-69: ``BRFFT(d)`` stores ``iseven(d)``; a tuple uses its last entry."""
    _abi_kind = 3

    def __init__(self, d=None, *, even_output: bool | None = None):
        if even_output is None:
            if isinstance(d, (tuple, list)):
                d = d[-1]
            even_output = int(d) % 2 == 0
        self.even_output = bool(even_output)

    def __repr__(self):
        return super().__repr__() + ("{even}" if self.even_output else "{odd}")


class BRFFT_(BRFFT):
    inplace = True


# -- r2r (reference src/Transforms/r2r.jl) -------------------------------------
class R2R(AbstractTransform):
    """reference r2r.jl:38-57: unsupported kinds raise ArgumentError."""
    _abi_kind = 4

    def __init__(self, kind: int):
        if kind not in R2R_SUPPORTED_KINDS:
            raise ArgumentError(f"unsupported r2r transform kind: {kind2string(kind)}")
        self.kind = int(kind)

    def __repr__(self):
        return f"{super().__repr__()}{{{kind2string(self.kind)}}}"


class R2R_(R2R):
    inplace = True


# -- identity (reference src/Transforms/no_transform.jl) -----------------------
class NoTransform(AbstractTransform):
    _abi_kind = 5


class NoTransform_(NoTransform):
    inplace = True


def kind(tr: R2R) -> int:
    """reference r2r.jl:76."""
    return tr.kind


def is_inplace(*trs):
    """reference Transforms.jl:141-147: None for a mix of in/out-of-place."""
    if len(trs) == 1:
        return trs[0].inplace
    flags = {t.inplace for t in trs}
    return flags.pop() if len(flags) == 1 else None


_R2R_INV = {REDFT00: REDFT00, REDFT01: REDFT10, REDFT10: REDFT01, REDFT11: REDFT11,
            RODFT00: RODFT00, RODFT01: RODFT10, RODFT10: RODFT01, RODFT11: RODFT11,
            DHT: DHT}


def _same_family(tr, cls_oop, cls_ip):
    return cls_ip() if tr.inplace else cls_oop()


def binv(tr: AbstractTransform, d: int) -> AbstractTransform:
    """reference c2c.jl:58-61, r2c.jl:98-101, r2r.jl:103-131, no_transform.jl:23."""
    if isinstance(tr, FFT):
        return _same_family(tr, BFFT, BFFT_)
    if isinstance(tr, BFFT):
        return _same_family(tr, FFT, FFT_)
    if isinstance(tr, RFFT):
        return BRFFT_(d) if tr.inplace else BRFFT(d)
    if isinstance(tr, BRFFT):
        return _same_family(tr, RFFT, RFFT_)
    if isinstance(tr, R2R):
        return (R2R_ if tr.inplace else R2R)(_R2R_INV[tr.kind])
    return tr


def length_output(tr: AbstractTransform, length_in: int) -> int:
    """reference c2c.jl:47, r2c.jl:74-75, r2r.jl:78, no_transform.jl:24."""
    if isinstance(tr, RFFT):
        return length_in // 2 + 1
    if isinstance(tr, BRFFT):
        return 2 * length_in - 1 - int(tr.even_output)
    return length_in


def _dims_tuple(dims, ndim):
    if dims is None:
        return tuple(range(1, ndim + 1))
    if isinstance(dims, int):
        return (dims,)
    if isinstance(dims, range):
        return tuple(dims)
    return tuple(dims)


def scale_factor(tr: AbstractTransform, A, dims=None) -> int:
    """Normalisation factor of ``tr`` on an array ``A`` along the 1-based ``dims``.

    ``A`` is an array (numpy/torch) or a shape tuple of the transform input.
    reference Transforms.jl:195-197, c2c.jl:71, r2c.jl:103-111,
    r2r.jl:96-101, no_transform.jl:26.
    """
    shape = tuple(A) if isinstance(A, tuple) else tuple(A.shape)
    dims = _dims_tuple(dims, len(shape))
    dtype = None if isinstance(A, tuple) else getattr(A, "dtype", None)
    is_cplx = None
    if dtype is not None:
        is_cplx = np.dtype(str(dtype).replace("torch.", "")).kind == "c"
    if isinstance(tr, RFFT) and is_cplx:
        raise TypeError(f"no method matching scale_factor({tr!r}, complex array)")
    if isinstance(tr, BRFFT) and is_cplx is False:
        raise TypeError(f"no method matching scale_factor({tr!r}, real array)")
    s = 1
    for i in dims:
        n = shape[i - 1]
        if isinstance(tr, (FFT, BFFT, RFFT)):
            s *= n
        elif isinstance(tr, BRFFT):
            s *= length_output(tr, n) if i == dims[-1] else n
        elif isinstance(tr, R2R):
            if tr.kind == REDFT00:
                s *= 2 * (n - 1)
            elif tr.kind == RODFT00:
                s *= 2 * (n + 1)
            elif tr.kind == DHT:
                s *= n
            else:
                s *= 2 * n
    return s


def expand_dims(tr: AbstractTransform, N: int) -> tuple:
    """reference Transforms.jl:285-291 and r2c.jl:114-124."""
    if N == 0:
        return ()
    if isinstance(tr, RFFT):
        rest = FFT_ if tr.inplace else FFT
        return (tr,) + tuple(rest() for _ in range(N - 1))
    if isinstance(tr, BRFFT):
        first = BFFT_ if tr.inplace else BFFT
        return tuple(first() for _ in range(N - 1)) + (tr,)
    return tuple(tr for _ in range(N))


def eltype_input(tr: AbstractTransform, real_type):
    """reference c2c.jl:49, r2c.jl:80-81, r2r.jl:79, no_transform.jl:25.

    ``None`` for transforms that accept both real and complex data.
    """
    real_type = np.dtype(real_type)
    cplx = np.dtype(np.complex64) if real_type == np.float32 else np.dtype(np.complex128)
    if isinstance(tr, (FFT, BFFT, BRFFT)):
        return cplx
    if isinstance(tr, RFFT):
        return real_type
    return None


def eltype_output(tr: AbstractTransform, t):
    """reference Transforms.jl:235-236, c2c.jl:48, r2c.jl:77-78, r2r.jl:80."""
    t = np.dtype(t)
    name = repr(tr)
    if isinstance(tr, (FFT, BFFT)):
        if t.kind != "c":
            raise ArgumentError(f"invalid input data type for {name}: {t}")
        return t
    if isinstance(tr, RFFT):
        if t.kind != "f":
            raise ArgumentError(f"invalid input data type for {name}: {t}")
        return np.dtype(np.complex64) if t == np.float32 else np.dtype(np.complex128)
    if isinstance(tr, BRFFT):
        if t.kind != "c":
            raise ArgumentError(f"invalid input data type for {name}: {t}")
        return np.dtype(np.float32) if t == np.complex64 else np.dtype(np.float64)
    return t
