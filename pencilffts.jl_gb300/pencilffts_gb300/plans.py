"""``PencilFFTPlan``, pencil arrays and the ``mul!``/``ldiv!``/``bmul!`` API.

Host-side mirror of the reference's user API (``src/plans.jl``,
``src/operations.jl``, ``src/allocate.jl``, ``src/multiarrays_r2c.jl``) at
``proc_dims = (1, ..., 1)``.  Device memory comes from PyTorch; every transform
runs in libpencilfft_gb300.so through its C ABI.

Julia names ending in ``!`` are spelled with a trailing underscore:
``mul_(dst, plan, src)`` is ``mul!(dst, plan, src)``; ``plan * u`` works as in
Julia and ``ldiv(plan, uF)`` (or ``plan.ldiv(uF)``) is ``plan \\ uF``.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import ArgumentError, PlanDesc, PlanInfo
from . import transforms as T

_TORCH = None


def _torch():
    global _TORCH
    if _TORCH is None:
        import torch
        _TORCH = torch
    return _TORCH


def _torch_dtype(dt: np.dtype):
    torch = _torch()
    return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
            np.dtype(np.complex64): torch.complex64,
            np.dtype(np.complex128): torch.complex128}[np.dtype(dt)]


# ---------------------------------------------------------------------------
# Pencils and arrays
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Pencil:
    """Global logical sizes and memory order of one pencil configuration.

    ``perm`` lists the logical dimensions (0-based) from fastest to slowest in
    memory; extra dimensions always follow, slowest.  ``pitch0`` is the
    allocated length of the fastest dimension (padded real views of in-place
    r2c plans, reference src/multiarrays_r2c.jl:69-79).
    """
    dims: tuple
    perm: tuple
    extra_dims: tuple = ()
    pitch0: int = 0

    @property
    def ndims(self):
        return len(self.dims)

    def memory_shape(self) -> tuple:
        """C-order shape of the memory buffer (slowest first)."""
        fast = [self.dims[d] for d in self.perm]
        if self.pitch0:
            fast[0] = self.pitch0
        return tuple(reversed(self.extra_dims)) + tuple(reversed(fast))

    def logical_permutation(self) -> tuple:
        """Axes permutation taking the memory tensor to logical index order.

        Memory axis i < K holds extra dimension K-1-i; memory axis K+q holds
        logical dimension perm[N-1-q].
        """
        N, K = len(self.dims), len(self.extra_dims)
        axis_to_logical = [N + (K - 1 - i) for i in range(K)]
        axis_to_logical += [self.perm[N - 1 - q] for q in range(N)]
        inv = [0] * (N + K)
        for ax, lg in enumerate(axis_to_logical):
            inv[lg] = ax
        return tuple(inv)

    def size_global(self, logical=True):
        return self.dims if logical else tuple(self.dims[d] for d in self.perm)


class PencilArray:
    """A device array attached to a pencil (reference PencilArrays.PencilArray).

    ``parent`` is the torch tensor in memory order (C-order shape
    ``pencil.memory_shape()``); ``logical()`` is a view indexed like the
    Julia array ``u[i1, ..., iN, e1, ...]``.
    """

    def __init__(self, pencil: Pencil, data, dtype):
        self.pencil = pencil
        self.data = data
        self.dtype = np.dtype(dtype)

    @property
    def parent(self):
        return self.data

    def data_ptr(self) -> int:
        return self.data.data_ptr()

    def nbytes(self) -> int:
        return self.data.numel() * self.data.element_size()

    def logical(self):
        v = self.data.permute(*self.pencil.logical_permutation())
        if self.pencil.pitch0:
            d0 = self.pencil.perm[0]
            v = v.narrow(d0, 0, self.pencil.dims[d0])
        return v

    @property
    def shape(self):
        return tuple(self.pencil.dims) + tuple(self.pencil.extra_dims)

    def size_global(self):
        return self.shape

    def copy_from_logical(self, arr):
        """Fills the array from a logical numpy/torch array."""
        torch = _torch()
        src = torch.as_tensor(np.asarray(arr) if not isinstance(arr, torch.Tensor) else arr)
        self.logical().copy_(src.to(self.data.device, dtype=self.data.dtype))
        return self

    def to_logical(self) -> np.ndarray:
        """Host copy in logical index order (reference ``gather``)."""
        return np.ascontiguousarray(self.logical().cpu().numpy())

    def fill_(self, v):
        self.data.fill_(v)
        return self

    def __repr__(self):
        return f"PencilArray{{{self.dtype}}}(dims={self.shape}, perm={self.pencil.perm})"


class ManyPencilArray:
    """Several pencil views aliasing one buffer (reference PencilArrays.ManyPencilArray
    and ``ManyPencilArrayRFFT!``, src/multiarrays_r2c.jl:26-79).  ``first()`` is
    the input view, ``last()`` the output view of an in-place plan."""

    def __init__(self, buffer, arrays: Sequence[PencilArray]):
        self.buffer = buffer
        self.arrays = tuple(arrays)

    def first(self) -> PencilArray:
        return self.arrays[0]

    def last(self) -> PencilArray:
        return self.arrays[-1]

    def data_ptr(self) -> int:
        return self.buffer.data_ptr()

    def __repr__(self):
        return f"ManyPencilArray({', '.join(repr(a) for a in self.arrays)})"


def gather(A) -> np.ndarray:
    """reference PencilArrays.gather at one process: the full logical array."""
    return A.to_logical()


# ---------------------------------------------------------------------------
# Plan
# ---------------------------------------------------------------------------
def _expand(transforms, N):
    if isinstance(transforms, T.AbstractTransform):
        return T.expand_dims(transforms, N)
    transforms = tuple(transforms)
    if len(transforms) != N:
        raise ArgumentError(f"expected {N} transforms, got {len(transforms)}")
    return transforms


PRECISION = {"default": 0, "native": 1, "tc": 2, "fx": 3}

# FFTW planner flags (FFTW.jl values); PencilFFTs passes fftw_flags to FFTW's
# planner, default FFTW.ESTIMATE (reference src/plans.jl:241-320)
FFTW_MEASURE, FFTW_EXHAUSTIVE, FFTW_PATIENT, FFTW_ESTIMATE = 0, 1 << 3, 1 << 5, 1 << 6


def _autotune_from(fftw_flags, autotune):
    """Planner measurement on (1) when requested explicitly, or when the FFTW
    planner flags ask for anything beyond FFTW.ESTIMATE, as FFTW would
    measure its candidate plans."""
    if autotune is not None:
        return 1 if autotune else 0
    if fftw_flags is None:
        return 0
    return 0 if int(fftw_flags) & FFTW_ESTIMATE else 1


def _descriptor(dims, transforms, real_type, permute_dims, extra_dims, precision="default",
                autotune=0) -> PlanDesc:
    N = len(dims)
    if N < 1 or N > _lib.MAX_DIMS:
        raise ArgumentError(f"number of dimensions must be in [1, {_lib.MAX_DIMS}]")
    if len(extra_dims) > _lib.MAX_EXTRA:
        raise ArgumentError("too many extra dimensions")
    d = PlanDesc()
    d.ndims = N
    for n, (sz, tr) in enumerate(zip(dims, transforms)):
        d.dims[n] = int(sz)
        d.kind[n] = tr._abi_kind
        d.inplace[n] = 1 if tr.inplace else 0
        d.r2r_kind[n] = tr.kind if isinstance(tr, T.R2R) else 0
        d.brfft_even[n] = 1 if (isinstance(tr, T.BRFFT) and tr.even_output) else 0
    rt = np.dtype(real_type)
    if rt not in (np.dtype(np.float32), np.dtype(np.float64)):
        raise ArgumentError("real_type must be float32 or float64")
    d.real_bytes = rt.itemsize
    d.permute_dims = 1 if permute_dims else 0
    d.n_extra = len(extra_dims)
    for e, sz in enumerate(extra_dims):
        d.extra_dims[e] = int(sz)
    if precision not in PRECISION:
        raise ArgumentError(f"precision must be one of {tuple(PRECISION)}")
    d.precision_mode = PRECISION[precision]
    d.autotune = int(autotune)
    return d


def plan_query(dims, transforms, real_type=np.float64, *, permute_dims=True, extra_dims=(),
               precision="default"):
    """Host-only analysis of a plan through the C ABI (no GPU needed)."""
    dims = tuple(int(x) for x in dims)
    transforms = _expand(transforms, len(dims))
    desc = _descriptor(dims, transforms, real_type, permute_dims, tuple(extra_dims), precision)
    info = PlanInfo()
    L = _lib.load()
    _lib.check(L.pfgb_plan_query(ctypes.byref(desc), ctypes.byref(info)), "pfgb_plan_query")
    return info


class PencilFFTPlan:
    """N-dimensional FFT-based transform plan (reference ``PencilFFTPlan``).

    ``PencilFFTPlan(dims_global, transforms, real_type=float64; permute_dims,
    extra_dims)`` mirrors the reference constructor ``src/plans.jl:306-320``;
    ``proc_dims`` must be all ones (one GPU, no MPI).  ``precision`` selects
    the kernel arithmetic: "default" (Float64 plans: double-float on the FP32
    pipes for power-of-two, 3 * 2^k and 5 * 2^k lines, other lines up to 2048
    points (Bluestein), the R2R kinds through their power-of-two forms or
    extensions, and lines beyond one pass up to 2^23 points; FP64 for the
    few lengths left, see the C header), "native" (Float64 plans:
    FP64 everywhere), "fx" (Float64 plans: block floating point, 64-bit
    integer components with one power-of-two scale per line, for
    power-of-two lines) or "tc" (Float32 plans: c2c lines of 256, 512 and
    1024 points as tensor-core DFT-matrix products with a tf32 hi/lo split;
    rel. L2 about 1e-6).  ``fftw_flags`` other than FFTW.ESTIMATE (e.g. FFTW.MEASURE =
    0), or ``autotune=True``, make plan creation time the alternative kernels
    of each pass and keep the faster, as FFTW measures its candidates.
    ``fftw_timelimit`` and ``transpose_method`` are accepted and ignored, as
    the reference does for GPU arrays (src/plans.jl:325-332).
    """

    def __init__(self, dims_global, transforms, real_type=np.float64, *,
                 proc_dims=None, permute_dims=True, extra_dims=(),
                 fftw_flags=None, fftw_timelimit=None, transpose_method=None,
                 timer=None, stream=None, precision="default", autotune=None):
        dims = tuple(int(x) for x in dims_global)
        if proc_dims is not None and any(int(p) != 1 for p in proc_dims):
            raise ArgumentError("this implementation runs on one GPU: proc_dims must be all ones")
        if isinstance(permute_dims, bool) is False and permute_dims not in (0, 1):
            raise ArgumentError("permute_dims must be a Bool")
        self.transforms = _expand(transforms, len(dims))
        if T.is_inplace(*self.transforms) is None:
            raise ArgumentError(
                f"cannot combine in-place and out-of-place transforms: {self.transforms}")
        self.real_type = np.dtype(real_type)
        self.permute_dims = bool(permute_dims)
        self.extra_dims = tuple(int(e) for e in extra_dims)
        self.timer = timer
        self._stream = stream
        self.precision = precision
        self.autotune = _autotune_from(fftw_flags, autotune)
        desc = _descriptor(dims, self.transforms, self.real_type, self.permute_dims, self.extra_dims,
                           precision, self.autotune)
        L = _lib.load()
        handle = ctypes.c_void_p()
        _lib.check(L.pfgb_plan_create(ctypes.byref(desc), ctypes.byref(handle)), "pfgb_plan_create")
        self._handle = handle
        self._L = L
        info = PlanInfo()
        _lib.check(L.pfgb_plan_info_get(handle, ctypes.byref(info)), "pfgb_plan_info_get")
        self.info = info
        N = len(dims)
        self.ndims = N
        self.size_global_in = dims
        self.size_global_out = tuple(int(info.dims_out[n]) for n in range(N))
        cdt = np.dtype(np.complex64) if self.real_type == np.float32 else np.dtype(np.complex128)
        self._eltype_in = cdt if info.eltype_in_complex else self.real_type
        self._eltype_out = cdt if info.eltype_out_complex else self.real_type
        self._scale = float(info.scale_factor)
        self._inplace = bool(info.inplace)
        perm_out = tuple(int(info.perm_out[q]) for q in range(N))
        natural = tuple(range(N))
        pad = 0
        if self._inplace and isinstance(self.transforms[0], T.RFFT):
            pad = 2 * (dims[0] // 2 + 1)
        self._pencil_in = Pencil(dims, natural, self.extra_dims, pad)
        self._pencil_out = Pencil(self.size_global_out, perm_out, self.extra_dims)

    # -- queries (reference plans.jl:338-361, 564-591) -------------------
    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                self._L.pfgb_plan_destroy(h)
            except Exception:
                pass
            self._handle = None

    def size(self):
        return self.size_global_in

    @property
    def scale_factor(self) -> float:
        return self._scale

    def is_inplace(self) -> bool:
        return self._inplace

    def eltype_input(self):
        return self._eltype_in

    def eltype_output(self):
        return self._eltype_out

    def pencil_input(self) -> Pencil:
        return self._pencil_in

    def pencil_output(self) -> Pencil:
        return self._pencil_out

    def get_comm(self):
        return None

    def __repr__(self):
        s = (f"Transforms: {self.transforms}\nInput type: {self._eltype_in}\n"
             f"Global dimensions: {self.size_global_in} -> {self.size_global_out}")
        if self.extra_dims:
            s += f"\nExtra dimensions: {self.extra_dims}"
        return s + "\nDevice: one GB300 (proc_dims all ones)"

    # -- per-pass timing (reference: TimerOutputs sections) -----------------
    def set_timing(self, on: bool = True):
        _lib.check(self._L.pfgb_plan_set_timing(self._handle, 1 if on else 0), "pfgb_plan_set_timing")

    def device_status(self):
        """Bits set by bounded device waits that gave up since the last call
        (1: TMA tile copy, 2: tensor-core product, 4: a wait for the copies or
        products in flight gave up too); synchronises the plan's stream and
        clears them."""
        flags = ctypes.c_int32(0)
        _lib.check(self._L.pfgb_device_status(self._handle, self._stream_ptr(), ctypes.byref(flags)),
                   "pfgb_device_status")
        return flags.value

    def set_wait_test(self, polls: int, tma: bool = False):
        """Test hook of the bounded waits' give-up path: with ``polls > 0`` the
        first data wait of every CTA of the persistent kernels polls an
        mbarrier that nothing signals ``polls`` times and gives up; ``tma``
        also runs eligible c2r passes in the TMA-fed form.  ``polls=0`` and
        ``tma=False`` restore normal execution."""
        _lib.check(self._L.pfgb_plan_set_wait_test(self._handle, int(polls), 1 if tma else 0),
                   "pfgb_plan_set_wait_test")

    def get_timing(self):
        """Per-pass event timings recorded since the last call (synchronises)."""
        buf = (_lib.PassTiming * 64)()
        n = ctypes.c_int(0)
        _lib.check(self._L.pfgb_plan_get_timing(self._handle, buf, 64, ctypes.byref(n)),
                   "pfgb_plan_get_timing")
        out = []
        for i in range(min(n.value, 64)):
            e = buf[i]
            out.append(dict(direction=e.direction, pass_=e.pass_, axis=e.axis, op=e.op,
                            launches=e.launches, total_ms=e.total_ms,
                            bytes_per_launch=e.bytes_per_launch,
                            kernel=e.kernel.decode()))
        return out

    # -- allocation (reference src/allocate.jl) ----------------------------
    def _new_pencil_array(self, pencil: Pencil, dtype):
        torch = _torch()
        t = torch.empty(pencil.memory_shape(), dtype=_torch_dtype(dtype), device="cuda")
        return PencilArray(pencil, t, dtype)

    def _new_many(self):
        torch = _torch()
        nbytes = int(self.info.inplace_bytes)
        buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        views = []
        for pen, dt in ((self._pencil_in, self._eltype_in), (self._pencil_out, self._eltype_out)):
            shape = pen.memory_shape()
            n = int(np.prod(shape)) * np.dtype(dt).itemsize
            t = buf[:n].view(_torch_dtype(dt)).view(shape)
            views.append(PencilArray(pen, t, dt))
        return ManyPencilArray(buf, views)

    def _allocate(self, which):
        if self._inplace:
            return self._new_many()
        if which == "in":
            return self._new_pencil_array(self._pencil_in, self._eltype_in)
        return self._new_pencil_array(self._pencil_out, self._eltype_out)

    def allocate_input(self, *dims):
        return _allocate_many(lambda: self._allocate("in"), dims)

    def allocate_output(self, *dims):
        return _allocate_many(lambda: self._allocate("out"), dims)

    # -- execution ---------------------------------------------------------
    def _stream_ptr(self):
        if self._stream is not None:
            return ctypes.c_void_p(int(self._stream))
        torch = _torch()
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _check_arrays(self, A_in, A_out):
        """reference operations.jl:87-127.  ``A_in`` holds data of the plan's
        input pencil and ``A_out`` of its output pencil (for a backward
        transform, the destination and the source respectively)."""
        s = "in-place" if self._inplace else "out-of-place"
        if self._inplace:
            if not (isinstance(A_in, ManyPencilArray) and isinstance(A_out, ManyPencilArray)):
                raise ArgumentError(f"array types ({type(A_in).__name__}, {type(A_out).__name__}) "
                                    f"incompatible with {s} plans")
            if A_in is not A_out:
                raise ArgumentError("input and output arrays for in-place plan must be the same")
            pin, pout = A_in.first(), A_in.last()
        else:
            if not (isinstance(A_in, PencilArray) and isinstance(A_out, PencilArray)):
                raise ArgumentError(f"array types ({type(A_in).__name__}, {type(A_out).__name__}) "
                                    f"incompatible with {s} plans")
            a0, a1 = A_in.data_ptr(), A_in.data_ptr() + A_in.nbytes()
            b0, b1 = A_out.data_ptr(), A_out.data_ptr() + A_out.nbytes()
            if a0 < b1 and b0 < a1:
                raise ArgumentError("out-of-place plan applied to aliased data")
            pin, pout = A_in, A_out
        if pin.pencil != self._pencil_in or pin.dtype != self._eltype_in:
            raise ArgumentError("unexpected dimensions of input data")
        if pout.pencil != self._pencil_out or pout.dtype != self._eltype_out:
            raise ArgumentError("unexpected dimensions of output data")

    def _run(self, dst, src, forward: bool, normalise: bool, deriv=None):
        L = self._L
        stream = self._stream_ptr()
        d = s = None
        if deriv is not None:
            dim, length = deriv
            if not (1 <= int(dim) <= self.ndims):
                raise ArgumentError(f"derivative dimension {dim} not in 1:{self.ndims}")
            d, s = int(dim) - 1, float(length)
        if forward:
            self._check_arrays(src, dst)
            if d is None:
                rc = L.pfgb_forward(self._handle, ctypes.c_void_p(dst.data_ptr()),
                                    ctypes.c_void_p(src.data_ptr()), stream)
            else:
                rc = L.pfgb_forward_deriv(self._handle, ctypes.c_void_p(dst.data_ptr()),
                                          ctypes.c_void_p(src.data_ptr()), stream, d, s)
            _lib.check(rc, "pfgb_forward")
        else:
            self._check_arrays(dst, src)
            if d is None:
                rc = L.pfgb_backward(self._handle, ctypes.c_void_p(dst.data_ptr()),
                                     ctypes.c_void_p(src.data_ptr()), stream, 1 if normalise else 0)
            else:
                rc = L.pfgb_backward_deriv(self._handle, ctypes.c_void_p(dst.data_ptr()),
                                           ctypes.c_void_p(src.data_ptr()), stream,
                                           1 if normalise else 0, d, s)
            _lib.check(rc, "pfgb_backward")
        return dst

    def _maybe_allocate(self, which, src):
        """reference operations.jl:72-85."""
        s = "in-place" if self._inplace else "out-of-place"
        if self._inplace:
            if not isinstance(src, ManyPencilArray):
                raise ArgumentError(f"input array type {type(src).__name__} incompatible with {s} plans")
            return src
        if not isinstance(src, PencilArray):
            raise ArgumentError(f"input array type {type(src).__name__} incompatible with {s} plans")
        return self._allocate(which)

    def __mul__(self, src):
        """``plan * u`` (reference operations.jl:54-57); maps over collections."""
        if _is_collection(src):
            return type(src)(self * s for s in src) if isinstance(src, tuple) else [self * s for s in src]
        dst = self._maybe_allocate("out", src)
        return mul_(dst, self, src)

    def ldiv(self, src):
        """``plan \\ uF`` (reference operations.jl:59-62)."""
        if _is_collection(src):
            return type(src)(self.ldiv(s) for s in src) if isinstance(src, tuple) else [self.ldiv(s) for s in src]
        dst = self._maybe_allocate("in", src)
        return ldiv_(dst, self, src)


def _is_collection(x):
    return isinstance(x, (tuple, list))


def _allocate_many(alloc, dims):
    """reference allocate.jl:442-446: ``dims...`` -> nested lists, ``Val(N)`` -> tuple."""
    if not dims:
        return alloc()
    if len(dims) == 1 and isinstance(dims[0], Val):
        return tuple(alloc() for _ in range(dims[0].n))

    def build(ds):
        if len(ds) == 1:
            return [alloc() for _ in range(ds[0])]
        return [build(ds[1:]) for _ in range(ds[0])]
    return build(tuple(int(d) for d in dims))


class Val:
    """Stand-in for Julia's ``Val(N)`` in ``allocate_input(plan, Val(3))``."""

    def __init__(self, n):
        self.n = int(n)


def _flatten(x):
    if _is_collection(x):
        out = []
        for e in x:
            out.extend(_flatten(e))
        return out
    return [x]


def _check_compatible(a, b):
    """reference operations.jl:130-137."""
    if len(a) != len(b):
        raise ArgumentError(f"collections have different lengths: {len(a)} ≠ {len(b)}")


def _apply(dst, plan, src, forward, normalise, deriv=None):
    if _is_collection(dst) or _is_collection(src):
        if not (_is_collection(dst) and _is_collection(src)):
            raise ArgumentError("collections and single arrays cannot be mixed")
        _check_compatible(dst, src)
        for d, s in zip(dst, src):
            _apply(d, plan, s, forward, normalise, deriv)
        return dst
    return plan._run(dst, src, forward, normalise, deriv)


class Batch:
    """Batched form: many transforms recorded once and replayed with one
    launch (``pfgb_batch_create_ex`` / ``pfgb_batch_launch``).

    ``ops`` is a sequence of ``(fn, dst, plan, src)`` or
    ``(fn, dst, plan, src, deriv)`` with ``fn`` one of ``mul_``, ``ldiv_``,
    ``bmul_``, exactly as the calls would be written (``deriv=(dim, L)`` as
    in ``mul_`` / ``ldiv_``); the arrays are bound at construction and every
    ``launch()`` repeats all of the recorded transforms on their current
    contents.

    ``form``: ``"graph"`` (default) records every transform's launches into
    one CUDA graph with a branch per plan; ``"persistent"`` runs the whole batch as one
    launch of a persistent kernel walking a work list of every tile of every
    pass (Float32 plans whose passes all have a tile form; ``LibraryError``
    otherwise); ``"auto"`` takes the persistent form where possible, else
    the graph form; ``"measure"`` times the persistent form in several work-list
    orders and the graph form at construction, which runs the batch and so
    overwrites the destination arrays as FFTW's MEASURE planning does, and
    keeps the fastest.
    """

    FORMS = {"graph": _lib.BATCH_GRAPH, "persistent": _lib.BATCH_PERSISTENT, "auto": _lib.BATCH_AUTO,
             "measure": _lib.BATCH_MEASURE}

    def __init__(self, ops, form="graph"):
        ops = list(ops)
        if not ops:
            raise ArgumentError("empty batch")
        if form not in self.FORMS:
            raise ArgumentError(f"batch form must be one of {sorted(self.FORMS)}")
        n = len(ops)
        desc = (_lib.BatchOp * n)()
        self._keep = []
        for i, op in enumerate(ops):
            if len(op) == 4:
                (fn, dst, plan, src), deriv = op, None
            elif len(op) == 5:
                fn, dst, plan, src, deriv = op
            else:
                raise ArgumentError("batch operations are (fn, dst, plan, src[, deriv])")
            if fn is mul_:
                plan._check_arrays(src, dst)
                direction, norm = 1, 0
            elif fn in (ldiv_, bmul_):
                plan._check_arrays(dst, src)
                direction, norm = -1, 1 if fn is ldiv_ else 0
            else:
                raise ArgumentError("batch operations are mul_, ldiv_ or bmul_")
            d = desc[i]
            d.plan = plan._handle.value
            d.direction, d.normalise = direction, norm
            d.dst, d.src = dst.data_ptr(), src.data_ptr()
            d.deriv_dim, d.deriv_length = -1, 0.0
            if deriv is not None:
                dim, length = deriv
                if not (1 <= int(dim) <= plan.ndims):
                    raise ArgumentError(f"derivative dimension {dim} not in 1:{plan.ndims}")
                d.deriv_dim, d.deriv_length = int(dim) - 1, float(length)
            self._keep.append((plan, dst, src))
        self._L = ops[0][2]._L
        h = ctypes.c_void_p()
        _lib.check(self._L.pfgb_batch_create_ex(desc, n, self.FORMS[form], ctypes.byref(h)),
                   "pfgb_batch_create_ex")
        self._h = h

    def launch(self, stream=None):
        if stream is None:
            stream = _torch().cuda.current_stream().cuda_stream
        _lib.check(self._L.pfgb_batch_launch(self._h, ctypes.c_void_p(int(stream))), "pfgb_batch_launch")

    def info(self) -> dict:
        """The recorded form ("graph" or "persistent"), and for the persistent
        form its work list (passes, tiles), grid, shared memory per CTA and
        the wave size of the list's order; with ``form="measure"`` also the
        measured times (graph form, best persistent order)."""
        i = _lib.BatchInfo()
        _lib.check(self._L.pfgb_batch_get_info(self._h, ctypes.byref(i)), "pfgb_batch_get_info")
        return dict(form="persistent" if i.form == _lib.BATCH_PERSISTENT else "graph", transforms=i.transforms,
                    items=i.items, tiles=i.tiles, grid=i.grid, smem=i.smem, wave_bytes=i.wave_bytes,
                    graph_ms=i.graph_ms, persistent_ms=i.persistent_ms)

    @property
    def form(self) -> str:
        return self.info()["form"]

    def status(self, stream=None) -> int:
        """Bits set by dependency waits of the persistent kernel that gave up
        since the last call (8), cleared by the call; synchronises."""
        if stream is None:
            stream = _torch().cuda.current_stream().cuda_stream
        f = ctypes.c_int32(0)
        _lib.check(self._L.pfgb_batch_status(self._h, ctypes.c_void_p(int(stream)), ctypes.byref(f)),
                   "pfgb_batch_status")
        return f.value

    def set_wait_test(self, polls: int) -> None:
        """Test hook: bound every dependency wait of later launches at
        ``polls`` polls (0 restores the default)."""
        _lib.check(self._L.pfgb_batch_set_wait_test(self._h, int(polls)), "pfgb_batch_set_wait_test")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.pfgb_batch_destroy(h)
            except Exception:
                pass
            self._h = None


def export_wisdom(path) -> None:
    """Writes the planner's measured kernel choices to ``path`` (FFTW.jl's
    ``export_wisdom``)."""
    L = _lib.load()
    _lib.check(L.pfgb_wisdom_export(os.fsencode(path)), "pfgb_wisdom_export")


def import_wisdom(path) -> None:
    """Merges kernel choices from a file written by ``export_wisdom``
    (FFTW.jl's ``import_wisdom``); later plans with ``fftw_flags`` other than
    ``FFTW_ESTIMATE`` use them instead of measuring."""
    L = _lib.load()
    _lib.check(L.pfgb_wisdom_import(os.fsencode(path)), "pfgb_wisdom_import")


def forget_wisdom() -> None:
    """Clears the planner's kernel choices (FFTW.jl's ``forget_wisdom``)."""
    _lib.load().pfgb_wisdom_forget()


def wisdom_stats():
    """(entries, lookups answered since the last forget)."""
    L = _lib.load()
    e, h = ctypes.c_int32(0), ctypes.c_int32(0)
    _lib.check(L.pfgb_wisdom_stats(ctypes.byref(e), ctypes.byref(h)), "pfgb_wisdom_stats")
    return e.value, h.value


def mul_(dst, plan: PencilFFTPlan, src, *, deriv=None):
    """``mul!(dst, plan, src)``: forward transform (reference operations.jl:24-31).

    ``deriv=(dim, L)`` multiplies the output by ``i k_dim`` (the spectral
    derivative along the 1-based dimension ``dim`` of a periodic domain of
    length ``L``), fused into the last pass.
    """
    return _apply(dst, plan, src, True, False, deriv)


def ldiv_(dst, plan: PencilFFTPlan, src, *, deriv=None):
    """``ldiv!(dst, plan, src)``: normalised backward transform (operations.jl:44-52).

    ``deriv=(dim, L)`` transforms ``i k_dim * src`` instead (``src`` is not
    modified): the derivative along ``dim`` in physical space, fused into the
    first pass (the gradient of examples/gradient.jl without its extra sweep).
    """
    return _apply(dst, plan, src, False, True, deriv)


def ldiv_deriv_sum_(dst, plan: PencilFFTPlan, terms, *, normalise=True):
    """``dst = plan \\ (sum of coef * i k_dim * src)`` in one backward transform.

    ``terms`` is a sequence of 1 to 3 tuples ``(src, dim, coef, L)``: a
    spectral array (the plan's output), the 1-based dimension of the
    derivative, its coefficient and the domain length along ``dim``.  The
    sum is formed as the first backward pass reads the sources (which are
    not modified), so a divergence or a curl component costs one backward
    transform (reference: the Fourier-space ``divergence`` and ``curl!`` of
    test/include/FourierOperations.jl:18-86, each followed by ``ldiv!``).
    ``normalise=False`` gives ``bmul!`` instead of ``ldiv!``.
    """
    terms = list(terms)
    if not 1 <= len(terms) <= 3:
        raise ArgumentError("a sum of derivatives takes 1 to 3 terms")
    n = len(terms)
    srcs = (ctypes.c_void_p * n)()
    dims = (ctypes.c_int * n)()
    coefs = (ctypes.c_double * n)()
    lens = (ctypes.c_double * n)()
    for i, (src, dim, coef, L) in enumerate(terms):
        if not 1 <= int(dim) <= plan.ndims:
            raise ArgumentError(f"derivative dimension {dim} not in 1:{plan.ndims}")
        plan._check_arrays(dst, src)
        srcs[i] = src.data_ptr()
        dims[i] = int(dim) - 1
        coefs[i] = float(coef)
        lens[i] = float(L)
    rc = plan._L.pfgb_backward_deriv_sum(plan._handle, ctypes.c_void_p(dst.data_ptr()), srcs, n, dims,
                                         coefs, lens, plan._stream_ptr(), 1 if normalise else 0)
    _lib.check(rc, "pfgb_backward_deriv_sum")
    return dst


def ldiv_divergence_(dst, plan: PencilFFTPlan, uF, lengths):
    """Physical divergence of the vector field whose spectrum is ``uF`` (one
    spectral array per dimension): one fused backward transform."""
    if len(uF) != plan.ndims or len(lengths) != plan.ndims:
        raise ArgumentError("divergence: one component and one domain length per dimension")
    return ldiv_deriv_sum_(dst, plan, [(uF[d], d + 1, 1.0, lengths[d]) for d in range(plan.ndims)])


def ldiv_curl_(omega, plan: PencilFFTPlan, uF, lengths):
    """Physical curl of the 3D vector field whose spectrum is ``uF``:
    ``omega[a] = d_b u_c - d_c u_b`` for (a, b, c) cyclic, one fused backward
    transform per component (reference curl!, test/include/FourierOperations.jl:57-86)."""
    if plan.ndims != 3 or len(uF) != 3 or len(omega) != 3 or len(lengths) != 3:
        raise ArgumentError("curl: a 3D plan with three components and three domain lengths")
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        ldiv_deriv_sum_(omega[a], plan, [(uF[c], b + 1, 1.0, lengths[b]), (uF[b], c + 1, -1.0, lengths[c])])
    return omega


def bmul_(dst, plan: PencilFFTPlan, src, *, deriv=None):
    """``bmul!(dst, plan, src)``: unnormalised backward transform (operations.jl:34-41)."""
    return _apply(dst, plan, src, False, False, deriv)


def ldiv(plan: PencilFFTPlan, src):
    """``plan \\ src``."""
    return plan.ldiv(src)


def allocate_input(plan: PencilFFTPlan, *dims):
    return plan.allocate_input(*dims)


def allocate_output(plan: PencilFFTPlan, *dims):
    return plan.allocate_output(*dims)


def scale_factor(plan: PencilFFTPlan) -> float:
    return plan.scale_factor


def is_inplace(plan: PencilFFTPlan) -> bool:
    return plan.is_inplace()
