"""Pencil decomposition over several GPUs: the reference's distributed path.

PencilFFTs splits an N-dimensional array over an M-dimensional Cartesian
grid of processes (``proc_dims``, M < N) and transforms one dimension at a
time: every 1D transform runs on a *pencil*, a configuration in which the
transformed dimension is local to each process, and consecutive pencils are
connected by a global transposition in which each process exchanges
sub-blocks with the processes of one row or column of the grid.  This module
restates that structure on ``torch.distributed`` (NCCL between GPUs, gloo on
the host):

* ``Topology``: the process grid; coordinates in row-major order (the last
  grid dimension varies fastest), as ``MPI.Cart_create`` without reordering
  (reference ``src/PencilFFTs.jl``, via PencilArrays' ``MPITopology``).
* ``local_range``: the balanced block partition of a dimension over the
  processes of one grid axis (PencilArrays' ``local_data_range``: process
  ``p`` of ``P`` owns ``[n p / P, n (p + 1) / P)``, 0-based).  PencilArrays is
  a dependency of the reference (compat 0.19) not contained in its tree; the
  rule is restated from its published definition.
* ``pencil_decompositions``: the decomposed dimensions of every stage
  (reference ``src/plans.jl:451-500``): the input pencil is split along the
  last M dimensions (``input_decomposition``); the pencil of transform n
  replaces dimension n, if it was split, by n - 1 on the same grid axis.
* ``DistributedPencilFFTPlan``: forward (``mul!``) and backward (``bmul!``,
  ``ldiv!``) transforms on the local blocks (reference
  ``src/operations.jl:227-257``): transpose into the next pencil, then the 1D
  transform along the now-local dimension; the backward transform applies
  the inverse transforms in reverse order and divides by the product of the
  scale factors.
* Transpositions (PencilArrays' ``transpose!``, called at
  ``src/operations.jl:239-240``): ``"PointToPoint"`` (non-blocking sends and
  receives to each process of the row or column, then a wait: the
  reference's default ``Transpositions.PointToPoint()`` and
  ``_wait_mpi_operations!``, ``src/operations.jl:259-262``) or
  ``"Alltoallv"`` (one all-to-all with per-process counts over the row or
  column's process group).

Each 1D transform runs on the local block through ``local_transform``; the
default builds (and caches) a single-dimension ``PencilFFTPlan`` of the
block's shape and runs the library's kernels on the GPU.  The exchanged
pieces are packed into contiguous send buffers and unpacked into the next
pencil's block with tensor copies on the same device, so the data stays in
local memory between the exchange and the next transform (no access to
another GPU's memory).

Local blocks are tensors in *logical index order* (shape = the local sizes
of dimensions 1..N).  Extra (batch) dimensions are not supported here.
This path has been run only with host (gloo) process groups: a multi-GPU
box was not available to measure it.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional, Sequence

import numpy as np

from . import transforms as Tr
from ._lib import ArgumentError


def _torch():
    import torch
    return torch


# ---------------------------------------------------------------------------
# partition and topology
# ---------------------------------------------------------------------------
def local_range(p: int, P: int, n: int) -> range:
    """Indices of dimension of size ``n`` owned by process ``p`` of ``P``
    (0-based, balanced blocks; PencilArrays' ``local_data_range``)."""
    if not (0 <= p < P):
        raise ArgumentError(f"process {p} not in 0:{P - 1}")
    return range((n * p) // P, (n * (p + 1)) // P)


@dataclass(frozen=True)
class Topology:
    """Cartesian grid of processes, coordinates in row-major order."""
    dims: tuple

    @property
    def size(self) -> int:
        return int(np.prod(self.dims))

    def coords(self, rank: int) -> tuple:
        c = []
        for P in reversed(self.dims):
            c.append(rank % P)
            rank //= P
        return tuple(reversed(c))

    def rank_of(self, coords: Sequence[int]) -> int:
        r = 0
        for c, P in zip(coords, self.dims):
            r = r * P + int(c)
        return r

    def axis_group(self, rank: int, axis: int) -> list:
        """Ranks sharing every coordinate of ``rank`` but the one along
        ``axis``, ordered by that coordinate (a row or column of the grid)."""
        c = list(self.coords(rank))
        out = []
        for j in range(self.dims[axis]):
            c[axis] = j
            out.append(self.rank_of(c))
        return out


def input_decomposition(N: int, M: int) -> tuple:
    """Decomposed dimensions of the input pencil: the last M (0-based)."""
    return tuple(range(N - M, N))


def pencil_decompositions(N: int, M: int) -> list:
    """Decomposed dimensions (per grid axis) of the pencil of each transform
    n = 0..N-1 (reference src/plans.jl:451-500, ``_make_intermediate_pencil``)."""
    dec = [input_decomposition(N, M)]
    for n in range(1, N):
        prev = dec[-1]
        dec.append(tuple(d - 1 if d == n else d for d in prev))
        assert len(set(dec[-1])) == M
    return dec


@dataclass(frozen=True)
class PencilConfig:
    """Global sizes and decomposed dimensions (``decomp[i]`` is split over
    grid axis i)."""
    size_global: tuple
    decomp: tuple
    topology: Topology

    def range_local(self, rank: int) -> tuple:
        c = self.topology.coords(rank)
        r = [range(0, n) for n in self.size_global]
        for i, d in enumerate(self.decomp):
            r[d] = local_range(c[i], self.topology.dims[i], self.size_global[d])
        return tuple(r)

    def size_local(self, rank: int) -> tuple:
        return tuple(len(r) for r in self.range_local(rank))


# ---------------------------------------------------------------------------
# local 1D transforms on the GPU (the library's kernels)
# ---------------------------------------------------------------------------
class GPULocalTransforms:
    """Runs the 1D transform of one stage on a local block with a cached
    single-dimension PencilFFTPlan (the other dimensions NoTransform)."""

    def __init__(self, real_type):
        self.real_type = np.dtype(real_type)
        self._plans = {}

    def __call__(self, x, axis: int, tr, n_out: int):
        from .plans import PencilArray, PencilFFTPlan, mul_
        torch = _torch()
        if x.is_complex() and isinstance(tr, Tr.R2R):
            # an R2R stage on complex data (after an FFT stage): the real and
            # imaginary parts as one real block with a trailing dimension of 2
            # (a plan of R2R and NoTransform alone takes real input)
            y = self(torch.view_as_real(x.contiguous()), axis, tr, n_out)
            return torch.view_as_complex(y.contiguous())
        N = x.dim()
        # a C-ordered logical block is the column-major array of the
        # reversed dimensions: transform dimension N - 1 - axis of that plan
        dims = tuple(reversed(x.shape))
        trs = [Tr.NoTransform()] * N
        trs[N - 1 - axis] = tr
        key = (dims, axis, repr(tr))
        plan = self._plans.get(key)
        if plan is None:
            plan = PencilFFTPlan(dims, tuple(trs), self.real_type, permute_dims=False)
            self._plans[key] = plan
        pin, pout = plan.pencil_input(), plan.pencil_output()
        src = PencilArray(pin, x.contiguous().view(pin.memory_shape()), plan.eltype_input())
        out = torch.empty(pout.memory_shape(), dtype=_torch_dtype(plan.eltype_output()), device=x.device)
        dst = PencilArray(pout, out, plan.eltype_output())
        mul_(dst, plan, src)
        assert out.shape[axis] == n_out
        return out


def _torch_dtype(dt):
    torch = _torch()
    return {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
            np.dtype(np.complex64): torch.complex64, np.dtype(np.complex128): torch.complex128}[np.dtype(dt)]


# ---------------------------------------------------------------------------
# the distributed plan
# ---------------------------------------------------------------------------
class DistributedPencilFFTPlan:
    """``PencilFFTPlan(dims_global, transforms, proc_dims, comm, real_type)``
    with ``prod(proc_dims)`` processes of a ``torch.distributed`` group
    (reference src/plans.jl:241-320, src/operations.jl)."""

    def __init__(self, dims_global, transforms, proc_dims, real_type=np.float64, *,
                 group=None, transpose_method: str = "PointToPoint",
                 local_transform: Optional[Callable] = None):
        import torch.distributed as dist
        self.dims = tuple(int(n) for n in dims_global)
        N = len(self.dims)
        self.proc_dims = tuple(int(p) for p in proc_dims)
        M = len(self.proc_dims)
        if not 1 <= M < N:
            raise ArgumentError(f"the process grid must have between 1 and {N - 1} dimensions")
        if transpose_method not in ("PointToPoint", "Alltoallv"):
            raise ArgumentError(f"unknown transpose method {transpose_method!r}")
        self.transpose_method = transpose_method
        self.group = group
        self.rank = dist.get_rank(group)
        world = dist.get_world_size(group)
        self.topology = Topology(self.proc_dims)
        if self.topology.size != world:
            raise ArgumentError(f"proc_dims {self.proc_dims} need {self.topology.size} processes, "
                                f"the group has {world}")
        if isinstance(transforms, Tr.AbstractTransform):
            transforms = Tr.expand_dims(transforms, N)
        self.transforms = tuple(transforms)
        if len(self.transforms) != N:
            raise ArgumentError("number of transforms must equal the number of dimensions")
        if any(t.inplace for t in self.transforms):
            raise ArgumentError("the distributed plan takes out-of-place transforms")
        self.real_type = np.dtype(real_type)
        self.local_transform = local_transform or GPULocalTransforms(self.real_type)
        # global sizes before and after each 1D transform, and the scale
        sizes = [self.dims]
        scale = 1.0
        for n, t in enumerate(self.transforms):
            s = list(sizes[-1])
            s[n] = Tr.length_output(t, s[n])
            sizes.append(tuple(s))
            scale *= float(Tr.scale_factor(Tr.binv(t, sizes[-2][n]), (s[n],)))
        self.scale_factor = scale
        decs = pencil_decompositions(N, M)
        # pencil_in[n]: data before transform n; pencil_out[n]: after it
        self.pencil_in = [PencilConfig(sizes[n], decs[n], self.topology) for n in range(N)]
        self.pencil_out = [PencilConfig(sizes[n + 1], decs[n], self.topology) for n in range(N)]
        self._groups = None
        if transpose_method == "Alltoallv":
            # every process creates every row / column group, in one order
            self._groups = {}
            for axis in range(M):
                seen = set()
                for r in range(world):
                    g = tuple(self.topology.axis_group(r, axis))
                    if g in seen:
                        continue
                    seen.add(g)
                    pg = dist.new_group(list(g)) if group is None else dist.new_group(
                        [dist.get_global_rank(group, q) for q in g])
                    if self.rank in g:
                        self._groups[axis] = pg

    # -- pencils of the user-visible arrays -------------------------------
    def input_range(self, rank: Optional[int] = None) -> tuple:
        return self.pencil_in[0].range_local(self.rank if rank is None else rank)

    def output_range(self, rank: Optional[int] = None) -> tuple:
        return self.pencil_out[-1].range_local(self.rank if rank is None else rank)

    def eltype_input(self):
        """reference src/global_params.jl:81-95: the first transform with a
        fixed input type decides; real data when none does."""
        for t in self.transforms:
            e = Tr.eltype_input(t, self.real_type)
            if e is not None:
                return e
        return self.real_type

    def allocate_input(self, device=None):
        torch = _torch()
        return torch.zeros(self.pencil_in[0].size_local(self.rank), dtype=_torch_dtype(self.eltype_input()),
                           device=device)

    # -- transposition between two pencils --------------------------------
    def _transpose(self, x, src: PencilConfig, dst: PencilConfig):
        """Moves the local block x of pencil src to pencil dst: the two differ
        on one grid axis, whose row or column of processes exchanges pieces."""
        import torch.distributed as dist
        torch = _torch()
        axes = [i for i, (a, b) in enumerate(zip(src.decomp, dst.decomp)) if a != b]
        if not axes:
            return x
        assert len(axes) == 1 and src.size_global == dst.size_global
        i = axes[0]
        a, b = src.decomp[i], dst.decomp[i]   # a: split in src, local in dst; b: the reverse
        members = self.topology.axis_group(self.rank, i)
        me = members.index(self.rank)
        # piece for member j: my block restricted along b to j's dst range
        send = []
        for r in members:
            rb = dst.range_local(r)[b]
            send.append(x.narrow(b, rb.start, len(rb)).contiguous())
        my_dst = dst.size_local(self.rank)
        recv_shapes = []
        for r in members:
            s = list(my_dst)
            s[a] = len(src.range_local(r)[a])
            recv_shapes.append(tuple(s))
        recv = [torch.empty(s, dtype=x.dtype, device=x.device) for s in recv_shapes]
        if self.transpose_method == "PointToPoint":
            ops = []
            for j, r in enumerate(members):
                if j == me:
                    recv[j].copy_(send[j])
                    continue
                gr = r if self.group is None else dist.get_global_rank(self.group, r)
                ops.append(dist.P2POp(dist.isend, send[j], gr, self.group))
                ops.append(dist.P2POp(dist.irecv, recv[j], gr, self.group))
            if ops:
                for req in dist.batch_isend_irecv(ops):
                    req.wait()
        else:
            sbuf = torch.cat([s.reshape(-1) for s in send])
            rbuf = torch.empty(sum(int(np.prod(s)) for s in recv_shapes), dtype=x.dtype, device=x.device)
            rview = torch.view_as_real(rbuf) if rbuf.is_complex() else rbuf
            sview = torch.view_as_real(sbuf) if sbuf.is_complex() else sbuf
            k = 2 if rbuf.is_complex() else 1
            dist.all_to_all_single(rview.reshape(-1), sview.reshape(-1),
                                   [k * int(np.prod(s)) for s in recv_shapes],
                                   [k * s.numel() for s in send], group=self._groups[i])
            off = 0
            for j, s in enumerate(recv_shapes):
                n = int(np.prod(s))
                recv[j] = rbuf[off:off + n].view(s)
                off += n
        return torch.cat(recv, dim=a)

    # -- transforms (reference src/operations.jl:24-70, 227-257) ----------
    def forward(self, u):
        """``mul!``: the local block of the output pencil."""
        x = u
        for n, t in enumerate(self.transforms):
            if n > 0:
                x = self._transpose(x, self.pencil_out[n - 1], self.pencil_in[n])
            x = self._apply(x, n, t, self.pencil_out[n].size_global[n])
        return x

    def backward(self, v, normalise: bool = True):
        """``ldiv!`` (normalise) or ``bmul!``: the local block of the input pencil."""
        x = v
        N = len(self.dims)
        for n in range(N - 1, -1, -1):
            if n < N - 1:
                x = self._transpose(x, self.pencil_in[n + 1], self.pencil_out[n])
            tb = Tr.binv(self.transforms[n], self.dims[n])
            x = self._apply(x, n, tb, self.dims[n])
        if normalise:
            x = x / self.scale_factor
        return x

    def _apply(self, x, n, t, n_out):
        if isinstance(t, Tr.NoTransform):
            return x
        return self.local_transform(x, n, t, n_out)
