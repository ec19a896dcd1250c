"""Pencil decomposition over several processes (CPU, gloo).

The distributed plan (pencilffts_gb300.distributed) restates the reference's
MPI path: balanced block partition, P1 x P2 process grid, one pencil per
transform and a global transposition between consecutive pencils
(PointToPoint sends / receives or Alltoallv).  Here the processes are CPU
ranks on a gloo group and the local 1D transforms are the oracle's (the GPU
kernels need a device); each rank's output block must equal the matching
block of the single-process oracle transform, and ldiv! must return the
input block.  Partition and decomposition rules are checked on the host
against the reference's documented examples.
"""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_partition_and_decompositions():
    from pencilffts_gb300.distributed import (Topology, input_decomposition, local_range,
                                              pencil_decompositions)
    # balanced blocks covering 0:n
    for n, P in ((10, 3), (7, 4), (512, 16), (5, 5)):
        rs = [local_range(p, P, n) for p in range(P)]
        assert rs[0].start == 0 and rs[-1].stop == n
        assert all(a.stop == b.start for a, b in zip(rs, rs[1:]))
        assert max(len(r) for r in rs) - min(len(r) for r in rs) <= 1
    # reference src/plans.jl:100-104 (N = 5, M = 2 -> decomposed (4, 5), 1-based)
    assert input_decomposition(5, 2) == (3, 4)
    # 3D over a 2D grid: x-pencil (y, z) split, y-pencil (x, z), z-pencil (x, y)
    assert pencil_decompositions(3, 2) == [(1, 2), (0, 2), (0, 1)]
    assert pencil_decompositions(3, 1) == [(2,), (2,), (1,)]
    t = Topology((2, 3))
    assert [t.coords(r) for r in range(6)] == [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (1, 2)]
    assert t.axis_group(4, 0) == [1, 4] and t.axis_group(4, 1) == [3, 4, 5]


CASES = [
    # (dims, transforms, proc_dims per world size)
    ((16, 12, 10), "RFFT", {2: [(2,), (1, 2), (2, 1)], 4: [(2, 2), (4,)]}),
    ((9, 8, 7), "FFT", {2: [(2, 1)], 4: [(2, 2)]}),
    ((10, 6, 9), "MIXED", {2: [(1, 2)], 4: [(4, 1)]}),
]


def _transforms(T, name):
    if name == "RFFT":
        return T.RFFT()
    if name == "FFT":
        return T.FFT()
    return (T.R2R(T.REDFT10), T.RFFT(), T.FFT())


def _worker(rank, world, port, method, out):
    import torch
    import torch.distributed as dist
    for p in (REPO, os.path.join(REPO, "pencilffts.jl_gb300"), os.path.join(REPO, "tests")):
        sys.path.insert(0, p)
    import pencilffts_gb300 as P
    from pencilffts_gb300.distributed import DistributedPencilFFTPlan
    from oracle import pencilfft_oracle as O
    from helpers import to_oracle

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    T = P.Transforms

    def cpu_local(x, axis, tr, n_out):  # the oracle's 1D transform on the host block
        y = O.transform_1d(to_oracle(tr), x.numpy(), axis, n_out=n_out)
        return torch.from_numpy(np.ascontiguousarray(y))

    errs = []
    try:
        for dims, name, grids in CASES:
            for proc_dims in grids.get(world, []):
                tr = _transforms(T, name)
                plan = DistributedPencilFFTPlan(dims, tr, proc_dims, np.float64,
                                                transpose_method=method, local_transform=cpu_local)
                orc = O.OraclePlan(dims, tuple(to_oracle(t) for t in plan.transforms), np.float64)
                rng = np.random.default_rng(5)
                x = rng.standard_normal(dims)
                if np.dtype(plan.eltype_input()).kind == "c":
                    x = x + 1j * rng.standard_normal(dims)
                ri = plan.input_range()
                u = torch.from_numpy(np.ascontiguousarray(x[tuple(slice(r.start, r.stop) for r in ri)]))
                v = plan.forward(u)
                ref = orc.forward(x)
                ro = plan.output_range()
                ref_loc = ref[tuple(slice(r.start, r.stop) for r in ro)]
                assert tuple(v.shape) == ref_loc.shape, (v.shape, ref_loc.shape)
                e_f = float(np.linalg.norm(v.numpy() - ref_loc) / max(np.linalg.norm(ref), 1e-300))
                w = plan.backward(v)
                e_b = float(np.linalg.norm(w.numpy() - u.numpy()) / max(np.linalg.norm(x), 1e-300))
                assert plan.scale_factor == orc.scale
                errs.append((dims, name, proc_dims, e_f, e_b))
        out[rank] = errs
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 4])
@pytest.mark.parametrize("method", ["PointToPoint", "Alltoallv"])
def test_distributed_plan_matches_oracle(world, method):
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, method, out), nprocs=world, join=True)
        res = dict(out)
    assert sorted(res) == list(range(world))
    n = sum(len(g.get(world, [])) for _, _, g in CASES)
    for r in range(world):
        assert len(res[r]) == n
        for dims, name, pd, e_f, e_b in res[r]:
            assert e_f <= 1e-14 and e_b <= 1e-14, (r, dims, name, pd, e_f, e_b)


@pytest.mark.gpu
def test_distributed_plan_gpu_local_transforms_one_rank(cuda):
    """One rank (a process grid of ones): the default local transforms run
    the library's kernels on the GPU block; the result matches the oracle."""
    import torch
    import torch.distributed as dist
    import pencilffts_gb300 as P
    from pencilffts_gb300.distributed import DistributedPencilFFTPlan
    from oracle import pencilfft_oracle as O
    from helpers import to_oracle
    T = P.Transforms
    port = _free_port()
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=0, world_size=1)
    try:
        for dims, tr, pd in (((32, 24, 16), T.RFFT(), (1, 1)), ((12, 10, 33), (T.FFT(), T.FFT(), T.R2R(T.REDFT00)), (1,))):
            plan = DistributedPencilFFTPlan(dims, tr, pd, np.float64)
            orc = O.OraclePlan(dims, tuple(to_oracle(t) for t in plan.transforms), np.float64)
            rng = np.random.default_rng(2)
            x = rng.standard_normal(dims)
            if np.dtype(plan.eltype_input()).kind == "c":
                x = x + 1j * rng.standard_normal(dims)
            u = torch.from_numpy(x).cuda()
            v = plan.forward(u)
            ref = orc.forward(x)
            assert np.linalg.norm(v.cpu().numpy() - ref) / np.linalg.norm(ref) <= 1e-13
            w = plan.backward(v)
            assert np.linalg.norm(w.cpu().numpy() - x) / np.linalg.norm(x) <= 1e-13
    finally:
        dist.destroy_process_group()
