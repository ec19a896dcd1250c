#!/usr/bin/env python
"""Benchmark of the PencilFFTs transform path on GB300.

Workload (the reference's headline benchmark, benchmarks/benchmarks.jl:200-266,
at one GPU): a 3D Float64 RFFT plan on a 512^3 grid, permute_dims=true,
out-of-place; one step = ``mul!(v, plan, u)`` followed by ``ldiv!(u, plan, v)``
(a forward r2c + backward c2r round trip, the scaling fused in the last pass).
Input: uniform [-1, 1), seeded.  Every array is far larger than L2 (1.07 GB).

Prints one JSON line.  ``--impl reference`` times the CPU oracle (the
restatement of the reference path with scipy.fft, all host cores) on the same
workload instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "pencilffts.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "512^3 r2c+c2r round-trip ms"
UNIT = "ms"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--dims", default="512,512,512")
    ap.add_argument("--real", default="f64", choices=["f64", "f32"])
    ap.add_argument("--precision", default="default", choices=["default", "native", "fx", "tc"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the Float32 plain vs tensor-core split comparison")
    ap.add_argument("--cpu-sample-s", type=float, default=20.0,
                    help="approximate CPU seconds for the cpu_baseline sample")
    return ap.parse_args()


def workload(args):
    dims = tuple(int(x) for x in args.dims.split(","))
    rb = 8 if args.real == "f64" else 4
    return dims, rb


def alg_bytes_round_trip(dims, rb):
    """One read + one write per pass: forward R + C + 2C*(N-1)... for a 3D r2c
    this is R + 5C per direction (2(R + 5C) per round trip)."""
    import numpy as np
    n = int(np.prod(dims))
    R = n * rb
    C = (dims[0] // 2 + 1) * int(np.prod(dims[1:])) * 2 * rb
    N = len(dims)
    per_dir = (R + C) + 2 * C * (N - 1)
    return 2 * per_dir, R, C


# ---------------------------------------------------------------------------
# CPU oracle timing (cpu_baseline and the reference arm)
# ---------------------------------------------------------------------------
def time_cpu_oracle(dims, rb, budget_s, max_iters=None):
    """Times the oracle's forward + ldiv (scipy.fft, all host threads) on the
    full workload; returns (ms per round trip, iterations, threads)."""
    import numpy as np
    import scipy.fft as sfft
    from oracle import pencilfft_oracle as O

    threads = os.cpu_count() or 1
    real = np.float64 if rb == 8 else np.float32
    rng = np.random.default_rng(1)
    u = rng.uniform(-1.0, 1.0, size=dims).astype(real)
    plan = O.OraclePlan(dims, O.RFFT(), real)
    times = []
    t_start = time.perf_counter()
    with sfft.set_workers(threads):
        while True:
            t0 = time.perf_counter()
            v = plan.forward(u)
            u2 = plan.ldiv(v)
            times.append(time.perf_counter() - t0)
            del v, u2
            if max_iters is not None and len(times) >= max_iters:
                break
            if max_iters is None and time.perf_counter() - t_start >= budget_s:
                break
    return 1e3 * statistics.mean(times), len(times), threads


def max_over_ranks(value: float, world: int, device=None) -> float:
    """Max of a per-rank timing over all ranks (the slowest replica sets the
    step time); identity at one rank."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        # raw samples (the JSON line carries their summary); PFGB_CLOCKS_DIR
        # keeps them in a chosen folder
        self.path = os.path.join(os.environ.get("PFGB_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"clocks_bench_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(parts)
            except ValueError:
                pass
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "", 1).isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for i, nm in enumerate(names):
                if r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ---------------------------------------------------------------------------
# Float32 forms: plain path against the tensor-core split form
# ---------------------------------------------------------------------------
def measure_forms(P, dims, steps, warmup, dev):
    """Times the Float32 RFFT round trip of the same workload with the plain
    kernels and with the tensor-core split form (precision="tc"), and states
    each form's error: rel. L2 of the forward spectrum against the Float64
    plan's spectrum (the double-float path, parity-tested against the FP64
    oracle at 1e-13) and of the round trip against the input."""
    import numpy as np
    import torch

    T = P.Transforms
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    p64 = P.PencilFFTPlan(dims, T.RFFT(), np.float64)
    u64 = p64.allocate_input()
    u64.data.uniform_(-1.0, 1.0, generator=g)
    ref = p64 * u64
    ref_norm = torch.linalg.vector_norm(ref.data).item()
    stream = torch.cuda.current_stream()
    out = {}
    for name, prec in (("f32_plain", "default"), ("f32_tc_split", "tc")):
        p = P.PencilFFTPlan(dims, T.RFFT(), np.float32, precision=prec)
        u, v, w = p.allocate_input(), p.allocate_output(), p.allocate_input()
        u.data.copy_(u64.data)
        P.mul_(v, p, u)
        e_fwd = (torch.linalg.vector_norm(v.data.to(ref.data.dtype) - ref.data).item() / ref_norm)
        P.ldiv_(w, p, v)
        e_rt = (torch.linalg.vector_norm(w.data - u.data).item() / torch.linalg.vector_norm(u.data).item())
        for _ in range(warmup):
            P.mul_(v, p, u)
            P.ldiv_(w, p, v)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            P.mul_(v, p, u)
            P.ldiv_(w, p, v)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = {"value": e0.elapsed_time(e1) / steps, "unit": UNIT,
                     "rel_l2_forward": e_fwd, "rel_l2_round_trip": e_rt}
        del p, u, v, w
        torch.cuda.empty_cache()
    out["tc_split_speedup_vs_plain"] = out["f32_plain"]["value"] / out["f32_tc_split"]["value"]
    out["error_reference"] = ("forward: Float64 plan on the same input (double-float path, "
                              "parity-tested against the FP64 oracle at 1e-13); round trip: the input")
    del p64, u64, ref
    torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------------------
# the GB300 arm
# ---------------------------------------------------------------------------
def run_gpu(args, rank, world, local_rank):
    import numpy as np
    import torch
    import torch.distributed as dist

    import pencilffts_gb300 as P

    dims, rb = workload(args)
    real = np.float64 if rb == 8 else np.float32
    T = P.Transforms

    # CPU baseline first (host threads only, before any GPU work of this rank)
    cpu_baseline = None
    if rank == 0 and not args.no_cpu_baseline:
        ms, iters, threads = time_cpu_oracle(dims, rb, args.cpu_sample_s)
        cpu_baseline = {"value": ms, "unit": UNIT, "cores": threads, "kind": "port",
                        "sample": f"{iters} full {'x'.join(map(str, dims))} "
                                  f"{'Float64' if rb == 8 else 'Float32'} RFFT round trips "
                                  f"(oracle: scipy.fft pocketfft, {threads} threads)"}

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    plan = P.PencilFFTPlan(dims, T.RFFT(), real, precision=args.precision)
    u = plan.allocate_input()
    v = plan.allocate_output()
    g = torch.Generator(device=dev)
    g.manual_seed(1 + rank)
    u.data.uniform_(-1.0, 1.0, generator=g)
    stream = torch.cuda.current_stream()

    def step():
        P.mul_(v, plan, u)
        P.ldiv_(u, plan, v)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()

    # ---- timed region (device events on the launching stream) ----
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    plan.set_timing(True)
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    ms_total = e0.elapsed_time(e1)
    timing = plan.get_timing()
    plan.set_timing(False)
    ms_step = max_over_ranks(ms_total / args.steps, world, dev)

    # ---- roofline of the dominant kernel ----
    per_kernel = {}
    launches = 0
    for e in timing:
        k = per_kernel.setdefault(e["kernel"], {"ms": 0.0, "bytes": 0, "launches": 0})
        k["ms"] += e["total_ms"]
        k["bytes"] += e["bytes_per_launch"] * e["launches"]
        k["launches"] += e["launches"]
        launches += e["launches"]
    dom_name, dom = max(per_kernel.items(), key=lambda kv: kv[1]["ms"])
    avg_launch_s = dom["ms"] / dom["launches"] * 1e-3
    bytes_per_launch = dom["bytes"] / dom["launches"]
    achieved = bytes_per_launch / avg_launch_s / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    traffic = None
    try:
        prof = json.load(open(os.path.join(REPO, "profiles", "traffic.json")))
        key = f"{dom_name}|{'x'.join(map(str, dims))}"
        if key in prof:
            traffic = prof[key]["dram_bytes_per_launch"]
    except Exception:
        pass
    alg_rt, R, C = alg_bytes_round_trip(dims, rb)

    # ---- end to end through the public API with host buffers ----
    # Every step copies its input from pinned host memory and its result back.
    # The copies run on their own streams, double-buffered, so the copy-in of
    # step k+1 and the copy-out of step k-1 overlap the transforms of step k.
    e2e = None
    if not args.no_e2e:
        host_in = torch.empty(u.data.shape, dtype=u.data.dtype, pin_memory=True)
        host_in.uniform_(-1.0, 1.0)
        host_out = [torch.empty_like(host_in, pin_memory=True) for _ in range(2)]
        us = [plan.allocate_input() for _ in range(2)]
        ws = [plan.allocate_input() for _ in range(2)]
        s_in, s_cmp, s_out = (torch.cuda.Stream(device=dev) for _ in range(3))
        ev_in = [torch.cuda.Event() for _ in range(2)]
        ev_cmp = [torch.cuda.Event() for _ in range(2)]
        ev_out = [torch.cuda.Event() for _ in range(2)]
        used = [False, False]

        def e2e_step(k):
            sl = k & 1
            if used[sl]:
                s_in.wait_event(ev_cmp[sl])    # transforms of step k-2 read us[sl]
                s_cmp.wait_event(ev_out[sl])   # copy-out of step k-2 read ws[sl]
            with torch.cuda.stream(s_in):
                us[sl].data.copy_(host_in, non_blocking=True)
                ev_in[sl].record(s_in)
            s_cmp.wait_event(ev_in[sl])
            with torch.cuda.stream(s_cmp):
                P.mul_(v, plan, us[sl])
                P.ldiv_(ws[sl], plan, v)
                ev_cmp[sl].record(s_cmp)
            s_out.wait_event(ev_cmp[sl])
            with torch.cuda.stream(s_out):
                host_out[sl].copy_(ws[sl].data, non_blocking=True)
                ev_out[sl].record(s_out)
            used[sl] = True

        for k in range(2):
            e2e_step(k)
        torch.cuda.synchronize()
        barrier()
        # three timed repetitions of the K steps, median reported: the host
        # link is shared with other jobs on the machine and varies run to run
        samples = []
        for _ in range(3):
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record(s_in)
            for k in range(args.steps):
                e2e_step(k)
            s_in.wait_stream(s_out)
            f1.record(s_in)
            torch.cuda.synchronize()
            samples.append(f0.elapsed_time(f1) / args.steps)
        e2e_ms = max_over_ranks(statistics.median(samples), world, dev)
        nb = host_in.numel() * host_in.element_size()
        e2e = {"value": e2e_ms, "unit": UNIT, "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb,
               "pipelined": "copy-in / transforms / copy-out on three streams, double-buffered",
               "samples_ms": samples, "statistic": "median of 3 timed repetitions of the K steps"}
        # the result of the last step round-trips the input
        diff = host_out[(args.steps - 1) & 1].double() - host_in.double()
        e2e["round_trip_rel_l2"] = float(diff.norm() / host_in.double().norm())
        e2e["round_trip_max_rel"] = float(diff.abs().max() / host_in.double().abs().max())

    if rank != 0:
        return
    forms = None
    if not args.no_forms:
        forms = measure_forms(P, dims, args.steps, args.warmup, dev)
    line = {
        "metric": METRIC, "value": ms_step, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if rb == 8 else "f32", "data": "synthetic: uniform [-1,1), seeded",
        "config": {"workload": f"RFFT round trip {'x'.join(map(str, dims))} "
                               f"{'Float64' if rb == 8 else 'Float32'} (mul! + ldiv!), "
                               "permute_dims=true, out-of-place",
                   "dims": list(dims), "transforms": "RFFT (RFFT, FFT, FFT)",
                   "l2": "inputs larger than L2 (1.07 GB arrays)",
                   "precision": args.precision,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        # per direction: the forward (mul!) and backward (ldiv!) passes' device time
        "forward_ms": sum(e["total_ms"] for e in timing if e["direction"] > 0) / args.steps,
        "backward_ms": sum(e["total_ms"] for e in timing if e["direction"] < 0) / args.steps,
        "hbm_gbs": alg_rt / (ms_step * 1e-3) / 1e9 * world,
        # compulsory bytes: one read of the input and one write of the output
        # per direction, 2 (R + C)
        "compulsory_gbs": 2 * (R + C) / (ms_step * 1e-3) / 1e9 * world,
        "gflops": 2 * 2.5 * np.prod(dims) * np.log2(np.prod(dims)) / (ms_step * 1e-3) / 1e9 * world,
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                     "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "alg_bytes_per_launch": bytes_per_launch,
                     "avg_launch_ms": avg_launch_s * 1e3},
        "passes": [{k: e[k] for k in ("direction", "pass_", "axis", "launches", "total_ms",
                                      "bytes_per_launch", "kernel")} for e in timing],
        "cpu_baseline": cpu_baseline,
        "e2e": e2e,
        "gpu_launches": launches,
        "forms": forms,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    """Reference arm: the CPU restatement of the path (oracle, scipy.fft on all
    host threads), the same workload and metric; rank 0 only."""
    if rank != 0:
        return
    dims, rb = workload(args)
    time_cpu_oracle(dims, rb, 0, max_iters=max(1, min(args.warmup, 1)))  # warm-up
    ms, iters, threads = time_cpu_oracle(dims, rb, 0, max_iters=args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": 0,
        "steps": iters, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if rb == 8 else "f32",
        "data": "synthetic: uniform [-1,1), seeded",
        "config": {"workload": f"RFFT round trip {'x'.join(map(str, dims))} "
                               f"{'Float64' if rb == 8 else 'Float32'} (mul! + ldiv!), "
                               "permute_dims=true, out-of-place", "dims": list(dims)},
        "cpu_baseline": {"value": ms, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{iters} full round trips (oracle: scipy.fft pocketfft, "
                                   f"{threads} threads; Julia/FFTW are not installed)"},
        "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    try:
        run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
