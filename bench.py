"""Benchmark: PageRank GTEPS per iteration on one GB300.

Workload (N=1 line): PageRank, FP32, damping 0.85, 1/N init, 30 fixed
iterations on a seeded R-MAT graph, scale 22 (4,194,304 vertices, edge
factor 16, a/b/c/d = 0.57/0.19/0.19/0.05, self-loops and duplicates
removed), the configuration the reference's PageRank metric is quoted on.
A step is one full 30-iteration PageRank over the device-resident graph.
GTEPS = edges x iterations / time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 (launched with torch.distributed.run): the path does not shard a
single graph, so every rank runs an independent replica (weak scaling).
`--impl reference` times the CPU restatement of the reference's PageRank
(vertex-pull + consolidateRank, OpenMP over all host cores) on a bounded
sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

METRIC = "GTEPS (BFS, PageRank/iter) on 1 GB300: learned-switched vs best fixed variant"
SCALE, EDGE_FACTOR, SEED, ITERATIONS = 22, 16, 22, 30
HEADLINE_VARIANT = "pull-segmented"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self._t:
            self._t.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() in ("active", "1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _measured_peak():
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def pagerank_launches(variant: str, iterations: int) -> int:
    """Kernels of ours one bw_pagerank_run launches (memsets not counted)."""
    fused = variant in ("vertex-pull", "vertex-pull-warp", "vertex-pull-nodiv", "vertex-pull-warp-nodiv",
                        "pull-segmented")
    deg = 0 if variant in ("vertex-push", "vertex-push-warp") else 1
    seg = 3 if variant == "pull-segmented" else 0
    return deg + seg + 1 + iterations * (1 if fused else 2)


def run_ours(args):
    import torch
    import torch.distributed as dist

    import belewitte_gb300 as bw

    ws, rank, local = _dist()
    if ws > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    dev = local
    torch.cuda.set_device(dev)
    ctx = bw.Context(dev)
    stream = torch.cuda.current_stream()
    g = bw.DeviceGraph.generate("rmat", scale=SCALE, edge_factor=EDGE_FACTOR, seed=SEED, device=dev,
                                reps=bw.REP_FWD_CSR | bw.REP_REV_CSR)
    n, m = g.vertex_count, g.edge_count
    ranks = torch.empty(n, dtype=torch.float32, device=f"cuda:{dev}")
    variant = args.variant

    # ---- device-resident timed region ------------------------------------
    for _ in range(args.warmup):
        bw.pagerank(ctx, g, variant, ITERATIONS, ranks=ranks)
    iter_ms = []
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clocks:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.steps):
            run = bw.pagerank_schedule(ctx, g, [variant], ITERATIONS, ranks=ranks, time_iterations=True)
            iter_ms.extend(run.iteration_ms)
        t1.record(stream)
        torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    ms = t0.elapsed_time(t1)
    if ws > 1:
        t = torch.tensor([ms], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = ws * m * ITERATIONS / (ms_per_step * 1e-3) / 1e9

    # ---- roofline of the dominant kernel (one launch = one iteration) -----
    kernel_ms = float(np.mean(iter_ms))
    alg_bytes = 4 * m + 16 * n + 4              # CSR-pull compulsory bytes per iteration
    peak, peak_kind = _measured_peak()
    achieved = alg_bytes / (kernel_ms * 1e-3) / 1e9

    # ---- end to end through the C ABI with host buffers ----------------------
    host = g.to_host_arrays()
    rv = torch.from_numpy(host["rev_vertices"].view(np.int32)).pin_memory()
    re = torch.from_numpy(host["rev_edges"].view(np.int32)).pin_memory()
    out_host = torch.empty(n, dtype=torch.float32).pin_memory()
    d_rv = torch.empty_like(rv, device=f"cuda:{dev}")
    d_re = torch.empty_like(re, device=f"cuda:{dev}")
    import ctypes as C
    from belewitte_gb300 import _abi
    view = _abi.GraphView(n, m, 0, 0, d_rv.data_ptr(), d_re.data_ptr(), 0, 0, 0, 0)

    class _G:                                   # a DeviceGraph-shaped view over the copies
        vertex_count, edge_count = n, m
    eg = _G()
    eg.view = view
    e2e_times = []
    for i in range(args.warmup + args.steps):
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()
        t = time.perf_counter()
        d_rv.copy_(rv, non_blocking=True)
        d_re.copy_(re, non_blocking=True)
        bw.pagerank(ctx, eg, variant, ITERATIONS, ranks=ranks)
        out_host.copy_(ranks, non_blocking=True)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t)
    e2e_s = max(np.mean(e2e_times), 1e-9)
    if ws > 1:
        t = torch.tensor([e2e_s], device=f"cuda:{dev}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = ws * m * ITERATIONS / e2e_s / 1e9

    # ---- CPU baseline (rank 0, N=1): bounded sample on all host cores ----
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(host, n, m, iterations=args.cpu_iterations)

    result = {
        "metric": METRIC, "value": round(value, 3), "unit": "GTEPS", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"pagerank R-MAT scale {SCALE} edge factor {EDGE_FACTOR} seed {SEED}, "
                               f"{ITERATIONS} iterations, variant {variant}",
                   "vertices": n, "edges": m, "iterations": ITERATIONS, "variant": variant,
                   "l2": "inputs larger than L2 (graph %.0f MB > 129 MB)" % ((4 * (n + 1) + 4 * m) / 1e6),
                   "parallelism": f"replicas x{ws}"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None,
                     "kernel": "k_pr_pull_segmented", "kernel_ms": round(kernel_ms, 5),
                     "algorithmic_bytes": alg_bytes, "peak_source": peak_kind},
        "e2e": {"value": round(e2e_value, 3), "unit": "GTEPS",
                "h2d_bytes_per_step": int(rv.numel() * 4 + re.numel() * 4),
                "d2h_bytes_per_step": int(n * 4)},
        "gpu_launches": pagerank_launches(variant, ITERATIONS) * args.steps,
        "clocks": clocks.summary(),
    }
    if cpu is not None:
        result["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(result))
    if ws > 1:
        dist.destroy_process_group()


def cpu_baseline(host, n, m, iterations):
    import oracle
    threads = os.cpu_count() or 1
    deg = np.diff(host["fwd_vertices"].astype(np.int64)).astype(np.uint32)
    t = time.perf_counter()
    oracle.pagerank_parallel(n, host["rev_vertices"], host["rev_edges"], iterations, deg=deg, threads=threads)
    dt = time.perf_counter() - t
    return {"value": round(m * iterations / dt / 1e9, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"{iterations} of {ITERATIONS} iterations of the same R-MAT-{SCALE} PageRank "
                      f"(vertex-pull + consolidateRank restated, OpenMP), {dt:.2f} s"}


def run_reference(args):
    """CPU restatement of the reference path, timed on the host cores."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import belewitte_gb300 as bw
    import torch
    g = bw.DeviceGraph.generate("rmat", scale=SCALE, edge_factor=EDGE_FACTOR, seed=SEED,
                                reps=bw.REP_FWD_CSR | bw.REP_REV_CSR)
    host = g.to_host_arrays()
    n, m = g.vertex_count, g.edge_count
    del g
    torch.cuda.empty_cache()
    import oracle
    threads = os.cpu_count() or 1
    deg = np.diff(host["fwd_vertices"].astype(np.int64)).astype(np.uint32)
    per_step_iters = args.cpu_iterations
    for _ in range(args.warmup):
        oracle.pagerank_parallel(n, host["rev_vertices"], host["rev_edges"], 1, deg=deg, threads=threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        oracle.pagerank_parallel(n, host["rev_vertices"], host["rev_edges"], per_step_iters, deg=deg,
                                 threads=threads)
    dt = time.perf_counter() - t
    value = m * per_step_iters * args.steps / dt / 1e9
    sample = (f"{per_step_iters} PageRank iterations per step on the R-MAT-{SCALE} graph "
              f"(vertex-pull + consolidateRank restated, OpenMP)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "GTEPS", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"pagerank R-MAT scale {SCALE} edge factor {EDGE_FACTOR} seed {SEED}, "
                               f"{ITERATIONS} iterations", "vertices": n, "edges": m},
        "cpu_baseline": {"value": round(value, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--variant", default=HEADLINE_VARIANT)
    ap.add_argument("--cpu-iterations", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
