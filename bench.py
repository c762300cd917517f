"""Benchmark: GTEPS on one GB300 (PageRank per iteration; BFS learned switch).

Headline line (N=1): PageRank, FP32, damping 0.85, 1/N init, 30 fixed
iterations on a seeded R-MAT graph of scale 22 (4,194,304 vertices, edge
factor 16, a/b/c/d = 0.57/0.19/0.19/0.05, self-loops and duplicates removed),
the PageRank configuration the metric is quoted on.  A step is one full
30-iteration PageRank over the device-resident graph with vertex-pull, the
fastest variant whose ranks are bit-identical to the reference's
(`--variant` picks another); the ranks are checked against the oracle.
GTEPS = edges x iterations / time.

The same JSON line carries:
  * learned_switch: BFS on the symmetrised R-MAT scale-24 graph, the 4096 x
    4096 grid and BA(8M, 8), 16 seeded sources of the giant component each --
    the learned per-level switch (shipped predictor, device-side decisions in
    a CUDA graph) against every fixed candidate variant; every depth array is
    checked against the oracle; the learned runs' fraction of the top-down
    compulsory bytes.
  * learned_pagerank: the learned per-iteration PageRank choice (shipped
    predictor) against every fixed div-class variant, 30 iterations, on the
    headline R-MAT graph and a 4096 x 4096 grid.
  * batched: many graphs (BFS + 20-iteration PageRank each) and many BFS
    sources, each in one persistent launch.
  * parity: the headline ranks against the oracle (bit for bit) and FP64.
  * roofline of the PageRank iteration, e2e through the C ABI with host
    buffers, the CPU baselines (PageRank, and BFS on the R-MAT-24 sources),
    clocks during the timed region.
  * gather_roofline: the PageRank iteration's gathers per second against the
    device's ceiling for scattered 4-byte loads, measured in the same run by
    the library's probe kernel (M uniform random gathers over N).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --case pagerank:VARIANT:rmat22|er[:BLOCK:HUBS]   (small profiling case)
  python bench.py --case bfs:VARIANT:rmat22            (small profiling case)
  python bench.py --case bfsgraph:VARIANT:grid          (device loop; the cluster kernel)
  python bench.py --case batch:graphs:COUNT             (the first COUNT batched graphs; k_batch)
  python bench.py --sweep      (every PageRank variant on R-MAT-22 and ER, every BFS variant
                                on R-MAT-24 sym, the grid and BA)

N > 1 (torch.distributed.run): the path does not shard one graph, so each
rank runs an independent replica (weak scaling).  --impl reference times the
CPU restatement of the reference's PageRank (vertex-pull + consolidateRank,
OpenMP on all host cores) on the same graph, made by the oracle's own
generator (the product library is not loaded).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import threading
import time

import numpy as np

METRIC = "GTEPS (BFS, PageRank/iter) on 1 GB300: learned-switched vs best fixed variant"
SCALE, EDGE_FACTOR, SEED, ITERATIONS = 22, 16, 22, 30
BFS_SCALE, BFS_SEED, BFS_SOURCES = 24, 24, 16


def _dist():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(value: float, ws: int, device="cpu") -> float:
    """The slowest rank's value (timings are reported as the max over ranks)."""
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ws: int, edges: int, iterations: int, seconds: float) -> float:
    """Whole-job GTEPS of `ws` independent replicas that each ran
    `iterations` PageRank iterations over `edges` edges in `seconds`."""
    return ws * edges * iterations / seconds / 1e9


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.proc, self.lines, self._t = gpu, None, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=lambda: [self.lines.append(x.strip()) for x in self.proc.stdout],
                                       daemon=True)
            self._t.start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

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
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def _profiled_traffic(variant: str):
    """DRAM bytes of one iteration of the variant on this workload (its
    kernels' dram__bytes_read + write), from the committed ncu summary
    (None when there is none)."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                        f"pagerank_{variant.replace('-', '_')}_rmat{SCALE}.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith(("traffic_bytes_per_iteration:", "traffic_bytes_per_launch:")):
                    return int(line.split(":")[1])
    except OSError:
        pass
    return None


def _measured_peak():
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# The PageRank variant the headline is measured with: the reference's own
# vertex-pull, whose ranks are bit-identical to the reference's (the
# work-list kernel and the long-row sequential sums; the fastest variant
# that meets the bar); --variant measures another one.
HEADLINE_VARIANT = "vertex-pull"

DOMINANT = {"pull-segmented": "k_pr_pull_items + k_pr_long_sums", "vertex-pull": "k_pr_pull_items + k_pr_long_sums",
            "vertex-pull-nodiv": "k_pr_pull_items + k_pr_long_sums",
            "vertex-pull-warp": "k_pr_vertex_pull_warp", "vertex-pull-warp-nodiv": "k_pr_vertex_pull_warp",
            "vertex-push": "k_pr_vertex_push", "vertex-push-warp": "k_pr_vertex_push_warp"}


def alg_bytes(variant: str, n: int, m: int, n_in: int) -> int:
    """Compulsory bytes of one steady-state PageRank iteration of the
    reference algorithm.  Pull variants: the 4M source indices, the offsets
    4(N+1), one read of the gathered vector (4N), and for each of the n_in
    rows with in-edges its degree, its previous rank (for the diff), its new
    rank and its contribution (16 bytes); the rows without in-edges keep
    rank and contribution from the second iteration on and are not touched.
    Edge-list variants: the 8M edge pairs plus 16N."""
    if variant.startswith(("edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list")):
        return 8 * m + 16 * n
    return 4 * m + 4 * (n + 1) + 4 * n + 16 * n_in


BFS_GRAPHS = (
    (f"BFS R-MAT scale {BFS_SCALE} symmetrised (seed {BFS_SEED})", "rmat",
     dict(scale=BFS_SCALE, edge_factor=EDGE_FACTOR, seed=BFS_SEED, symmetrise=True)),
    ("BFS grid 4096 x 4096", "grid", dict(h=4096, w=4096)),
    ("BFS BA n=8388608 m=8 (seed 8)", "ba", dict(n=8388608, m=8, seed=8)),
)


def bfs_compulsory_bytes(n: int, m: int) -> int:
    """Top-down compulsory bytes of one traversal: offsets, adjacency, depth
    initialisation and final write."""
    return 4 * (n + 1) + 4 * m + 8 * n


def bfs_learned_vs_fixed(ctx, dev, label, kind, kw, peak, cpu_seconds=0.0):
    """The learned per-level switch against every fixed candidate variant
    from BFS_SOURCES seeded sources of the giant component; every depth
    array is checked against the oracle's BFS on the host (the OpenMP
    restatement of the reference's CPU BFS, evolve/Connectivity.cpp:29-77,
    on the R-MAT graph -- timed, it is the BFS CPU baseline -- and the
    sequential queue BFS on the grid, whose 8190 levels the level-synchronous
    scan of every vertex makes impractical).  With cpu_seconds > 0 the
    baseline is a bounded sample: sources are timed until that much CPU time
    is spent; the rest are checked with the queue BFS."""
    import torch

    import belewitte_gb300 as bw
    import oracle
    from belewitte_gb300 import learn
    g = bw.DeviceGraph.generate(kind, device=dev, reps=63, **kw)
    n, m = g.vertex_count, g.edge_count
    pred = learn.load_predictor(device=dev)
    deg = g.fwd_vertices[1:] - g.fwd_vertices[:-1]
    hub = int(torch.argmax(deg).item())
    reach = torch.nonzero(bw.bfs(ctx, g, "frontier-pull", hub).levels != bw.INF).flatten().cpu().numpy()
    sources = [int(x) for x in np.random.default_rng(BFS_SEED).choice(reach, BFS_SOURCES, replace=False)]
    fixed = ["edge-list-bulk", "struct-edge-list-bulk", "frontier-push", "frontier-pull", "vertex-pull-warp-bulk"]
    if kind == "grid":
        fixed = ["frontier-push", "frontier-pull"]     # the rest do O(N) or O(M) work on each of ~8190 levels
    times = {k: 0.0 for k in ["learned"] + fixed}
    edges, depths = 0, []
    for r in sources:
        learn.run_learned(ctx, g, pred, r, loop="graph", stats=False)          # warm-up of this source
        run = learn.run_learned(ctx, g, pred, r, loop="graph", stats=False)
        times["learned"] += run.device_ms
        edges += run.traversed_edges
        for v in fixed:
            rr = bw.bfs(ctx, g, v, r, loop="graph")
            if not torch.equal(rr.levels, run.levels):
                raise AssertionError(f"BFS depths of {v} differ from the learned run")
            times[v] += rr.device_ms
        depths.append(run.levels.cpu().numpy())
    host = g.to_host_arrays()
    del g, deg
    torch.cuda.empty_cache()
    # the oracle on the host cores: every source's depths, bit for bit
    threads = os.cpu_count() or 1
    cpu_edges, cpu_s, timed = 0, 0.0, 0
    hdeg = np.diff(host["fwd_vertices"].astype(np.int64))
    for r, got in zip(sources, depths):
        if kind != "grid" and (cpu_seconds <= 0 or cpu_s < cpu_seconds):
            t = time.perf_counter()
            want, _ = oracle.bfs_parallel(n, host["fwd_vertices"], host["fwd_edges"], r, threads=threads)
            cpu_s += time.perf_counter() - t
            timed += 1
            cpu_edges += int(hdeg[want != oracle.INF].sum())
        else:
            want, _ = oracle.bfs(n, host["fwd_vertices"], host["fwd_edges"], r)
        if not np.array_equal(got, want):
            raise AssertionError(f"learned BFS depths from source {r} differ from the oracle")
    best = min(fixed, key=lambda v: times[v])
    ab = bfs_compulsory_bytes(n, m) * len(sources)
    achieved = ab / (times["learned"] * 1e-3) / 1e9
    out = {"workload": f"{label}, {BFS_SOURCES} seeded sources of the giant component",
           "vertices": n, "edges": m, "sources": len(sources),
           "learned_gteps": round(edges / (times["learned"] * 1e-3) / 1e9, 2),
           "best_fixed_variant": best, "best_fixed_gteps": round(edges / (times[best] * 1e-3) / 1e9, 2),
           "speedup_vs_best_fixed": round(times[best] / times["learned"], 3),
           "ms_total": {k: round(v, 3) for k, v in times.items()},
           "depths_vs_oracle": "identical (every source)",
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4),
                        "bytes": "top-down compulsory 4(N+1) + 4M + 8N per traversal; direction-optimising "
                                 "levels read less, so the fraction can exceed 1"}}
    cpu = None
    if timed:
        cpu = {"value": round(cpu_edges / cpu_s / 1e9, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
               "sample": f"{timed} of the {len(sources)} sources on this graph, {cpu_s:.1f} s "
                         "(level-synchronous atomic-min BFS of evolve/Connectivity.cpp:29-77 restated in C, OpenMP)"}
    return out, cpu


def pagerank_learned_vs_fixed(ctx, dev):
    """The learned per-iteration PageRank choice against every fixed
    div-class variant, 30 iterations each, device-timed (CUDA events around
    the run), on the headline R-MAT graph and a 4096 x 4096 grid."""
    import torch

    import belewitte_gb300 as bw
    from belewitte_gb300 import learn
    pred = learn.load_pagerank_predictor(device=dev)
    out = {}
    for label, kind, kw in ((f"R-MAT scale {SCALE} edge factor {EDGE_FACTOR} seed {SEED}", "rmat",
                             dict(scale=SCALE, edge_factor=EDGE_FACTOR, seed=SEED)),
                            ("grid 4096 x 4096", "grid", dict(h=4096, w=4096))):
        g = bw.DeviceGraph.generate(kind, device=dev, reps=63, **kw)
        ranks = torch.empty(g.vertex_count, dtype=torch.float32, device=f"cuda:{dev}")
        times = {}
        for v in learn.PR_CANDIDATES:
            bw.pagerank(ctx, g, v, 2, ranks=ranks)
            times[v] = bw.pagerank(ctx, g, v, ITERATIONS, ranks=ranks).device_ms
        learn.run_pagerank_learned(ctx, g, pred, 2, ranks=ranks)
        run, sched = learn.run_pagerank_learned(ctx, g, pred, ITERATIONS, ranks=ranks)
        best = min(times, key=times.get)
        out[label] = {"learned_ms": round(run.device_ms, 3), "learned_schedule": sorted(set(sched)),
                      "best_fixed_variant": best, "best_fixed_ms": round(times[best], 3),
                      "speedup_vs_best_fixed": round(times[best] / run.device_ms, 3),
                      "ms_fixed": {k: round(v, 3) for k, v in times.items()}}
        del g, ranks
        torch.cuda.empty_cache()
    return out


def batched(ctx, dev, graphs: int):
    import torch

    import belewitte_gb300 as bw
    from belewitte_gb300 import batch
    out = {}
    t0 = time.time()
    specs = batch.workload_a_specs(graphs, seed=5)
    gs = [bw.DeviceGraph.generate("rmat_n", n=s["n"], edge_factor=s["edge_factor"], seed=s["seed"],
                                  device=dev) for s in specs]
    packed = batch.pack(gs, device=dev)
    del gs
    gen_s = time.time() - t0
    batch.run_graphs(ctx, packed, pr_iterations=20)                     # warm-up
    _, _, res = batch.run_graphs(ctx, packed, pr_iterations=20)
    out["graphs"] = {"workload": f"{graphs} R-MAT graphs, vertex counts log-uniform in 1,000..200,000, "
                                 "edge factor 8-32; "
                                 "BFS from each max-degree vertex + 20 PageRank iterations, one persistent launch",
                     "vertices": packed.vertex_count, "edges": packed.edge_count, "ms": round(res.device_ms, 3),
                     "gteps": round((res.traversed_edges + 20 * packed.edge_count) / (res.device_ms * 1e-3) / 1e9, 2),
                     "generation_s": round(gen_s, 1)}
    del packed
    torch.cuda.empty_cache()
    g = bw.DeviceGraph.generate("rmat", scale=20, edge_factor=16, seed=20, symmetrise=True, device=dev)
    reach = torch.nonzero(bw.bfs(ctx, g, "frontier-pull", 0).levels != bw.INF).flatten().cpu().numpy()
    srcs = np.random.default_rng(20).choice(reach, 1024, replace=False)
    batch.run_sources(ctx, g, srcs[:64])
    levels, res = batch.run_sources(ctx, g, srcs)
    out["sources"] = {"workload": "1024 BFS sources on R-MAT scale 20 (symmetrised), one persistent launch",
                      "ms": round(res.device_ms, 3), "gteps": round(res.traversed_edges / (res.device_ms * 1e-3) / 1e9, 2)}
    del levels, g
    torch.cuda.empty_cache()
    return out


class HostToDevice:
    """The e2e leg: a caller holding the CSR in pinned host memory copies it
    to preallocated device buffers every step and derives the edge-list /
    struct-edge-list arrays the variant reads on the device (as
    DeviceGraph does), then calls bw_pagerank_run through the C ABI.  Pull
    variants get the reverse CSR plus the forward offsets (for the
    out-degrees)."""

    def __init__(self, host, variant, n, m, dev):
        import torch
        fwd = variant in ("vertex-push", "vertex-push-warp") or variant.startswith(("edge-list", "struct-edge-list"))
        side = "fwd" if fwd else "rev"
        self.side, self.n, self.m = side, n, m
        self.el = variant.startswith(("edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list"))
        self.st = "struct" in variant
        self.host = {k: torch.from_numpy(host[f"{side}_{k}"].view(np.int32)).pin_memory()
                     for k in ("vertices", "edges")}
        if side == "rev":
            # the forward offsets as well (4(N+1) bytes): the out-degrees are
            # then their row lengths, one pass over N, instead of a histogram
            # over the M source ids of the reverse CSR
            self.host["out_offsets"] = torch.from_numpy(host["fwd_vertices"].view(np.int32)).pin_memory()
        self.dev = {k: torch.empty_like(v, device=f"cuda:{dev}") for k, v in self.host.items()}
        self.in_edges = torch.empty(max(m, 1), dtype=torch.int32, device=f"cuda:{dev}") if self.el else None
        self.struct = torch.empty(2 * max(m, 1), dtype=torch.int32, device=f"cuda:{dev}") if self.st else None
        self.h2d_bytes = int(sum(v.numel() * 4 for v in self.host.values()))

    def upload(self, stream):
        from belewitte_gb300 import _abi
        import belewitte_gb300 as bw
        lib, sp = bw.library(), C.c_void_p(stream.cuda_stream)
        for k in self.host:
            self.dev[k].copy_(self.host[k], non_blocking=True)
        off, adj = self.dev["vertices"].data_ptr(), self.dev["edges"].data_ptr()
        inn = st = 0
        if self.el:
            inn = self.in_edges.data_ptr()
            bw.check(lib.bw_expand_edge_list(C.c_void_p(off), self.n, self.m, C.c_void_p(inn), sp), "expand")
        if self.st:
            st = self.struct.data_ptr()
            bw.check(lib.bw_build_struct_edges(C.c_void_p(inn), C.c_void_p(adj), self.m, C.c_void_p(st), sp),
                     "struct")
        if self.side == "fwd":
            v = _abi.GraphView(self.n, self.m, off, adj, 0, 0, inn, 0, st, 0)
        else:
            v = _abi.GraphView(self.n, self.m, self.dev["out_offsets"].data_ptr(), 0, off, adj, 0, inn, 0, st)

        class _View:
            vertex_count, edge_count, view = self.n, self.m, v
        return _View()


def headline_config(n: int, m: int, ws: int) -> dict:
    """The workload both arms measure (the same dict in both JSON lines)."""
    return {"workload": f"pagerank R-MAT scale {SCALE} edge factor {EDGE_FACTOR} seed {SEED}, {ITERATIONS} iterations",
            "vertices": n, "edges": m, "iterations": ITERATIONS,
            "l2": "inputs larger than L2 (graph %.0f MB > 129 MB)" % ((4 * (n + 1) + 4 * m) / 1e6),
            "parallelism": f"independent replicas x{ws}"}


def headline_parity(host, n, ranks_dev) -> dict:
    """The headline run's ranks against the oracle: bit for bit against the
    OpenMP restatement of the reference's vertex-pull (the order the
    reference sums in), and the max relative error against the FP64 oracle
    (the bar: 1e-4)."""
    import oracle
    deg = np.diff(host["fwd_vertices"].astype(np.int64)).astype(np.uint32)
    got = ranks_dev.cpu().numpy()
    want = oracle.pagerank_parallel(n, host["rev_vertices"], host["rev_edges"], ITERATIONS, deg=deg)
    r64 = oracle.pagerank_f64(oracle.PR_DIV, n, host["rev_vertices"], host["rev_edges"], ITERATIONS, deg=deg)
    rel_ref = float((np.abs(got.astype(np.float64) - want) / np.abs(want.astype(np.float64))).max())
    rel64 = float((np.abs(got.astype(np.float64) - r64) / np.abs(r64)).max())
    out = {"bit_identical_to_reference_order": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32))),
           "max_rel_err_vs_reference": rel_ref, "max_rel_err_vs_fp64": rel64,
           "oracle": "oracle.pagerank_parallel (vertex-pull + consolidateRank restated in C) and the FP64 oracle"}
    if not out["bit_identical_to_reference_order"] and rel_ref > 1e-5:
        raise AssertionError(f"headline ranks {rel_ref:.3g} from the reference's order")
    if rel64 > 1e-4:
        raise AssertionError(f"headline ranks {rel64:.3g} from FP64")
    return out


def cpu_baseline(host, n, m, seconds: float = 10.0):
    """The oracle's OpenMP PageRank (the reference's vertex-pull arithmetic)
    on all host cores: whole 30-iteration runs, repeated for ~`seconds`."""
    import oracle
    threads = os.cpu_count() or 1
    deg = np.diff(host["fwd_vertices"].astype(np.int64)).astype(np.uint32)
    runs, t0 = 0, time.perf_counter()
    while True:
        oracle.pagerank_parallel(n, host["rev_vertices"], host["rev_edges"], ITERATIONS, deg=deg, threads=threads)
        runs += 1
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    return {"value": round(m * ITERATIONS * runs / dt / 1e9, 4), "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"{runs} full {ITERATIONS}-iteration PageRanks of the same R-MAT-{SCALE} graph "
                      f"(vertex-pull + consolidateRank restated in C, OpenMP), {dt:.1f} s"}


def run_ours(args):
    import torch
    import torch.distributed as dist

    import belewitte_gb300 as bw
    from belewitte_gb300 import _abi

    ws, rank, local = _dist()
    if ws > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    dev = local
    torch.cuda.set_device(dev)
    ctx = bw.Context(dev)
    stream = torch.cuda.current_stream()
    g = bw.DeviceGraph.generate("rmat", scale=SCALE, edge_factor=EDGE_FACTOR, seed=SEED, device=dev, reps=63)
    n, m = g.vertex_count, g.edge_count
    variant = args.variant or HEADLINE_VARIANT
    ranks = torch.empty(n, dtype=torch.float32, device=f"cuda:{dev}")

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
        launches = 0
        for _ in range(args.steps):
            run = bw.pagerank_schedule(ctx, g, [variant], ITERATIONS, ranks=ranks, time_iterations=True)
            iter_ms.extend(run.iteration_ms)
            launches += run.kernel_launches
        t1.record(stream)
        torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    ms = max_over_ranks(t0.elapsed_time(t1), ws, device=f"cuda:{dev}")
    ms_per_step = ms / args.steps
    value = replica_throughput(ws, m, ITERATIONS, ms_per_step * 1e-3)

    kernel_ms = float(np.median(iter_ms))
    n_in = int((g.rev_vertices[1:] != g.rev_vertices[:-1]).sum().item())   # rows with in-edges
    ab = alg_bytes(variant, n, m, n_in)
    peak, peak_kind = _measured_peak()
    achieved = ab / (kernel_ms * 1e-3) / 1e9
    # The gathered vector (4N bytes) fits in L2: the pull kernels are bound
    # by scattered 4-byte loads, not by HBM.  Their ceiling on this device:
    # M uniform random gathers over N entries by the probe kernel.
    gen = torch.Generator(device=f"cuda:{dev}")
    gen.manual_seed(SEED)
    probe_idx = torch.randint(0, n, (m,), dtype=torch.int32, device=f"cuda:{dev}", generator=gen)
    probe_src = torch.rand(n, dtype=torch.float32, device=f"cuda:{dev}", generator=gen)
    ceiling = bw.gather_ceiling(ctx, probe_src, probe_idx)
    del probe_idx, probe_src
    gathers = m / (kernel_ms * 1e-3)

    # ---- end to end through the C ABI with host buffers ----------------------
    host = g.to_host_arrays()
    parity = headline_parity(host, n, ranks) if rank == 0 else None
    e2e = HostToDevice(host, variant, n, m, dev)
    out_host = torch.empty(n, dtype=torch.float32).pin_memory()
    e2e_times = []
    for i in range(args.warmup + args.steps):
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()
        t = time.perf_counter()
        view = e2e.upload(stream)
        bw.pagerank(ctx, view, variant, ITERATIONS, ranks=ranks)
        out_host.copy_(ranks, non_blocking=True)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t)
    e2e_s = max_over_ranks(float(np.mean(e2e_times)), ws, device=f"cuda:{dev}")
    e2e_value = replica_throughput(ws, m, ITERATIONS, e2e_s)
    h2d = e2e.h2d_bytes
    del g, e2e
    torch.cuda.empty_cache()

    extras = {}
    cpu_bfs = None
    if not args.no_bfs:
        sw = {}
        for label, kind, kw in BFS_GRAPHS:
            want_cpu = kind == "rmat" and rank == 0 and ws == 1 and not args.no_cpu
            sw[label], c = bfs_learned_vs_fixed(ctx, dev, label, kind, kw, peak, cpu_seconds=20.0 if want_cpu else 0.0)
            cpu_bfs = cpu_bfs or c
        extras["learned_switch"] = sw
        extras["learned_pagerank"] = pagerank_learned_vs_fixed(ctx, dev)
    if not args.no_batched:
        extras["batched"] = batched(ctx, dev, args.batch_graphs)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(host, n, m)
        if cpu_bfs:
            cpu["bfs"] = cpu_bfs

    result = {
        "metric": METRIC, "value": round(value, 3), "unit": "GTEPS", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(n, m, ws),
        "variant": variant,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": _profiled_traffic(variant),
                     "kernel": DOMINANT.get(variant, "k_pr_edge"), "kernel_ms": round(kernel_ms, 5),
                     "algorithmic_bytes": ab, "rows_with_in_edges": n_in, "peak_source": peak_kind},
        "gather_roofline": {"bound": "scattered 4-byte loads", "achieved": round(gathers / 1e9, 1),
                            "peak": round(ceiling / 1e9, 1), "unit": "Ggathers/s",
                            "frac": round(gathers / ceiling, 4),
                            "peak_source": "bw_gather_probe: M uniform random gathers over N, measured in this run"},
        "e2e": {"value": round(e2e_value, 3), "unit": "GTEPS", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(n * 4)},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if parity is not None:
        result["parity"] = parity
    result.update(extras)
    if cpu is not None:
        result["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(result))
    if ws > 1:
        dist.destroy_process_group()


def run_reference(args):
    """The reference path's CPU implementation timed on the host cores: the
    OpenMP restatement of the reference's vertex-pull + consolidateRank
    (the reference itself has no CPU PageRank; its host glue does not build
    with CUDA 13), on the same R-MAT graph, made by the oracle's own
    generator -- nothing of the product library is loaded.  Each step is one
    full 30-iteration PageRank; rank 0 alone runs under torchrun."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import oracle
    t = time.perf_counter()
    host = oracle.generate_rmat(SCALE, EDGE_FACTOR, seed=SEED)
    gen_s = time.perf_counter() - t
    n, m = len(host["fwd_vertices"]) - 1, len(host["fwd_edges"])
    threads = os.cpu_count() or 1
    deg = np.diff(host["fwd_vertices"].astype(np.int64)).astype(np.uint32)
    for _ in range(args.warmup):
        oracle.pagerank_parallel(n, host["rev_vertices"], host["rev_edges"], ITERATIONS, deg=deg, threads=threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        oracle.pagerank_parallel(n, host["rev_vertices"], host["rev_edges"], ITERATIONS, deg=deg, threads=threads)
    dt = time.perf_counter() - t
    value = m * ITERATIONS * args.steps / dt / 1e9
    sample = (f"{args.steps} full {ITERATIONS}-iteration PageRanks of the R-MAT-{SCALE} graph "
              f"(vertex-pull + consolidateRank restated in C, OpenMP on {threads} threads; "
              f"graph made by the oracle's generator in {gen_s:.1f} s)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "GTEPS", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(n, m, ws),
        "cpu_baseline": {"value": round(value, 4), "unit": "GTEPS", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_case(spec: str):
    """Small, self-contained runs for profiler captures."""
    import torch

    import belewitte_gb300 as bw
    algo, variant, graph, *shape = spec.split(":")
    block, hubs = (int(shape[0]), int(shape[1])) if len(shape) == 2 else (0, 0)
    ctx = bw.Context(0)
    if algo == "batch":
        # batch:graphs:COUNT -- the first COUNT graphs of the batched
        # workload (BFS + 20 PageRank iterations each), one warm-up launch,
        # then the profiled one
        from belewitte_gb300 import batch
        specs = batch.workload_a_specs(4096, seed=5)[:int(graph)]
        gs = [bw.DeviceGraph.generate("rmat_n", n=s["n"], edge_factor=s["edge_factor"], seed=s["seed"])
              for s in specs]
        packed = batch.pack(gs)
        del gs
        for _ in range(2):
            _, _, res = batch.run_graphs(ctx, packed, pr_iterations=20)
        torch.cuda.synchronize()
        print("case done", spec, f"{res.device_ms:.3f} ms, {packed.vertex_count} vertices, {packed.edge_count} edges")
        return
    if graph == "er":
        g = bw.DeviceGraph.generate("er", n=4194304, m=67108864, seed=23, reps=63)
    elif graph == "rmat24s":
        g = bw.DeviceGraph.generate("rmat", scale=24, edge_factor=16, seed=24, symmetrise=True, reps=63)
    elif graph == "rmat22s":
        g = bw.DeviceGraph.generate("rmat", scale=22, edge_factor=16, seed=22, symmetrise=True, reps=63)
    elif graph == "grid":
        g = bw.DeviceGraph.generate("grid", h=4096, w=4096, reps=63)
    else:
        g = bw.DeviceGraph.generate("rmat", scale=22, edge_factor=16, seed=22, reps=63)
    if algo == "pagerank":
        # 5 iterations: enough for the run to take the hub-first order, as
        # the 30-iteration workload does
        bw.pagerank(ctx, g, variant, 5, block=block, chunk=hubs)
    elif algo == "learned":
        # host loop: a profiler sees each level's kernels (graph bodies it does not)
        from belewitte_gb300 import learn
        root = int(torch.argmax(g.fwd_vertices[1:] - g.fwd_vertices[:-1]).item())
        learn.run_learned(ctx, g, learn.load_predictor(), root, loop="host", stats=False)
    elif algo == "bfsgraph":
        # device loop: small frontiers run in frontier-push's cluster kernel
        bw.bfs(ctx, g, variant, int(torch.argmax(g.fwd_vertices[1:] - g.fwd_vertices[:-1]).item()), loop="graph")
    else:
        bw.bfs(ctx, g, variant, int(torch.argmax(g.fwd_vertices[1:] - g.fwd_vertices[:-1]).item()), loop="host")
    torch.cuda.synchronize()
    print("case done", spec)


def sweep():
    """Every PageRank variant, 30 iterations, on R-MAT scale 22 and ER(4M, 67M):
    the per-iteration median (CUDA events per iteration) as one JSON line
    per graph; then every BFS variant and the learned switch on the
    symmetrised R-MAT-24, the 4096 x 4096 grid and BA(8M, 8), one
    traversal each from the highest-degree vertex."""
    import torch

    import belewitte_gb300 as bw
    ctx = bw.Context(0)
    for label, kind, kw in (("R-MAT scale 22 edge factor 16 seed 22", "rmat", dict(scale=22, edge_factor=16, seed=22)),
                            ("ER n=4194304 m=67108864 seed 23", "er", dict(n=4194304, m=67108864, seed=23))):
        g = bw.DeviceGraph.generate(kind, reps=63, **kw)
        out = {}
        for v in bw.pagerank_variant_names():
            bw.pagerank(ctx, g, v, 3)
            run = bw.pagerank_schedule(ctx, g, [v], ITERATIONS, time_iterations=True)
            out[v] = round(float(np.median(run.iteration_ms)) * 1e3, 1)
        print(json.dumps({"graph": label, "vertices": g.vertex_count, "edges": g.edge_count,
                          "us_per_iteration": out}), flush=True)
        del g
        torch.cuda.empty_cache()
    # BFS: every variant from the highest-degree vertex (device loop), and
    # the learned switch; depths checked identical to frontier-push
    from belewitte_gb300 import learn
    pred = learn.load_predictor()
    for label, kind, kw in (("R-MAT scale 24 symmetrised seed 24", "rmat",
                             dict(scale=24, edge_factor=16, seed=24, symmetrise=True)),
                            ("grid 4096 x 4096", "grid", dict(h=4096, w=4096)),
                            ("BA n=8388608 m=8 seed 8", "ba", dict(n=8388608, m=8, seed=8))):
        g = bw.DeviceGraph.generate(kind, reps=63, **kw)
        root = int(torch.argmax(g.fwd_vertices[1:] - g.fwd_vertices[:-1]).item())
        want = bw.bfs(ctx, g, "frontier-push", root, loop="graph")
        ms, skipped = {}, []
        for v in bw.bfs_variant_names() + ["learned"]:
            if kind == "grid" and not v.startswith("frontier") and v != "learned":
                skipped.append(v)                   # O(N) or O(M) work per level x 8190 levels
                continue
            if v == "learned":
                learn.run_learned(ctx, g, pred, root, loop="graph", stats=False)
                run = learn.run_learned(ctx, g, pred, root, loop="graph", stats=False)
            else:
                bw.bfs(ctx, g, v, root, loop="graph")
                run = bw.bfs(ctx, g, v, root, loop="graph")
            if not torch.equal(run.levels, want.levels):
                raise AssertionError(f"BFS depths of {v} differ")
            ms[v] = round(run.device_ms, 3)
        print(json.dumps({"graph": label, "vertices": g.vertex_count, "edges": g.edge_count, "root": root,
                          "levels": want.level_count, "traversed_edges": want.traversed_edges,
                          "ms_per_bfs": ms, "not_run": skipped}), flush=True)
        del g, want
        torch.cuda.empty_cache()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--variant", default="")
    ap.add_argument("--batch-graphs", type=int, default=4096)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-bfs", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--case", default="")
    ap.add_argument("--sweep", action="store_true")
    args = ap.parse_args()
    if args.sweep:
        sweep()
        return
    if args.case:
        run_case(args.case)
        return
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
