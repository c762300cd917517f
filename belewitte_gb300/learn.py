"""Learned variant switching: per BFS level and per PageRank iteration.
Data, training, evaluation.

Pipeline (all compute on the GPU through the C ABI):

1. ``catalogue(seed)`` lists seeded synthetic graphs: R-MAT with
   a in [0.45, 0.70] and scale 16-23, 2-D grids 512^2-4096^2, Erdos-Renyi
   with average degree 4-64, Barabasi-Albert with m in 2-32 (symmetric, so a
   BFS reaches the giant component).
2. ``profile_graph`` runs ``bw_bfs_profile``: every candidate variant timed
   on every level from the same saved state, plus the 12 level features.
3. ``build_dataset`` turns timings into soft targets
   q_k = softmax(-log2(t_k / t_min) / tau) and weights proportional to the
   level's cost, so near-equal variants are not penalised and expensive
   levels count more.
4. ``train`` normalises features, initialises and trains the MLP
   12 -> 64 -> 64 -> K with the device kernels (bw_mlp_train).
5. ``evaluate`` scores held-out graphs: the chosen sequence against the
   oracle-best per-level sequence (sum of per-level minima, the reference's
   StepAggregate definition) and the best fixed variant (minimum over
   variants of the summed levels, as in the reference's Evaluate).

The trained predictor ships as data/bfs_predictor.npz and is loaded by
``load_predictor``.

PageRank (``--algo pagerank``): ``profile_pagerank`` times every div-class
variant per iteration on the same graph specs, with R-MAT and ER left
directed, and with the 12 features of ``bw_pagerank_features`` (the whole
vertex set as the frontier; the level separates the first iteration from
the rest); the same dataset, training and scoring follow, and the
predictor ships as data/pagerank_predictor.npz (``load_pagerank_predictor``,
``run_pagerank_learned``).
"""
from __future__ import annotations

import ctypes as C
import json
import math
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _abi, bfs_variant_id, library
from ._abi import check

CANDIDATES = ["edge-list-bulk", "rev-edge-list-bulk", "struct-edge-list-bulk", "rev-struct-edge-list-bulk",
              "vertex-pull-bulk", "vertex-pull-warp-bulk", "frontier-push", "frontier-pull"]
PREDICTOR_PATH = Path(__file__).resolve().parent / "data" / "bfs_predictor.npz"
# PageRank: every reference variant of the div semantics class (a schedule
# cannot mix it with the nodiv variants, whose ranks differ by construction;
# pull-segmented runs vertex-pull's kernels)
PR_CANDIDATES = ["edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list", "vertex-push",
                 "vertex-pull", "vertex-push-warp", "vertex-pull-warp"]
PR_PREDICTOR_PATH = Path(__file__).resolve().parent / "data" / "pagerank_predictor.npz"
PR_PROFILE_ITERATIONS = 8      # timed per candidate: the first iteration, then the steady state
PR_RUN_ITERATIONS = 30         # the run a profile stands for
TAU = 0.15


# ---------------------------------------------------------------------------
# graphs
# ---------------------------------------------------------------------------
@dataclass
class GraphSpec:
    kind: str
    params: dict
    seed: int

    def name(self) -> str:
        p = ",".join(f"{k}={v}" for k, v in sorted(self.params.items()))
        return f"{self.kind}({p};seed={self.seed})"

    def build(self, device: int = 0, reps: int = 63, symmetrise: bool = True):
        """The graph; R-MAT and ER are symmetrised unless `symmetrise` is
        False (grids and BA are symmetric by construction)."""
        from . import DeviceGraph
        p = dict(self.params)
        if self.kind == "rmat":
            return DeviceGraph.generate("rmat", scale=p["scale"], edge_factor=p["edge_factor"], a=p["a"],
                                        b=p["b"], c=p["c"], seed=self.seed, symmetrise=symmetrise, device=device,
                                        reps=reps)
        if self.kind == "er":
            return DeviceGraph.generate("er", n=p["n"], m=p["m"], seed=self.seed, symmetrise=symmetrise,
                                        device=device, reps=reps)
        if self.kind == "grid":
            return DeviceGraph.generate("grid", h=p["side"], w=p["side"], device=device, reps=reps)
        return DeviceGraph.generate("ba", n=p["n"], m=p["m"], seed=self.seed, device=device, reps=reps)


def catalogue(count: int, seed: int, max_scale: int = 23, max_side: int = 4096) -> list[GraphSpec]:
    """`count` seeded graph specs mixed over the four families."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        fam = ["rmat", "grid", "er", "ba"][i % 4]
        s = int(rng.integers(1, 2 ** 31))
        if fam == "rmat":
            a = float(rng.uniform(0.45, 0.70))
            rest = 1.0 - a
            b = c = round(rest * 0.38, 4)
            lo = min(16, max_scale)
            out.append(GraphSpec("rmat", dict(scale=int(rng.integers(lo, max_scale + 1)), edge_factor=16,
                                              a=round(a, 4), b=b, c=c), s))
        elif fam == "grid":
            side = int(round(2 ** rng.uniform(math.log2(min(512, max_side)), math.log2(max_side))))
            out.append(GraphSpec("grid", dict(side=side), s))
        elif fam == "er":
            n = int(2 ** rng.uniform(min(16, max_scale), min(22, max_scale + 1)))
            deg = float(2 ** rng.uniform(2, 6))
            out.append(GraphSpec("er", dict(n=n, m=int(n * deg / 2)), s))
        else:
            n = int(2 ** rng.uniform(min(16, max_scale), min(22, max_scale + 1)))
            out.append(GraphSpec("ba", dict(n=n, m=int(2 ** rng.uniform(1, 5))), s))
    return out


def pick_root(g, seed: int) -> int:
    """A seeded random vertex with at least one edge."""
    deg = (g.fwd_vertices[1:] - g.fwd_vertices[:-1]).cpu().numpy()
    nz = np.flatnonzero(deg > 0)
    rng = np.random.default_rng(seed)
    return int(nz[rng.integers(0, len(nz))]) if len(nz) else 0


# ---------------------------------------------------------------------------
# profiling
# ---------------------------------------------------------------------------
def profile_graph(ctx, g, root: int, candidates=CANDIDATES, max_levels: int = 0, repeats: int = 1,
                  sample_every: int = 64, default: str = "frontier-push"):
    """(level_ms[L][K], features[L][12]) from bw_bfs_profile; rows of
    unsampled levels hold -1."""
    import torch
    lib = library()
    K = len(candidates)
    ids = (C.c_int32 * K)(*[bfs_variant_id(c) for c in candidates])
    cap = max_levels or (g.vertex_count + 1)
    cap = min(cap, 20000)
    times = np.zeros((cap, K), dtype=np.float32)
    feats = np.zeros((cap, 12), dtype=np.float32)
    levels = torch.empty(g.vertex_count, dtype=torch.int32, device=g.device)
    count = C.c_uint32()
    st = torch.cuda.current_stream(g.device)
    rc = lib.bw_bfs_profile(ctx.handle, C.byref(g.view), root, C.c_void_p(levels.data_ptr()), ids, K, cap, repeats,
                            sample_every, list(candidates).index(default),
                            times.ctypes.data_as(C.POINTER(C.c_float)), feats.ctypes.data_as(C.POINTER(C.c_float)),
                            C.byref(count), C.c_void_p(st.cuda_stream))
    check(rc, "bw_bfs_profile")
    L = count.value
    return times[:L], feats[:L], levels


def subsample_levels(times, feats, limit: int = 64):
    """Keep the sampled levels; long traversals (grids) contribute at most
    `limit` evenly spaced ones."""
    keep = times[:, 0] >= 0
    times, feats = times[keep], feats[keep]
    L = len(times)
    if L <= limit:
        return times, feats
    idx = np.unique(np.linspace(0, L - 1, limit).round().astype(int))
    return times[idx], feats[idx]


def build_dataset(records):
    """records: list of (times[L][K], feats[L][12]) -> X, T, W (float32)."""
    X, T, W = [], [], []
    for times, feats in records:
        t = np.maximum(times.astype(np.float64), 1e-4)
        tmin = t.min(axis=1, keepdims=True)
        logits = -np.log2(t / tmin) / TAU
        q = np.exp(logits - logits.max(axis=1, keepdims=True))
        q /= q.sum(axis=1, keepdims=True)
        X.append(feats)
        T.append(q)
        W.append(t.mean(axis=1))
    X = np.concatenate(X).astype(np.float32)
    T = np.concatenate(T).astype(np.float32)
    W = np.concatenate(W)
    W = np.clip(W / W.mean(), 0.05, 20.0).astype(np.float32)
    return X, T, W


# ---------------------------------------------------------------------------
# MLP
# ---------------------------------------------------------------------------
def param_count(K: int) -> int:
    return int(library().bw_mlp_param_count(K))


def init_params(K: int, mu, sd, seed: int = 1, device: int = 0):
    import torch
    p = torch.zeros(param_count(K), dtype=torch.float32, device=f"cuda:{device}")
    mu = np.ascontiguousarray(mu, np.float32)
    sd = np.ascontiguousarray(sd, np.float32)
    st = torch.cuda.current_stream(p.device)
    check(library().bw_mlp_init(C.c_void_p(p.data_ptr()), K, mu.ctypes.data_as(C.POINTER(C.c_float)),
                                sd.ctypes.data_as(C.POINTER(C.c_float)), seed, C.c_void_p(st.cuda_stream)),
          "bw_mlp_init")
    return p


def train(ctx, X, T, W, *, steps: int = 20000, batch: int = 64, lr: float = 3e-3, seed: int = 7,
          weight_decay: float = 1e-5, loss_points: int = 20, params=None):
    """Train on the device; returns (params tensor, loss curve)."""
    import torch
    dev = f"cuda:{ctx.device}"
    K = T.shape[1]
    if params is None:
        mu = X.mean(axis=0)
        sd = X.std(axis=0) + 1e-3
        params = init_params(K, mu, sd, seed=seed, device=ctx.device)
    dX = torch.from_numpy(np.ascontiguousarray(X)).to(dev)
    dT = torch.from_numpy(np.ascontiguousarray(T)).to(dev)
    dW = torch.from_numpy(np.ascontiguousarray(W)).to(dev)
    cfg = _abi.MlpTrainConfig(steps, batch, lr, 0.9, 0.999, 1e-8, weight_decay, 0, seed)
    curve = (C.c_float * loss_points)()
    st = torch.cuda.current_stream(dX.device)
    check(library().bw_mlp_train(ctx.handle, C.c_void_p(params.data_ptr()), K, C.c_void_p(dX.data_ptr()),
                                 C.c_void_p(dT.data_ptr()), C.c_void_p(dW.data_ptr()), len(X), C.byref(cfg),
                                 curve, loss_points, C.c_void_p(st.cuda_stream)), "bw_mlp_train")
    return params, list(curve)


def gradient(ctx, params, X, T, W=None):
    import torch
    dev = params.device
    K = T.shape[1]
    dX = torch.from_numpy(np.ascontiguousarray(X, np.float32)).to(dev)
    dT = torch.from_numpy(np.ascontiguousarray(T, np.float32)).to(dev)
    dW = None if W is None else torch.from_numpy(np.ascontiguousarray(W, np.float32)).to(dev)
    grad = torch.zeros_like(params)
    loss = C.c_float()
    st = torch.cuda.current_stream(dev)
    check(library().bw_mlp_gradient(ctx.handle, C.c_void_p(params.data_ptr()), K, C.c_void_p(dX.data_ptr()),
                                    C.c_void_p(dT.data_ptr()), C.c_void_p(0 if dW is None else dW.data_ptr()),
                                    len(X), C.c_void_p(grad.data_ptr()), C.byref(loss), C.c_void_p(st.cuda_stream)),
          "bw_mlp_gradient")
    return grad.cpu().numpy(), loss.value


def predict(ctx, params, X, K):
    import torch
    dev = params.device
    dX = torch.from_numpy(np.ascontiguousarray(X, np.float32)).to(dev)
    out = torch.empty((len(X), K), dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    check(library().bw_mlp_predict(ctx.handle, C.c_void_p(params.data_ptr()), K, C.c_void_p(dX.data_ptr()),
                                   len(X), C.c_void_p(out.data_ptr()), C.c_void_p(st.cuda_stream)), "bw_mlp_predict")
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


# ---------------------------------------------------------------------------
# PageRank: per-iteration timings and features
# ---------------------------------------------------------------------------
def pagerank_features(ctx, g, iteration: int):
    """The 12 features of PageRank iteration `iteration` (bw_pagerank_features)."""
    import torch
    out = (C.c_float * 12)()
    st = torch.cuda.current_stream(g.device)
    check(library().bw_pagerank_features(ctx.handle, C.byref(g.view), iteration, out, C.c_void_p(st.cuda_stream)),
          "bw_pagerank_features")
    return np.frombuffer(out, np.float32).copy()


def profile_pagerank(ctx, g, candidates=PR_CANDIDATES, iterations: int = PR_PROFILE_ITERATIONS,
                     run_iterations: int = PR_RUN_ITERATIONS):
    """(ms[2][K], features[2][12]) for a `run_iterations`-iteration run:
    row 0 the first iteration, row 1 the other run_iterations - 1 at the
    steady-state rate (median of the last half of `iterations` timed
    iterations: some variants settle after the first few, e.g.
    vertex-pull takes its hub-first order).  Every candidate runs alone
    after a warm-up run, timed per iteration with CUDA events
    (pagerank_schedule)."""
    from . import pagerank, pagerank_schedule
    times = np.zeros((2, len(candidates)), np.float32)
    for k, v in enumerate(candidates):
        # the library's default launch: what the learned run executes
        pagerank(ctx, g, v, 1, tuned=False)
        run = pagerank_schedule(ctx, g, [v], iterations, time_iterations=True, tuned=False)
        t = np.asarray(run.iteration_ms[:iterations], np.float64)
        times[0, k] = t[0]
        times[1, k] = np.median(t[iterations // 2:]) * (run_iterations - 1)
    feats = np.stack([pagerank_features(ctx, g, it) for it in (0, 1)])
    return times, feats


def collect_pagerank(ctx, specs, log=print):
    import torch
    records = []
    for i, spec in enumerate(specs):
        t0 = time.time()
        g = spec.build(device=ctx.device, symmetrise=False)    # PageRank runs on directed graphs
        records.append(profile_pagerank(ctx, g))
        log(f"[{i + 1}/{len(specs)}] {spec.name()} N={g.vertex_count} M={g.edge_count} ({time.time() - t0:.1f}s)")
        del g
        torch.cuda.empty_cache()
    return records


def run_pagerank_learned(ctx, g, predictor: "Predictor", iterations: int = 30, *, ranks=None, loop: str = "host"):
    """PageRank with the learned per-iteration choice
    (bw_pagerank_run_learned); returns (PageRankRun, schedule of names)."""
    import torch
    from . import PageRankRun, pagerank_variant_names
    if ranks is None:
        ranks = torch.empty(g.vertex_count, dtype=torch.float32, device=g.device)
    cfg = predictor.switch_config(pagerank=True)
    res = _abi.PagerankResult()
    diffs = (C.c_float * max(iterations, 1))()
    sched = (C.c_int32 * max(iterations, 1))()
    st = torch.cuda.current_stream(g.device)
    check(library().bw_pagerank_run_learned(ctx.handle, C.byref(g.view), C.byref(cfg), iterations,
                                            C.c_void_p(ranks.data_ptr()), 1 if loop == "graph" else 0, C.byref(res),
                                            diffs, sched, C.c_void_p(st.cuda_stream)), "bw_pagerank_run_learned")
    names = pagerank_variant_names()
    run = PageRankRun(ranks, res.iterations, res.device_ms, list(diffs)[:iterations],
                      kernel_launches=res.kernel_launches)
    return run, [names[v] for v in list(sched)[:iterations]]


# ---------------------------------------------------------------------------
# scoring
# ---------------------------------------------------------------------------
def choose(probs, fallback: int, threshold: float):
    best = probs.argmax(axis=1)
    conf = probs.max(axis=1)
    return np.where(conf < threshold, fallback, best)


def score_graph(times, chosen):
    """Times of the oracle-best sequence, every fixed variant and the choice."""
    oracle_best = float(times.min(axis=1).sum())
    fixed = times.sum(axis=0)
    return {"oracle_best": oracle_best, "best_fixed": float(fixed.min()), "best_fixed_k": int(fixed.argmin()),
            "chosen": float(times[np.arange(len(times)), chosen].sum()), "fixed": fixed.tolist()}


def fallback_variant(records):
    """The single variant with the lowest total time relative to each
    graph's oracle-best: the plain fixed-variant method."""
    K = records[0][0].shape[1]
    score = np.zeros(K)
    for times, _ in records:
        score += times.sum(axis=0) / max(times.min(axis=1).sum(), 1e-9)
    return int(score.argmin())


# ---------------------------------------------------------------------------
# predictor file
# ---------------------------------------------------------------------------
@dataclass
class Predictor:
    params: object          # torch tensor on the device
    candidates: list
    fallback: int
    threshold: float

    def switch_config(self, mlp_only: bool = False, pagerank: bool = False):
        """bw_switch_config; mlp_only sets BW_SWITCH_MLP_ONLY (the device
        loop then leaves cluster-sized frontiers to the MLP too); pagerank:
        the candidates are PageRank variant names."""
        from . import pagerank_variant_id
        vid = pagerank_variant_id if pagerank else bfs_variant_id
        ids = (C.c_int32 * len(self.candidates))(*[vid(c) for c in self.candidates])
        cfg = _abi.SwitchConfig(C.c_void_p(self.params.data_ptr()), len(self.candidates), self.fallback, ids,
                                self.threshold, 1 if mlp_only else 0)
        cfg._keep = ids
        return cfg


def save_predictor(path, params, candidates, fallback, threshold, meta=None):
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez(path, params=params.detach().cpu().numpy(), candidates=np.array(candidates),
             fallback=np.int64(fallback), threshold=np.float32(threshold), meta=json.dumps(meta or {}))


def load_pagerank_predictor(path=PR_PREDICTOR_PATH, device: int = 0) -> Predictor:
    return load_predictor(path, device)


def load_predictor(path=PREDICTOR_PATH, device: int = 0) -> Predictor:
    import torch
    d = np.load(path, allow_pickle=False)
    params = torch.from_numpy(d["params"].astype(np.float32)).to(f"cuda:{device}")
    return Predictor(params, [str(c) for c in d["candidates"]], int(d["fallback"]), float(d["threshold"]))


def run_learned(ctx, g, predictor: Predictor, root: int, *, loop: str = "graph", levels=None, stats: bool = True,
                max_levels: int = 0, mlp_only: bool = False):
    """BFS with the learned per-level switch (bw_bfs_run_learned)."""
    import torch
    from . import BfsRun, _stats_list
    if levels is None:
        levels = torch.empty(g.vertex_count, dtype=torch.int32, device=g.device)
    cfg = predictor.switch_config(mlp_only)
    res = _abi.BfsResult()
    cap = min(max_levels or g.vertex_count + 1, 1 << 16) if stats else 0
    arr = (_abi.BfsLevelStats * cap)() if cap else None
    st = torch.cuda.current_stream(g.device)
    rc = library().bw_bfs_run_learned(ctx.handle, C.byref(g.view), C.byref(cfg), root, C.c_void_p(levels.data_ptr()),
                                      1 if loop == "graph" else 0, max_levels, C.byref(res), arr, cap,
                                      C.c_void_p(st.cuda_stream))
    check(rc, "bw_bfs_run_learned")
    run = BfsRun(levels, res.level_count, res.visited, res.traversed_edges, res.device_ms)
    if arr is not None:
        run.level_stats = _stats_list(arr, min(res.level_count, cap))
    return run


# ---------------------------------------------------------------------------
# end-to-end training run (CLI)
# ---------------------------------------------------------------------------
def collect(ctx, specs, log=print, level_limit: int = 64):
    import torch
    records = []
    for i, spec in enumerate(specs):
        t0 = time.time()
        g = spec.build(device=ctx.device)
        root = pick_root(g, spec.seed)
        times, feats, _ = profile_graph(ctx, g, root)
        times, feats = subsample_levels(times, feats, level_limit)
        records.append((times, feats))
        log(f"[{i + 1}/{len(specs)}] {spec.name()} N={g.vertex_count} M={g.edge_count} levels={len(times)} "
            f"({time.time() - t0:.1f}s)")
        del g
        torch.cuda.empty_cache()
    return records


def main(argv=None):
    import argparse
    import torch
    from . import Context
    ap = argparse.ArgumentParser(description="train the BFS (per level) or PageRank (per iteration) variant predictor")
    ap.add_argument("--algo", choices=["bfs", "pagerank"], default="bfs")
    ap.add_argument("--train", type=int, default=240)
    ap.add_argument("--heldout", type=int, default=40)
    ap.add_argument("--max-scale", type=int, default=23)
    ap.add_argument("--max-side", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--threshold", type=float, default=0.35)
    ap.add_argument("--out", default="")
    ap.add_argument("--report", default="")
    args = ap.parse_args(argv)
    ctx = Context(0)
    pr = args.algo == "pagerank"
    cands = PR_CANDIDATES if pr else CANDIDATES
    out_path = args.out or str(PR_PREDICTOR_PATH if pr else PREDICTOR_PATH)
    gather = collect_pagerank if pr else collect
    train_specs = catalogue(args.train, seed=2024, max_scale=args.max_scale, max_side=args.max_side)
    held_specs = catalogue(args.heldout, seed=4048, max_scale=args.max_scale, max_side=args.max_side)
    t0 = time.time()
    recs = gather(ctx, train_specs)
    held = gather(ctx, held_specs)
    X, T, W = build_dataset(recs)
    params, curve = train(ctx, X, T, W, steps=args.steps)
    fb = fallback_variant(recs)
    K = len(cands)
    report = {"algo": args.algo, "candidates": cands, "fallback": cands[fb], "threshold": args.threshold,
              "train_samples": int(len(X)), "loss_curve": curve, "collect_s": time.time() - t0}
    for label, rs, specs in (("train", recs, train_specs), ("heldout", held, held_specs)):
        tot = {"oracle_best": 0.0, "best_fixed": 0.0, "chosen": 0.0, "fallback_only": 0.0}
        per = []
        for (times, feats), spec in zip(rs, specs):
            probs = predict(ctx, params, feats, K)
            ch = choose(probs, fb, args.threshold)
            sc = score_graph(times, ch)
            sc["fallback_only"] = float(times[:, fb].sum())
            for k in tot:
                tot[k] += sc[k]
            per.append({"graph": spec.name(), **{k: sc[k] for k in ("oracle_best", "best_fixed", "chosen",
                                                                     "fallback_only")}})
        report[label] = {"totals_ms": tot, "speedup_vs_best_fixed": tot["best_fixed"] / tot["chosen"],
                         "speedup_vs_fallback": tot["fallback_only"] / tot["chosen"],
                         "efficiency_vs_oracle_best": tot["oracle_best"] / tot["chosen"], "graphs": per}
    save_predictor(out_path, params, cands, fb, args.threshold,
                   meta={"algo": args.algo, "train_graphs": [s.name() for s in train_specs], "steps": args.steps})
    if args.report:
        Path(args.report).write_text(json.dumps(report, indent=1))
    print(json.dumps({k: report[k] for k in ("fallback", "train_samples")} |
                     {lab: {k: report[lab][k] for k in ("totals_ms", "speedup_vs_best_fixed",
                                                        "efficiency_vs_oracle_best")} for lab in ("train", "heldout")}))


if __name__ == "__main__":
    main()
