"""Launch-geometry and push/pull-threshold autotuner for the BFS and
PageRank variants and the batched launch.

The reference fixes its geometry with Backend::computeDivision
(Backend.cpp:52-70) and takes the virtual-warp width and chunk of the warp
variants from -w/-c (ImplementationTemplate.hpp:431-436, defaults 32/32).
This tuner times each variant on a graph over a small grid of choices --
block size, grid size as a multiple of the SM count, and (warp variants)
virtual-warp width and chunk -- on the device, and keeps the fastest per
(algorithm, variant, graph shape class) in a JSON cache.  Results are
identical for every configuration (BFS depths bit-exact, PageRank within
the variant's tolerance), so tuning changes time only.

The batched launch (bw_batch_run) switches each BFS level between
top-down and bottom-up by a divisor: bottom-up once the frontier holds more
than 1/divisor of the unit's vertices.  ``tune_batch`` times the batched
BFS over a range of divisors and keeps the fastest per mode and graph shape
class; ``lookup_batch`` is what batch.run_graphs / run_sources use.
"""
from __future__ import annotations

import itertools
import json
import math
from pathlib import Path

import numpy as np

from . import bfs, bfs_variant_names, pagerank, pagerank_variant_names

CACHE = Path(__file__).resolve().parent / "data" / "autotune.json"

BLOCKS = {"edge": [128, 256, 512], "vertex": [128, 256, 512], "warp": [128, 256, 512], "fixed": [256]}
GRID_MULT = [2, 4, 8, 16]
WARP = [(4, 32), (8, 64), (16, 64), (32, 32), (32, 128)]


def shape_class(g) -> str:
    """Coarse graph class: log2 vertices, log2 average degree, skew."""
    deg = (g.fwd_vertices[1:] - g.fwd_vertices[:-1]).float()
    avg = max(g.edge_count / max(g.vertex_count, 1), 1.0)
    skew = float(deg.max().item()) / avg
    return f"v{int(math.log2(max(g.vertex_count, 2)))}-d{int(math.log2(avg))}-s{int(math.log2(max(skew, 1)))}"


def _kind(algorithm: str, name: str) -> str:
    base = name
    for suffix in ("-bulk", "-warpreduce", "-blockreduce"):
        if base.endswith(suffix):
            base = base[: -len(suffix)]
    if base.startswith("frontier-") or base == "pull-segmented":
        return "fixed"
    if algorithm == "pagerank" and base in ("vertex-pull", "vertex-pull-nodiv"):
        return "fixed"
    if base in ("vertex-push-warp", "vertex-pull-warp", "vertex-pull-warp-nodiv"):
        return "warp"
    if base in ("edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list"):
        return "edge"
    return "vertex"


def candidates(algorithm: str, name: str, sm_count: int):
    """The library's default launch ({}) first, then the tuning grid."""
    yield {}
    kind = _kind(algorithm, name)
    blocks = BLOCKS[kind]
    if algorithm == "pagerank" and kind in ("edge", "vertex"):
        blocks = [128, 256]                    # PageRank kernels are built for <= 256 threads
    if algorithm == "pagerank" and name in ("edge-list", "struct-edge-list"):
        return                                 # their hot-destination kernel has one geometry
    if algorithm == "pagerank" and kind == "fixed":
        # work-list kernels: the block shape and the long-row threshold
        for blk, long_row in itertools.product([0, 256], [0, 384, 512]):
            if blk or long_row:
                yield {k: v for k, v in (("block", blk), ("warp", long_row)) if v}
        return
    for blk, mult in itertools.product(blocks, GRID_MULT if kind != "fixed" else [0]):
        grid = sm_count * mult if mult else 0
        if kind == "warp":
            for w, c in WARP:
                if blk % w == 0:
                    yield dict(block=blk, grid=grid, warp=w, chunk=c)
        else:
            yield dict(block=blk, grid=grid)


def _time_bfs(ctx, g, name, root, cfg, repeats):
    ts = [bfs(ctx, g, name, root, loop="graph", tuned=False, **cfg).device_ms for _ in range(repeats)]
    return float(np.median(ts))


def _time_pagerank(ctx, g, name, cfg, repeats, iterations):
    ts = [pagerank(ctx, g, name, iterations, tuned=False, **cfg).device_ms for _ in range(repeats)]
    return float(np.median(ts))


def tune(ctx, g, algorithm: str, variants=None, *, root: int = 0, repeats: int = 3, iterations: int = 5,
         cache: Path | None = CACHE, log=None):
    """Tune `variants` on graph `g`; returns {variant: (config, ms)} and
    updates the cache."""
    names = variants or (bfs_variant_names() if algorithm == "bfs" else pagerank_variant_names())
    cls = shape_class(g)
    out = {}
    for name in names:
        best = None
        for cfg in candidates(algorithm, name, ctx.sm_count):
            try:
                if algorithm == "bfs":
                    ms = _time_bfs(ctx, g, name, root, cfg, repeats)
                else:
                    ms = _time_pagerank(ctx, g, name, cfg, repeats, iterations)
            except Exception:
                continue                         # e.g. shared memory limit for a warp config
            if best is None or ms < best[1]:
                best = (cfg, ms)
        if best is None:
            continue
        out[name] = best
        if log:
            log(f"{algorithm} {name} {cls}: {best[0]} {best[1]:.3f} ms")
    if cache is not None:
        data = json.loads(cache.read_text()) if cache.exists() else {}
        for name, (cfg, ms) in out.items():
            data.setdefault(algorithm, {}).setdefault(name, {})[cls] = {"config": cfg, "ms": ms}
        cache.parent.mkdir(parents=True, exist_ok=True)
        cache.write_text(json.dumps(data, indent=1, sort_keys=True))
        export_tsv(cache)
    return out


def export_tsv(cache: Path = CACHE, out: Path | None = None) -> Path:
    """The per-variant entries of the cache as tab-separated lines
    `algorithm variant class block grid warp chunk`, the form the C++ plugins
    read (kernel-runner runs without Python)."""
    out = out or cache.with_suffix(".tsv")
    data = json.loads(cache.read_text()) if cache.exists() else {}
    lines = []
    for algorithm in ("bfs", "pagerank"):
        for name, classes in sorted(data.get(algorithm, {}).items()):
            for cls, entry in sorted(classes.items()):
                c = entry["config"]
                lines.append("\t".join([algorithm, name, cls] + [str(int(c.get(k, 0)))
                                                                  for k in ("block", "grid", "warp", "chunk")]))
    out.write_text("".join(line + "\n" for line in lines))
    return out


# A tuned entry is used for graphs whose shape class is at most this far
# (sum of the log2 differences of vertices, average degree and skew) from
# the class it was tuned on; farther graphs keep the library default.
MAX_CLASS_DISTANCE = 2


def class_distance(a: str, b: str) -> int:
    """Sum of the differences of two shape classes' log2 fields."""
    x = [int(t[1:]) for t in a.split("-")]
    y = [int(t[1:]) for t in b.split("-")]
    return sum(abs(p - q) for p, q in zip(x, y))


_loaded: dict = {}


def _load(cache: Path) -> dict:
    """The cache's contents, re-read only when the file changes."""
    try:
        stamp = cache.stat().st_mtime_ns
    except OSError:
        return {}
    hit = _loaded.get(cache)
    if hit is None or hit[0] != stamp:
        hit = (stamp, json.loads(cache.read_text()))
        _loaded[cache] = hit
    return hit[1]


def graph_class(g) -> str | None:
    """shape_class(g), kept on the graph object (None for views without the
    forward offsets)."""
    cls = getattr(g, "_shape_class", None)
    if cls is None:
        if getattr(g, "fwd_vertices", None) is None or not getattr(g, "vertex_count", 0):
            return None
        cls = shape_class(g)
        try:
            g._shape_class = cls
        except AttributeError:
            pass
    return cls


def tuned_config(algorithm: str, name: str, g, cache: Path = CACHE) -> dict:
    """What bfs() / pagerank() launch a variant with when the caller gives
    no geometry: the tuned configuration of the graph's shape class (or of
    the nearest cached class within MAX_CLASS_DISTANCE), else {} -- the
    library's default."""
    cls = graph_class(g)
    if cls is None:
        return {}
    entries = _load(cache).get(algorithm, {}).get(name, {})
    return _nearest(entries, cls)


def _nearest(entries: dict, cls: str) -> dict:
    if not entries:
        return {}
    if cls in entries:
        return dict(entries[cls]["config"])
    near = min(entries, key=lambda other: class_distance(cls, other))
    if class_distance(cls, near) > MAX_CLASS_DISTANCE:
        return {}
    return dict(entries[near]["config"])


def lookup(algorithm: str, name: str, g, cache: Path = CACHE) -> dict:
    """The tuned configuration for the nearest cached shape class within
    MAX_CLASS_DISTANCE (or {}: the library default)."""
    if not cache.exists():
        return {}
    entries = json.loads(cache.read_text()).get(algorithm, {}).get(name, {})
    if not entries:
        return {}
    cls = shape_class(g)
    if cls in entries:
        return dict(entries[cls]["config"])
    near = min(entries, key=lambda other: class_distance(cls, other))
    if class_distance(cls, near) > MAX_CLASS_DISTANCE:
        return {}
    return dict(entries[near]["config"])


# ---------------------------------------------------------------------------
# batched launch: the push/pull divisor
# ---------------------------------------------------------------------------
BU_DIVISORS = [4, 8, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 1024, 2048]


def tune_batch(ctx, run, key: str, *, divisors=BU_DIVISORS, repeats: int = 3, cache: Path | None = CACHE,
               log=None):
    """`run(bu_div)` runs one batched launch and returns its bw_batch_result;
    keeps the divisor with the lowest median device time under
    cache["batch"][key].  Depths are identical for every divisor (the level
    direction changes how, not what, a level visits)."""
    best = None
    for d in divisors:
        run(d)                                        # warm-up
        ms = float(np.median([run(d).device_ms for _ in range(repeats)]))
        if log:
            log(f"batch {key} divisor {d}: {ms:.3f} ms")
        if best is None or ms < best[1]:
            best = (d, ms)
    if cache is not None:
        data = json.loads(cache.read_text()) if cache.exists() else {}
        data.setdefault("batch", {})[key] = {"bu_div": best[0], "ms": best[1]}
        cache.parent.mkdir(parents=True, exist_ok=True)
        cache.write_text(json.dumps(data, indent=1, sort_keys=True))
    return best


def batch_key(mode: str, g=None) -> str:
    """Cache key: the mode, and for many sources on one graph its shape class."""
    return f"sources/{shape_class(g)}" if mode == "sources" and g is not None else mode


def lookup_batch(mode: str, g=None, cache: Path = CACHE) -> int:
    """The tuned divisor for this mode (and, for sources, the nearest shape
    class of `g` within MAX_CLASS_DISTANCE), or 0 (the library default)."""
    if not cache.exists():
        return 0
    entries = json.loads(cache.read_text()).get("batch", {})
    key = batch_key(mode, g)
    if key in entries:
        return int(entries[key]["bu_div"])
    if mode != "sources" or g is None:
        return 0
    cands = [k for k in entries if k.startswith("sources/")]
    if not cands:
        return 0
    cls = shape_class(g)
    near = min(cands, key=lambda k: class_distance(cls, k.split("/", 1)[1]))
    if class_distance(cls, near.split("/", 1)[1]) > MAX_CLASS_DISTANCE:
        return 0
    return int(entries[near]["bu_div"])


# ---------------------------------------------------------------------------
# the shipped cache: every variant on the benchmark configurations' shapes
# ---------------------------------------------------------------------------
STANDARD = (
    ("pagerank", "rmat", dict(scale=22, edge_factor=16, seed=22)),
    ("pagerank", "er", dict(n=4194304, m=67108864, seed=23)),
    ("pagerank", "rmat", dict(scale=16, edge_factor=16, seed=16)),
    ("bfs", "rmat", dict(scale=22, edge_factor=16, seed=22, symmetrise=True)),
    ("bfs", "rmat", dict(scale=16, edge_factor=16, seed=16)),
    ("bfs", "ba", dict(n=2097152, m=8, seed=8)),
)


def tune_standard(ctx, cache: Path = CACHE, log=print):
    """Tune every BFS and PageRank variant on the benchmark configurations'
    graph shapes (BFS from the highest out-degree vertex; PageRank over 5
    iterations, enough for the pull variants to take the hub-first order)."""
    import torch

    from . import DeviceGraph
    for algorithm, kind, kw in STANDARD:
        g = DeviceGraph.generate(kind, reps=63, **kw)
        root = int(torch.argmax(g.fwd_vertices[1:] - g.fwd_vertices[:-1]).item())
        log(f"{algorithm} on {kind} {kw}: class {shape_class(g)}")
        tune(ctx, g, algorithm, root=root, cache=cache, log=log)
        del g
        torch.cuda.empty_cache()


if __name__ == "__main__":
    import argparse

    from . import Context
    ap = argparse.ArgumentParser(description="tune every variant on the benchmark graph shapes")
    ap.add_argument("--cache", default=str(CACHE))
    a = ap.parse_args()
    tune_standard(Context(0), cache=Path(a.cache), log=lambda s: print(s, flush=True))
