"""Batched persistent traversal (bw_batch_run): many graphs or many sources
in one launch fed by a device work queue.

Workload A (many graphs): graphs of uneven size packed into one
concatenated CSR (global vertex ids, per-graph vertex offsets); each unit is
a BFS from the graph's max-out-degree vertex followed by a PageRank of that
graph.  Workload B (many sources): BFS from many sources on one graph.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import DeviceGraph, _abi, _ptr, library
from ._abi import check

GRAPHS, SOURCES = 0, 1


@dataclass
class PackedGraphs:
    view: object
    vertex_count: int
    edge_count: int
    offsets: object           # torch uint32-as-int32 [count + 1]
    count: int
    max_vertices: int
    roots: object             # torch int32 [count] global ids
    order: object             # torch int32 [count], largest first
    tensors: tuple = ()
    sizes: list = None        # (vertices, edges) per graph


def pack(graphs: list[DeviceGraph], device: int = 0) -> PackedGraphs:
    """Concatenate device graphs into one CSR with global vertex ids."""
    import torch
    dev = f"cuda:{device}"
    vb = eb = 0
    fv, fe, rv, re, offs, roots, sizes = [], [], [], [], [0], [], []
    for g in graphs:
        n, m = g.vertex_count, g.edge_count
        f_off = g.fwd_vertices[: n + 1].to(torch.int64)
        r_off = g.rev_vertices[: n + 1].to(torch.int64)
        fv.append((f_off[:-1] + eb).to(torch.int32))
        rv.append((r_off[:-1] + eb).to(torch.int32))
        fe.append((g.fwd_edges[:m].to(torch.int64) + vb).to(torch.int32))
        re.append((g.rev_edges[:m].to(torch.int64) + vb).to(torch.int32))
        deg = f_off[1:] - f_off[:-1]
        roots.append(int(torch.argmax(deg).item()) + vb)
        sizes.append((n, m))
        vb += n
        eb += m
        offs.append(vb)
    if eb >= 2 ** 32:
        raise ValueError("packed edge count exceeds uint32 offsets")
    tail = torch.tensor([eb], dtype=torch.int64, device=dev).to(torch.int32)
    fwd_v = torch.cat(fv + [tail])
    rev_v = torch.cat(rv + [tail])
    fwd_e = torch.cat(fe)
    rev_e = torch.cat(re)
    offsets = torch.tensor(offs, dtype=torch.int64).to(torch.int32).to(dev)
    order = torch.tensor(np.argsort([-m for _, m in sizes], kind="stable"), dtype=torch.int32, device=dev)
    view = _abi.GraphView(vb, eb, _ptr(fwd_v), _ptr(fwd_e), _ptr(rev_v), _ptr(rev_e), 0, 0, 0, 0)
    return PackedGraphs(view, vb, eb, offsets, len(graphs), max(n for n, _ in sizes),
                        torch.tensor(roots, dtype=torch.int32, device=dev), order,
                        (fwd_v, fwd_e, rev_v, rev_e), sizes)


def run_graphs(ctx, packed: PackedGraphs, pr_iterations: int = 20, levels=None, ranks=None, grid: int = 0,
               stream=None, bu_div: int | None = None):
    """Workload A: per graph a BFS and a PageRank, in one persistent launch.
    bu_div: the push/pull divisor (None: the autotuner's, else the
    library default)."""
    import torch
    from . import autotune
    if bu_div is None:
        bu_div = autotune.lookup_batch("graphs")
    dev = packed.offsets.device
    if levels is None:
        levels = torch.empty(packed.vertex_count, dtype=torch.int32, device=dev)
    if ranks is None:
        ranks = torch.empty(packed.vertex_count, dtype=torch.float32, device=dev)
    res = _abi.BatchResult()
    cfg = _abi.LaunchConfig(0, grid, 0, bu_div)
    st = stream or torch.cuda.current_stream(dev)
    check(library().bw_batch_run(ctx.handle, C.byref(packed.view), GRAPHS, _ptr(packed.offsets), packed.count,
                                 _ptr(packed.roots), _ptr(packed.order), packed.count, packed.max_vertices,
                                 pr_iterations, _ptr(levels), _ptr(ranks), C.byref(cfg), C.byref(res),
                                 C.c_void_p(st.cuda_stream)), "bw_batch_run(graphs)")
    return levels, ranks, res


def run_sources(ctx, g: DeviceGraph, sources, levels=None, grid: int = 0, stream=None, bu_div: int | None = None):
    """Workload B: BFS from every source of `sources` on graph `g`.
    bu_div: the push/pull divisor (None: the autotuner's for g's shape
    class, else the library default)."""
    import torch
    from . import autotune
    if bu_div is None:
        bu_div = autotune.lookup_batch("sources", g)
    dev = g.device
    src = torch.as_tensor(np.asarray(sources, dtype=np.int32), device=dev)
    if levels is None:
        levels = torch.empty((len(sources), g.vertex_count), dtype=torch.int32, device=dev)
    res = _abi.BatchResult()
    cfg = _abi.LaunchConfig(0, grid, 0, bu_div)
    st = stream or torch.cuda.current_stream(dev)
    check(library().bw_batch_run(ctx.handle, C.byref(g.view), SOURCES, None, 1, _ptr(src), None, len(sources),
                                 g.vertex_count, 0, _ptr(levels), None, C.byref(cfg), C.byref(res),
                                 C.c_void_p(st.cuda_stream)), "bw_batch_run(sources)")
    return levels, res


def workload_a_specs(count: int = 4096, seed: int = 5, min_vertices: int = 1000, max_vertices: int = 200000):
    """Seeded R-MAT graphs with vertex counts drawn log-uniformly from
    [min_vertices, max_vertices] and edge factors 8-32 (generated with
    DeviceGraph.generate("rmat_n", n=..., edge_factor=...))."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(min_vertices), np.log(max_vertices)
    out = []
    for _ in range(count):
        n = int(round(float(np.exp(rng.uniform(lo, hi)))))
        out.append(dict(n=min(max(n, min_vertices), max_vertices), edge_factor=int(rng.integers(8, 33)),
                        seed=int(rng.integers(1, 2 ** 31))))
    return out
