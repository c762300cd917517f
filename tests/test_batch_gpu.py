"""Batched persistent traversal against the oracle, graph by graph."""
import numpy as np
import pytest

import belewitte_gb300 as bw
import oracle
from belewitte_gb300 import batch

pytestmark = pytest.mark.gpu


def test_many_graphs_bfs_and_pagerank(ctx):
    specs = batch.workload_a_specs(24, seed=3, min_vertices=200, max_vertices=9000)
    hosts = [bw.HostGraph.rmat_n(s["n"], s["edge_factor"], seed=s["seed"]) for s in specs]
    packed = batch.pack([bw.DeviceGraph(h, reps=bw.REP_FWD_CSR | bw.REP_REV_CSR) for h in hosts])
    levels, ranks, res = batch.run_graphs(ctx, packed, pr_iterations=20)
    lv_all, pr_all = levels.cpu().numpy(), ranks.cpu().numpy()
    offs = packed.offsets.cpu().numpy().astype(np.int64)
    roots = packed.roots.cpu().numpy().astype(np.int64)
    total_trav = 0
    for i, h in enumerate(hosts):
        lo, hi = offs[i], offs[i + 1]
        want, _ = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, int(roots[i] - lo))
        assert np.array_equal(lv_all[lo:hi], want), i
        deg = h.out_degrees().astype(np.int64)
        total_trav += int(deg[want != oracle.INF].sum())
        pr, _ = oracle.pagerank(oracle.PR_DIV, h.vertex_count, h.rev_vertices, h.rev_edges, 20)
        assert np.array_equal(pr_all[lo:hi].view(np.uint32), pr.view(np.uint32)), i   # vertex-pull order
    assert res.traversed_edges == total_trav and res.units == len(hosts)


def test_many_sources(ctx):
    h = bw.HostGraph.rmat(13, 16, seed=8, symmetrise=True)
    g = bw.DeviceGraph(h, reps=bw.REP_FWD_CSR | bw.REP_REV_CSR)
    rng = np.random.default_rng(1)
    srcs = rng.choice(h.vertex_count, 40, replace=False)
    levels, res = batch.run_sources(ctx, g, srcs)
    got = levels.cpu().numpy()
    for k, s in enumerate(srcs):
        want, _ = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, int(s))
        assert np.array_equal(got[k], want), k
    assert res.units == 40


def test_push_pull_divisor_keeps_depths(ctx):
    """The batched BFS's push/pull divisor (cfg chunk_size) changes only
    which levels run bottom-up: depths are identical for every divisor."""
    import torch
    from belewitte_gb300 import batch
    g = bw.DeviceGraph.generate("rmat", scale=14, edge_factor=16, seed=3, symmetrise=True)
    srcs = [0, 5, 77, 1000, 4095]
    ref = None
    for d in (0, 2, 4, 24, 96, 100000):
        levels, _ = batch.run_sources(ctx, g, srcs, bu_div=d)
        got = levels.cpu()
        if ref is None:
            ref = got
        assert torch.equal(got, ref), d
