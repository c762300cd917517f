"""Graphs without edges (M = 0, edge arrays null): every BFS and PageRank
entry point gives the reference's result -- the root at depth 0 and every
other vertex unreached after one level; PageRank's constant rank from a zero
in-sum -- against the oracle, bit for bit."""
import ctypes as C

import numpy as np
import pytest

import belewitte_gb300 as bw
import oracle

pytestmark = pytest.mark.gpu

CASES = [(1, 0), (7, 3), (4097, 4096)]      # (vertices, root)


def _graph(n):
    e = np.array([], np.uint32)
    h = bw.HostGraph.from_edges(n, e, e)
    assert h.edge_count == 0
    return h, bw.DeviceGraph(h)


class _NullEdges:
    """The same graph seen through a view whose edge arrays are null."""

    def __init__(self, g):
        self.g = g                                 # keeps the offset arrays alive
        self.vertex_count, self.edge_count, self.device = g.vertex_count, 0, g.device
        self.view = bw._abi.GraphView(g.vertex_count, 0, g.fwd_vertices.data_ptr(), 0, g.rev_vertices.data_ptr(),
                                      0, 0, 0, 0, 0)


def _views(g):
    return [("arrays", g), ("null", _NullEdges(g))]


@pytest.mark.parametrize("n,root", CASES)
def test_bfs_every_variant(ctx, n, root):
    h, g = _graph(n)
    lv, cnt = oracle.bfs(n, h.fwd_vertices, h.fwd_edges, root)
    assert list(cnt) == [0]
    for variant in range(bw.library().bw_bfs_variant_count()):
        for (vname, view), loop in [(v, lp) for v in _views(g) for lp in ("host", "graph")]:
            run = bw.bfs(ctx, view, variant, root, loop=loop, stats=True)
            assert np.array_equal(run.levels.cpu().numpy(), lv), (variant, vname, loop)
            assert run.level_count == 1 and run.visited == 1 and run.traversed_edges == 0
            assert [s["frontier_vertices"] for s in run.level_stats] == [0]


@pytest.mark.parametrize("n,root", CASES)
def test_bfs_level_api_learned_and_noalloc(ctx, n, root):
    import torch
    from belewitte_gb300 import learn
    h, g = _graph(n)
    lv, _ = oracle.bfs(n, h.fwd_vertices, h.fwd_edges, root)
    lib = bw.library()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    levels = torch.full((n,), -5, dtype=torch.int32, device="cuda")
    assert lib.bw_bfs_init(ctx.handle, n, root, C.c_void_p(levels.data_ptr()), st) == 0
    f = C.c_uint32(99)
    assert lib.bw_bfs_level(ctx.handle, C.byref(g.view), bw.bfs_variant_id("vertex-push"),
                            C.c_void_p(levels.data_ptr()), 0, None, C.byref(f), st) == 0
    assert f.value == 0 and np.array_equal(levels.cpu().numpy(), lv)
    s = bw._abi.BfsLevelStats()
    assert lib.bw_bfs_frontier_stats(ctx.handle, C.byref(g.view), root, -1, C.byref(s), st) == 0
    assert s.frontier_vertices == 1 and s.frontier_edges == 0 and s.log_degree_sum == 0.0
    assert lib.bw_bfs_frontier_stats(ctx.handle, C.byref(g.view), root, 0, C.byref(s), st) == 0
    assert s.frontier_vertices == 0
    pred = learn.load_predictor()
    for loop in ("host", "graph"):
        run = learn.run_learned(ctx, g, pred, root, loop=loop)
        assert np.array_equal(run.levels.cpu().numpy(), lv) and run.level_count == 1
    for _, view in _views(g):
        sched = bw.bfs_schedule(ctx, view, ["frontier-pull", "edge-list"], root)
        assert np.array_equal(sched.levels.cpu().numpy(), lv) and sched.level_count == 1
        levels.fill_(-5)
        count = C.c_uint32()
        assert lib.bw_bfs_run_noalloc(C.byref(view.view), root, C.c_void_p(levels.data_ptr()), 0, C.byref(count),
                                      st) == 0
        assert count.value == 1 and np.array_equal(levels.cpu().numpy(), lv)


@pytest.mark.parametrize("n", [1, 7, 4097])
@pytest.mark.parametrize("iterations", [0, 1, 5])
def test_pagerank_every_variant(ctx, n, iterations):
    h, g = _graph(n)
    names = bw.pagerank_variant_names()
    want = {sem: oracle.pagerank(sem, n, h.rev_vertices, h.rev_edges, iterations)
            for sem in (oracle.PR_DIV, oracle.PR_NODIV)}
    for variant, name in enumerate(names):
        sem = oracle.PR_NODIV if "nodiv" in name else oracle.PR_DIV
        ref, diffs = want[sem]
        for (vname, view), loop in [(v, lp) for v in _views(g) for lp in ("host", "graph")]:
            run = bw.pagerank(ctx, view, variant, iterations, loop=loop)
            got = run.ranks.cpu().numpy()
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (name, vname, loop)
            assert run.iterations == iterations
            assert np.allclose(run.diffs, diffs, rtol=1e-6, atol=0), (name, run.diffs, diffs)
