"""The CPU oracle against closed-form answers, FP64 and (when present) the
golden fixtures recorded from the reference's own kernels.  CPU only."""
from pathlib import Path

import numpy as np
import pytest

import belewitte_gb300 as bw
import oracle
from tests.graphs import catalog, chain, root_of, star

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_bfs_chain_star_grid():
    g = chain(100)
    lv, cnt = oracle.bfs(g.vertex_count, g.fwd_vertices, g.fwd_edges, 0)
    assert np.array_equal(lv, np.arange(100))
    assert len(cnt) == 100 and cnt[-1] == 0
    lv, _ = oracle.bfs(g.vertex_count, g.fwd_vertices, g.fwd_edges, 50)
    assert np.all(lv[:50] == oracle.INF) and np.array_equal(lv[50:], np.arange(50))
    s = star(64)
    lv, cnt = oracle.bfs(s.vertex_count, s.fwd_vertices, s.fwd_edges, 0)
    assert lv[0] == 0 and np.all(lv[1:] == 1) and list(cnt) == [63, 0]
    h, w = 9, 11
    gr = bw.HostGraph.grid(h, w)
    lv, cnt = oracle.bfs(gr.vertex_count, gr.fwd_vertices, gr.fwd_edges, 0)
    yy, xx = np.divmod(np.arange(h * w), w)
    assert np.array_equal(lv, yy + xx)             # Manhattan distance
    assert len(cnt) == (h - 1) + (w - 1) + 1


@pytest.mark.parametrize("name", ["rmat10", "rmat12_sym", "er", "grid", "ba", "isolated"])
def test_parallel_bfs_matches(name):
    make, root = catalog()[name]
    g = make()
    r = root_of(g, root)
    a, _ = oracle.bfs(g.vertex_count, g.fwd_vertices, g.fwd_edges, r)
    b, _ = oracle.bfs_parallel(g.vertex_count, g.fwd_vertices, g.fwd_edges, r, threads=4)
    assert np.array_equal(a, b)


def test_out_degrees():
    g = bw.HostGraph.rmat(11, 16, seed=3)
    assert np.array_equal(oracle.out_degrees(g.vertex_count, g.rev_vertices, g.rev_edges), g.out_degrees())


@pytest.mark.parametrize("name", ["rmat10", "rmat14", "er", "grid", "ba"])
@pytest.mark.parametrize("sem", [oracle.PR_DIV, oracle.PR_NODIV])
def test_pagerank_fp32_vs_fp64(name, sem):
    g = catalog()[name][0]()
    pr, diffs = oracle.pagerank(sem, g.vertex_count, g.rev_vertices, g.rev_edges, 30)
    ref = oracle.pagerank_f64(sem, g.vertex_count, g.rev_vertices, g.rev_edges, 30)
    rel = np.abs(pr.astype(np.float64) - ref) / np.abs(ref)
    assert rel.max() < 1e-4                          # the FP64 bar
    assert np.all(np.diff(diffs[5:]) <= 1e-6)        # converging


def test_pagerank_parallel_bitexact():
    g = bw.HostGraph.rmat(13, 16, seed=7)
    a, _ = oracle.pagerank(oracle.PR_DIV, g.vertex_count, g.rev_vertices, g.rev_edges, 20)
    b = oracle.pagerank_parallel(g.vertex_count, g.rev_vertices, g.rev_edges, 20, threads=4)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_pagerank_nodiv_first_iteration_trap():
    # vertex-pull-nodiv sums undivided 1/N values in iteration 1
    # (pagerank/pagerank.cpp:88), so it differs from the div variants.
    g = bw.HostGraph.rmat(10, 16, seed=1)
    a, _ = oracle.pagerank(oracle.PR_DIV, g.vertex_count, g.rev_vertices, g.rev_edges, 30)
    b, _ = oracle.pagerank(oracle.PR_NODIV, g.vertex_count, g.rev_vertices, g.rev_edges, 30)
    assert np.abs(a - b).max() / a.max() > 1e-3


def test_pagerank_single_iteration_closed_form():
    # one iteration, div semantics, on a star 0 -> {1..k}: leaves get
    # 0.15/N + 0.85 * (1/N)/k, the centre 0.15/N.
    k = 9
    g = star(k + 1)
    n = g.vertex_count
    pr, _ = oracle.pagerank(oracle.PR_DIV, n, g.rev_vertices, g.rev_edges, 1)
    init = np.float32(1.0) / np.float32(n)
    leaf = np.float32((1.0 - np.float64(np.float32(0.85))) / n +
                      np.float64(np.float32(0.85) * (init / np.float32(k))))
    assert pr[0] == np.float32((1.0 - np.float64(np.float32(0.85))) / n)
    assert np.all(pr[1:] == leaf)


def test_format_rank():
    # --validate output: setprecision(digits10 + 1) (pagerank/pagerank.cpp:135-141)
    assert oracle.format_rank(0.00123456789) == "0.001234568"
    assert oracle.format_rank(1.0) == "1"


def _golden_files():
    return sorted(GOLDEN.glob("*.npz"))


@pytest.mark.skipif(not _golden_files(), reason="no golden fixtures recorded yet")
def test_oracle_matches_reference_golden():
    """Golden fixtures recorded by running the reference's own kernels
    (tests/golden/make_golden.py).  BFS depths and level counts bit-exact;
    vertex-pull and vertex-pull-nodiv ranks bit-exact; the atomic variants
    within the float-atomic reordering tolerance."""
    for f in _golden_files():
        d = np.load(f)
        n = int(d["n"])
        fv, fe, rv, re = d["fwd_vertices"], d["fwd_edges"], d["rev_vertices"], d["rev_edges"]
        lv, cnt = oracle.bfs(n, fv, fe, int(d["root"]))
        assert np.array_equal(lv, d["bfs_levels"]), f.name
        assert np.array_equal(cnt, d["bfs_counts"]), f.name
        it = int(d["iterations"])
        div, _ = oracle.pagerank(oracle.PR_DIV, n, rv, re, it)
        nodiv, _ = oracle.pagerank(oracle.PR_NODIV, n, rv, re, it)
        for name in [k for k in d.files if k.startswith("pr_")]:
            ref = d[name]
            mine = nodiv if "nodiv" in name else div
            if name in ("pr_vertex-pull", "pr_vertex-pull-nodiv"):
                assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32)), (f.name, name)
            else:
                rel = np.abs(mine.astype(np.float64) - ref) / np.abs(ref.astype(np.float64))
                assert rel.max() <= 1e-5, (f.name, name, rel.max())
