"""Graph substrate (host C++ through the C ABI): generators, CSR layout,
.graph file format, degree statistics.  CPU only."""
import numpy as np
import pytest

import belewitte_gb300 as bw
from tests.graphs import catalog


def _check_csr(g):
    n, m = g.vertex_count, g.edge_count
    for off, edg in ((g.fwd_vertices, g.fwd_edges), (g.rev_vertices, g.rev_edges)):
        assert off[0] == 0 and off[-1] == m
        assert np.all(np.diff(off.astype(np.int64)) >= 0)
        assert m == 0 or edg.max() < n
        # rows sorted, no duplicates (utils/Graph.hpp output -> sort -> unique)
        for v in range(min(n, 2000)):
            row = edg[off[v]:off[v + 1]]
            assert np.all(np.diff(row.astype(np.int64)) > 0)
    # reverse CSR is the transpose of the forward CSR
    src = np.repeat(np.arange(n), np.diff(g.fwd_vertices.astype(np.int64)))
    fwd = set(zip(src.tolist(), g.fwd_edges.tolist()))
    rsrc = np.repeat(np.arange(n), np.diff(g.rev_vertices.astype(np.int64)))
    rev = set(zip(g.rev_edges.tolist(), rsrc.tolist()))
    assert fwd == rev


@pytest.mark.parametrize("name", ["rmat10", "rmat12_sym", "er", "grid", "ba", "chain", "star", "tiny"])
def test_csr_valid(name):
    make, _ = catalog()[name]
    g = make()
    _check_csr(g)
    src = np.repeat(np.arange(g.vertex_count), np.diff(g.fwd_vertices.astype(np.int64)))
    assert not np.any(src == g.fwd_edges), "self-loops must be removed"


def test_generators_deterministic():
    a = bw.HostGraph.rmat(12, 16, seed=9)
    b = bw.HostGraph.rmat(12, 16, seed=9)
    c = bw.HostGraph.rmat(12, 16, seed=10)
    assert np.array_equal(a.fwd_edges, b.fwd_edges) and np.array_equal(a.fwd_vertices, b.fwd_vertices)
    assert not np.array_equal(a.fwd_vertices, c.fwd_vertices)
    e1 = bw.HostGraph.erdos_renyi(3000, 20000, seed=1)
    e2 = bw.HostGraph.erdos_renyi(3000, 20000, seed=1)
    assert np.array_equal(e1.fwd_edges, e2.fwd_edges)
    b1 = bw.HostGraph.barabasi_albert(3000, 4, seed=1)
    b2 = bw.HostGraph.barabasi_albert(3000, 4, seed=1)
    assert np.array_equal(b1.fwd_edges, b2.fwd_edges)


def test_rmat_skew():
    g = bw.HostGraph.rmat(14, 16, seed=1)
    deg = g.out_degrees()
    # a = 0.57 concentrates edges on low ids: vertex 0 is the hub
    assert deg.argmax() == 0
    assert deg.max() > 20 * deg.mean()
    # edge factor 16 before dedupe
    assert 0.5 * 16 * 2 ** 14 < g.edge_count <= 16 * 2 ** 14


def test_symmetrise():
    g = bw.HostGraph.rmat(11, 8, seed=3, symmetrise=True)
    assert g.undirected
    assert np.array_equal(g.fwd_vertices, g.rev_vertices)
    src = np.repeat(np.arange(g.vertex_count), np.diff(g.fwd_vertices.astype(np.int64)))
    s = set(zip(src.tolist(), g.fwd_edges.tolist()))
    assert all((b, a) in s for a, b in s)


def test_grid_shape():
    h, w = 13, 17
    g = bw.HostGraph.grid(h, w)
    deg = g.out_degrees()
    assert g.edge_count == 2 * (h * (w - 1) + w * (h - 1))
    assert deg[0] == 2 and deg[w + 1] == 4 and deg.max() == 4


def test_ba_degrees():
    g = bw.HostGraph.barabasi_albert(20000, 4, seed=2)
    deg = g.out_degrees()
    assert deg.min() >= 1
    assert deg.max() > 30 * np.median(deg)   # power-law hubs


def test_from_edges_flags():
    g = bw.HostGraph.from_edges(4, [0, 0, 1, 2, 2], [1, 1, 1, 3, 0])
    assert g.edge_count == 3                   # duplicate and self-loop removed
    g2 = bw.HostGraph.from_edges(4, [0, 0, 1], [1, 1, 1], dedupe=False, drop_self_loops=False)
    assert g2.edge_count == 3
    with pytest.raises(bw.BwError):
        bw.HostGraph.from_edges(3, [0], [7])


def test_graph_file_roundtrip(tmp_path):
    for g in (bw.HostGraph.rmat(10, 8, seed=1), bw.HostGraph.grid(5, 6)):
        p = tmp_path / "g.graph"
        g.write(p)
        h = bw.HostGraph.read(p)
        assert h.vertex_count == g.vertex_count and h.edge_count == g.edge_count
        assert h.undirected == g.undirected
        for a in ("fwd_vertices", "fwd_edges", "rev_vertices", "rev_edges"):
            assert np.array_equal(getattr(g, a), getattr(h, a))
        # size rule of utils/Graph.hpp:784-807 (v1, 4-byte fields)
        n, m = g.vertex_count, g.edge_count
        per = (n + 1) * 4 + m * 4
        assert p.stat().st_size == 40 + per * (1 if g.undirected else 2)


def test_graph_file_v0(tmp_path):
    # version 0: {undirected, N, M} header, then CSR (and reverse CSR)
    n, off, edg = 3, np.array([0, 1, 2, 2], np.uint32), np.array([1, 2], np.uint32)
    roff, redg = np.array([0, 0, 1, 2], np.uint32), np.array([0, 1], np.uint32)
    p = tmp_path / "v0.graph"
    np.concatenate([np.array([0, n, 2], np.uint32), off, edg, roff, redg]).tofile(p)
    g = bw.HostGraph.read(p)
    assert g.vertex_count == 3 and g.edge_count == 2 and not g.undirected
    assert np.array_equal(g.rev_edges, redg)


def test_graph_file_malformed(tmp_path):
    p = tmp_path / "bad.graph"
    np.array([1, 0, 0, 0, 4, 4, 5, 0, 3, 0, 0, 0], np.uint32).tofile(p)
    with pytest.raises(bw.BwError):
        bw.HostGraph.read(p)
    with pytest.raises(bw.BwError):
        bw.HostGraph.read(tmp_path / "missing.graph")


def _summary(values):
    # utils/StatisticalSummary.hpp:30-76 restated in numpy
    v = np.sort(np.asarray(values, dtype=np.float64))
    n = len(v)
    def med(c):
        return (c // 2 - 1, c // 2) if c % 2 == 0 else (c // 2, c // 2)
    half = n // 2
    mp, lo = med(n), med(half)
    hi = (lo[0] + half + n % 2, lo[1] + half + n % 2)
    std = np.sqrt(((v - v.mean()) ** 2).sum() / (n - 1)) if n > 1 else 0.0
    return dict(min=v[0], lower=(v[lo[0]] + v[lo[1]]) / 2, mean=v.mean(), median=(v[mp[0]] + v[mp[1]]) / 2,
                upper=(v[hi[0]] + v[hi[1]]) / 2, max=v[-1], stddev=std)


@pytest.mark.parametrize("kind", ["abs", "in", "out"])
def test_degree_statistics(kind):
    g = bw.HostGraph.rmat(10, 16, seed=4)
    out = np.diff(g.fwd_vertices.astype(np.int64))
    inn = np.diff(g.rev_vertices.astype(np.int64))
    vals = {"out": out, "in": inn, "abs": out + inn}[kind]
    got = g.degree_statistics(kind)
    want = _summary(vals)
    for k in want:
        assert got[k] == pytest.approx(want[k], rel=1e-12, abs=1e-12), k


@pytest.mark.parametrize("scale,ef,seed,sym", [(10, 16, 11, False), (12, 8, 5, True), (16, 16, 16, False),
                                               (13, 32, 2, True)])
def test_oracle_generator_equals_library_generator(scale, ef, seed, sym):
    """oracle.generate_rmat (the oracle's own C, used where the product
    library must not be loaded) gives the library's R-MAT graph bit for bit."""
    import oracle
    o = oracle.generate_rmat(scale, ef, seed=seed, symmetrise=sym)
    h = bw.HostGraph.rmat(scale, ef, seed=seed, symmetrise=sym)
    for k in ("fwd_vertices", "fwd_edges", "rev_vertices", "rev_edges"):
        assert np.array_equal(o[k], getattr(h, k)), k


@pytest.mark.parametrize("n", [2, 3, 1000, 1500, 4097, 199999])
def test_rmat_over_any_vertex_count(n):
    """R-MAT over n vertices: valid CSR of exactly n vertices, the hubs at
    the low ids like the power-of-two generator's."""
    g = bw.HostGraph.rmat_n(n, 16, seed=7)
    assert g.vertex_count == n
    _check_csr(g)
    if n >= 1000:
        deg = np.diff(g.fwd_vertices.astype(np.int64))
        assert int(np.argmax(deg)) < n // 16
