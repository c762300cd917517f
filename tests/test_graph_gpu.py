"""The device graph generator against the host generator: the same seeded
graph, forward and reverse CSR bit for bit, for every kind (the device
generator makes the benchmark graphs; the host one the parity graphs)."""
import numpy as np
import pytest

import belewitte_gb300 as bw

pytestmark = pytest.mark.gpu

CASES = [
    ("rmat", dict(scale=12, edge_factor=16, seed=3), lambda: bw.HostGraph.rmat(12, 16, seed=3)),
    ("rmat", dict(scale=16, edge_factor=16, seed=16), lambda: bw.HostGraph.rmat(16, 16, seed=16)),
    ("rmat", dict(scale=18, edge_factor=16, seed=24, symmetrise=True),
     lambda: bw.HostGraph.rmat(18, 16, seed=24, symmetrise=True)),
    ("rmat", dict(scale=14, edge_factor=8, a=0.45, b=0.25, c=0.15, seed=9),
     lambda: bw.HostGraph.rmat(14, 8, a=0.45, b=0.25, c=0.15, seed=9)),
    ("rmat_n", dict(n=1000, edge_factor=8, seed=5), lambda: bw.HostGraph.rmat_n(1000, 8, seed=5)),
    ("rmat_n", dict(n=199999, edge_factor=32, seed=6), lambda: bw.HostGraph.rmat_n(199999, 32, seed=6)),
    ("er", dict(n=70000, m=1 << 20, seed=23), lambda: bw.HostGraph.erdos_renyi(70000, 1 << 20, seed=23)),
    ("er", dict(n=5000, m=40000, seed=4, symmetrise=True),
     lambda: bw.HostGraph.erdos_renyi(5000, 40000, seed=4, symmetrise=True)),
    ("grid", dict(h=512, w=300), lambda: bw.HostGraph.grid(512, 300)),
    ("ba", dict(n=100000, m=8, seed=8), lambda: bw.HostGraph.barabasi_albert(100000, 8, seed=8)),
]


@pytest.mark.parametrize("kind,kw,host", CASES, ids=[f"{c[0]}-{i}" for i, c in enumerate(CASES)])
def test_device_generator_equals_host_generator(kind, kw, host):
    g = bw.DeviceGraph.generate(kind, **kw)
    h = host()
    assert (g.vertex_count, g.edge_count, g.undirected) == (h.vertex_count, h.edge_count, h.undirected)
    got = g.to_host_arrays()
    for k in ("fwd_vertices", "fwd_edges", "rev_vertices", "rev_edges"):
        assert np.array_equal(got[k], getattr(h, k)), (kind, k)


@pytest.mark.parametrize("name", ["rmat14", "rmat12_sym", "er", "grid", "ba", "star", "tiny", "isolated", "chain"])
def test_device_degree_statistics_equal_host(ctx, name):
    """graph-details statistics on the device equal the host restatement:
    the order statistics and the mean exactly, the standard deviation to
    1e-12 (exact integer sums on the device, a Welford loop on the host)."""
    from tests.graphs import catalog
    h = catalog()[name][0]()
    g = bw.DeviceGraph(h)
    for kind in ("abs", "in", "out"):
        want = h.degree_statistics(kind)
        got = g.degree_statistics(ctx, kind)
        for k in ("min", "lower", "mean", "median", "upper", "max"):
            assert got[k] == want[k], (name, kind, k)
        assert got["stddev"] == pytest.approx(want["stddev"], rel=1e-12, abs=1e-12), (name, kind)


def test_device_degree_statistics_at_scale(ctx):
    """R-MAT scale 22 (the headline graph), generated on the device."""
    h = bw.HostGraph.rmat(20, 16, seed=22)
    g = bw.DeviceGraph.generate("rmat", scale=20, edge_factor=16, seed=22)
    for kind in ("abs", "in", "out"):
        want = h.degree_statistics(kind)
        got = g.degree_statistics(ctx, kind)
        assert [got[k] for k in ("min", "lower", "mean", "median", "upper", "max")] == \
            [want[k] for k in ("min", "lower", "mean", "median", "upper", "max")]
        assert got["stddev"] == pytest.approx(want["stddev"], rel=1e-12)
