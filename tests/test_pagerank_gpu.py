"""PageRank parity on the GPU through the C ABI, every variant.

Tolerances (stated by the requirement this library is built to):
  * vertex-pull, vertex-pull-nodiv, pull-segmented: bit-exact against the
    oracle (the reference's sequential row order and the same float /
    double operations);
  * the float-atomic variants (edge lists, push, warp pull -- the reference's
    own kernels of these names add with float atomics in no fixed order):
    max relative error <= 1e-5 against the oracle of their semantics class
    where the reference's own sum is that close to exact, and <= 1e-4
    against the FP64 oracle.
"""
import numpy as np
import pytest

import belewitte_gb300 as bw
import oracle
from tests.graphs import catalog

pytestmark = pytest.mark.gpu

REL_REF = 1e-5
REL_F64 = 1e-4
GRAPHS = ["rmat10", "rmat12_sym", "rmat14", "er", "grid", "ba", "chain", "star", "tiny", "isolated"]
BITEXACT = {"vertex-pull", "vertex-pull-nodiv", "pull-segmented"}


@pytest.fixture(scope="module")
def graphs(ctx):
    out = {}
    for name in GRAPHS:
        h = catalog()[name][0]()
        out[name] = (h, bw.DeviceGraph(h))
    return out


def _oracles(h, it, cache={}):
    key = (id(h), it)
    if key not in cache:
        n = h.vertex_count
        div, _ = oracle.pagerank(oracle.PR_DIV, n, h.rev_vertices, h.rev_edges, it)
        nodiv, _ = oracle.pagerank(oracle.PR_NODIV, n, h.rev_vertices, h.rev_edges, it)
        d64 = oracle.pagerank_f64(oracle.PR_DIV, n, h.rev_vertices, h.rev_edges, it)
        n64 = oracle.pagerank_f64(oracle.PR_NODIV, n, h.rev_vertices, h.rev_edges, it)
        cache[key] = (div, nodiv, d64, n64)
    return cache[key]


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float((np.abs(a - b) / np.abs(b)).max())


@pytest.mark.parametrize("variant", list(range(11)))
@pytest.mark.parametrize("iterations", [1, 30])
def test_variant_parity(ctx, graphs, variant, iterations):
    name = bw.pagerank_variant_names()[variant]
    for gname, (h, g) in graphs.items():
        run = bw.pagerank(ctx, g, variant, iterations)
        got = run.ranks.cpu().numpy()
        div, nodiv, d64, n64 = _oracles(h, iterations)
        ref, r64 = (nodiv, n64) if "nodiv" in name else (div, d64)
        if name in BITEXACT:
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (name, gname)
        else:
            assert _rel(got, ref) <= REL_REF, (name, gname, _rel(got, ref))
        assert _rel(got, r64) <= REL_F64, (name, gname)


def _chosen_in_degrees(n=80000, seed=9):
    """In-rows of chosen lengths around every boundary of the long-row paths
    (pieces of 512, batches of rows up to 2048 terms, piece-parallel rows
    above it, their 1024-term serial start), sources drawn at random with
    varied out-degrees."""
    rng = np.random.default_rng(seed)
    lengths = [1, 255, 256, 257, 300, 511, 512, 513, 1023, 1024, 1025, 1535, 1536, 1537, 2047, 2048, 2049,
               2560, 2561, 4095, 4096, 4097, 5000, 20000]
    lengths += list(rng.integers(257, 6000, 70))
    src, dst = [], []
    for v, d in enumerate(lengths):
        src.append(rng.choice(np.arange(len(lengths), n), size=d, replace=False))
        dst.append(np.full(d, v))
    src.append(rng.integers(len(lengths), n, 200000))      # background edges
    dst.append(rng.integers(len(lengths), n, 200000))      # the chosen rows keep their lengths
    return bw.HostGraph.from_edges(n, np.concatenate(src).astype(np.uint32), np.concatenate(dst).astype(np.uint32))


@pytest.fixture(scope="module")
def long_graphs(ctx):
    from tests.graphs import star_in
    out = {}
    for kind, h in (("star_in", star_in(200000)), ("rmat16", bw.HostGraph.rmat(16, 32, seed=3)),
                    ("chosen", _chosen_in_degrees())):
        out[kind] = (h, bw.DeviceGraph(h))
    return out


@pytest.mark.parametrize("variant", ["vertex-pull", "vertex-pull-nodiv", "pull-segmented"])
@pytest.mark.parametrize("iterations", [1, 2, 30])
def test_long_rows(ctx, long_graphs, variant, iterations):
    """In-rows far longer than one work item, on every path the exact
    variants take (batches of rows up to 2048 terms summed one row per lane,
    longer rows summed piece-parallel), including a 199,999-term row of
    equal terms (a round-half-even tie at nearly every step), rows at every
    length boundary and R-MAT hubs: bit-identical to the reference (whose
    own loop is 1.2e-3 from FP64 after one iteration on the equal-term
    row)."""
    for kind, (h, g) in long_graphs.items():
        got = bw.pagerank(ctx, g, variant, iterations).ranks.cpu().numpy()
        div, nodiv, d64, n64 = _oracles(h, iterations)
        ref = nodiv if "nodiv" in variant else div
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (variant, kind)


@pytest.mark.parametrize("variant", ["vertex-pull", "vertex-pull-nodiv", "pull-segmented"])
@pytest.mark.parametrize("block,hubs,long_row", [(256, 0, 0), (256, 4, 512), (256, 2048, 64), (1024, 0, 300),
                                                  (1024, 16384, 0), (1024, 16384, 512), (1024, 1 << 20, 1)])
@pytest.mark.parametrize("relabel", [False, True])
def test_pull_shapes(ctx, graphs, long_graphs, variant, block, hubs, long_row, relabel):
    """Both block shapes of the work-list kernels, with and without the
    shared-memory hub cache (sizes beyond the graph or the shared memory
    are clamped), long-row thresholds from 1 to 512 and the hub-first
    source order: results do not depend on any of them."""
    for name, (h, g) in list(long_graphs.items()) + [("rmat14", graphs["rmat14"]), ("chain", graphs["chain"])]:
        got = bw.pagerank(ctx, g, variant, 30, block=block, chunk=hubs, warp=long_row,
                          relabel=relabel).ranks.cpu().numpy()
        div, nodiv, d64, n64 = _oracles(h, 30)
        ref = nodiv if "nodiv" in variant else div
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (variant, name, block, hubs)


@pytest.mark.parametrize("variant", ["vertex-push-warp", "vertex-pull-warp", "vertex-pull-warp-nodiv"])
@pytest.mark.parametrize("w,c", [(1, 1), (4, 8), (16, 64), (32, 32)])
def test_warp_configs(ctx, graphs, variant, w, c):
    h, g = graphs["rmat14"]
    run = bw.pagerank(ctx, g, variant, 10, warp=w, chunk=c)
    div, nodiv, _, _ = _oracles(h, 10)
    ref = nodiv if "nodiv" in variant else div
    assert _rel(run.ranks.cpu().numpy(), ref) <= REL_REF


def test_switching_schedule(ctx, graphs):
    """A per-iteration schedule over div variants stays within tolerance."""
    h, g = graphs["rmat14"]
    sched = ["edge-list", "vertex-pull", "pull-segmented", "rev-struct-edge-list", "vertex-push-warp",
             "vertex-pull-warp", "vertex-push", "rev-edge-list", "struct-edge-list"]
    run = bw.pagerank_schedule(ctx, g, sched, 30, time_iterations=True)
    div, _, _, _ = _oracles(h, 30)
    assert _rel(run.ranks.cpu().numpy(), div) <= REL_REF
    assert len(run.iteration_ms) == 30 and all(t > 0 for t in run.iteration_ms)
    with pytest.raises(bw.BwError):
        bw.pagerank_schedule(ctx, g, ["vertex-pull", "vertex-pull-nodiv"], 5)


def test_diffs_reported(ctx, graphs):
    h, g = graphs["rmat10"]
    run = bw.pagerank(ctx, g, "vertex-pull", 30)
    _, diffs = oracle.pagerank(oracle.PR_DIV, h.vertex_count, h.rev_vertices, h.rev_edges, 30)
    assert np.allclose(run.diffs, diffs, rtol=1e-3, atol=1e-9)


def test_kernel_launch_count(ctx, graphs, long_graphs):
    """The run reports exactly the kernels of this library it launched, and
    no set-up step is a library call:
    - degrees (row lengths): 1;
    - the work list: row counts, two tile scans, the partition, the long-row
      sort (count, three scan launches, scatter), piece count, scan (three)
      and emission, short-item count, scan (three) and emission: 20;
    - the hub-first order: the degree-class sort (5; its scatter also
      writes the slots), the device-side decision unless forced, and for
      the nodiv variants the source translation (the div variants' first
      iteration translates the sources itself);
    - init: 1;
    - per iteration two kernels: work list + long-row sums for the exact
      variants, scatter + consolidation for the atomic ones."""
    _, g = graphs["rmat14"]
    assert bw.pagerank(ctx, g, "vertex-pull", 5).kernel_launches == 1 + 20 + 6 + 1 + 2 * 5
    assert bw.pagerank(ctx, g, "vertex-pull", 2).kernel_launches == 1 + 20 + 1 + 2 * 2
    assert bw.pagerank(ctx, g, "vertex-pull-nodiv", 5).kernel_launches == 1 + 20 + 7 + 1 + 2 * 5
    assert bw.pagerank(ctx, g, "rev-edge-list", 5).kernel_launches == 1 + 1 + 2 * 5
    assert bw.pagerank(ctx, g, "pull-segmented", 5, relabel=True).kernel_launches == 1 + 20 + 5 + 1 + 2 * 5
    assert bw.pagerank(ctx, g, "pull-segmented", 5, relabel=False).kernel_launches == 1 + 20 + 1 + 2 * 5


@pytest.mark.parametrize("variant", ["vertex-pull", "vertex-pull-nodiv", "pull-segmented", "vertex-pull-warp"])
def test_reverse_only_view(ctx, graphs, long_graphs, variant):
    """A caller holding only the reverse CSR (as the reference's pull
    variants load it): degrees are counted from the source stream (shared-
    memory counters for the low ids, global ones for the rest) and every
    result matches the full view's."""
    from belewitte_gb300 import _abi
    for name, (h, g) in [("rmat14", graphs["rmat14"]), ("star", graphs["star"])] + list(long_graphs.items()):
        v = g.view

        class RevOnly:
            vertex_count, edge_count = g.vertex_count, g.edge_count
            view = _abi.GraphView(v.vertex_count, v.edge_count, 0, 0, v.rev_vertices, v.rev_edges, 0, 0, 0, 0)
        got = bw.pagerank(ctx, RevOnly, variant, 30).ranks.cpu().numpy()
        div, nodiv, d64, n64 = _oracles(h, 30)
        ref, r64 = (nodiv, n64) if "nodiv" in variant else (div, d64)
        if variant in BITEXACT:
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (variant, name)
        else:
            # vertex-pull-warp: the reference's kernel adds its lanes' partial
            # sums with float atomics, so its order is unspecified; held to
            # the oracle where the reference's own sum is within 1e-5 of
            # exact, and to FP64 everywhere
            if _rel(ref, r64) <= REL_REF:
                assert _rel(got, ref) <= REL_REF, (variant, name)
            assert _rel(got, r64) <= REL_F64, (variant, name)


def test_gather_probe(ctx):
    """bw_gather_probe sums exactly the gathered values (indices past the
    array skipped) and reports a positive rate."""
    torch = pytest.importorskip("torch")
    gen = torch.Generator(device="cuda:0")
    gen.manual_seed(5)
    n, m = 1 << 20, 3_000_001
    src = torch.randint(0, 8, (n,), dtype=torch.int32, device="cuda:0", generator=gen).float()
    idx = torch.randint(0, n + 1000, (m,), dtype=torch.int32, device="cuda:0", generator=gen)
    ok = idx < n
    want = float(src[idx[ok].long()].double().sum().item())
    assert bw.gather_probe_sum(ctx, src, idx) == want         # small integers: exact in any order
    assert bw.gather_ceiling(ctx, src, idx, warmup=1, repeats=3) > 1e9


@pytest.mark.parametrize("variant", ["vertex-pull", "pull-segmented", "vertex-push", "vertex-pull-warp-nodiv",
                                     "rev-edge-list"])
def test_graph_loop_matches_host_loop(ctx, graphs, long_graphs, variant):
    """loop="graph" (the iterations captured into one CUDA graph) gives the
    host loop's ranks: bit for bit where the variant is deterministic,
    within the reference tolerance where it adds with float atomics."""
    for name, (h, g) in [("rmat14", graphs["rmat14"]), ("star", graphs["star"])] + list(long_graphs.items()):
        want = bw.pagerank(ctx, g, variant, 12).ranks.cpu().numpy()
        got = bw.pagerank(ctx, g, variant, 12, loop="graph").ranks.cpu().numpy()
        if variant in BITEXACT:
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (variant, name)
        else:
            assert _rel(got, want) <= REL_REF, (variant, name)


@pytest.mark.parametrize("variant", ["pull-segmented", "vertex-pull-nodiv", "rev-edge-list"])
@pytest.mark.parametrize("loop", ["host", "graph"])
def test_l2_window_leaves_results_unchanged(ctx, graphs, long_graphs, variant, loop):
    """BW_LAUNCH_L2_WINDOW (the gathered vector persisting in L2) changes
    where the lines live, not what the kernels compute."""
    import torch
    side = torch.cuda.Stream()                    # a window is an attribute of a created stream
    for name, (h, g) in [("rmat14", graphs["rmat14"])] + list(long_graphs.items()):
        want = bw.pagerank(ctx, g, variant, 12, loop=loop).ranks.cpu().numpy()
        with torch.cuda.stream(side):
            got = bw.pagerank(ctx, g, variant, 12, loop=loop, l2_window=True).ranks.cpu().numpy()
        if variant in BITEXACT:
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (variant, name)
        else:
            assert _rel(got, want) <= REL_REF, (variant, name)


@pytest.mark.parametrize("n_graph", ["grid_odd", "ba_odd"])
def test_fresh_context_odd_vertex_count(n_graph):
    """A context whose first graph has a vertex count that is not a multiple
    of 4: both contribution buffers it allocates are gathered with 16-byte
    vector loads (the hub cache), so both must start aligned.  Every variant,
    several iterations, against the oracle."""
    h = bw.HostGraph.grid(37, 41) if n_graph == "grid_odd" else bw.HostGraph.barabasi_albert(70001, 3, seed=5)
    assert h.vertex_count % 4 != 0
    c = bw.Context(0)
    try:
        g = bw.DeviceGraph(h)
        div, _ = oracle.pagerank(oracle.PR_DIV, h.vertex_count, h.rev_vertices, h.rev_edges, 7)
        nodiv, _ = oracle.pagerank(oracle.PR_NODIV, h.vertex_count, h.rev_vertices, h.rev_edges, 7)
        for name in bw.pagerank_variant_names():
            for loop in ("host", "graph"):
                got = bw.pagerank(c, g, name, 7, loop=loop).ranks.cpu().numpy()
                ref = nodiv if "nodiv" in name else div
                if name in BITEXACT:
                    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (name, loop)
                else:
                    assert _rel(got, ref) <= REL_REF, (name, loop)
    finally:
        c.close()
