"""BFS parity on the GPU through the C ABI: every variant, bit-exact depths
and per-level frontier counts against the oracle."""
import ctypes as C

import numpy as np
import pytest

import belewitte_gb300 as bw
import oracle
from tests.graphs import catalog, root_of

pytestmark = pytest.mark.gpu

GRAPHS = ["rmat10", "rmat12_sym", "rmat14", "er", "grid", "ba", "chain", "star", "tiny", "isolated"]


@pytest.fixture(scope="module")
def graphs(ctx):
    out = {}
    for name in GRAPHS:
        make, root = catalog()[name]
        h = make()
        r = root_of(h, root)
        lv, cnt = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, r)
        out[name] = (h, bw.DeviceGraph(h), r, lv, cnt)
    return out


@pytest.mark.parametrize("variant", list(range(34)))
def test_variant_bitexact(ctx, graphs, variant):
    for name, (h, g, r, lv, cnt) in graphs.items():
        run = bw.bfs(ctx, g, variant, r)
        got = run.levels.cpu().numpy()
        assert np.array_equal(got, lv), (bw.bfs_variant_names()[variant], name)
        assert run.level_count == len(cnt), (name, run.level_count, len(cnt))
        assert run.visited == int((lv != oracle.INF).sum())


@pytest.mark.parametrize("variant", ["edge-list", "vertex-push-blockreduce", "vertex-pull-warp-bulk",
                                     "frontier-push", "frontier-pull"])
def test_graph_loop(ctx, graphs, variant):
    for name, (h, g, r, lv, cnt) in graphs.items():
        run = bw.bfs(ctx, g, variant, r, loop="graph", stats=True)
        assert np.array_equal(run.levels.cpu().numpy(), lv), (variant, name)
        assert run.level_count == len(cnt)
        assert [s["frontier_vertices"] for s in run.level_stats] == list(cnt)


def test_level_statistics(ctx, graphs):
    h, g, r, lv, cnt = graphs["rmat14"]
    run = bw.bfs(ctx, g, "frontier-push", r, stats=True)
    deg = h.out_degrees().astype(np.int64)
    for L, s in enumerate(run.level_stats):
        new = lv == L + 1
        assert s["frontier_vertices"] == int(new.sum())
        assert s["frontier_edges"] == int(deg[new].sum())
        if new.any():
            l = np.log2(1.0 + deg[new])
            assert s["log_degree_max"] == pytest.approx(l.max(), rel=1e-3)
            assert s["log_degree_sum"] == pytest.approx(l.sum(), rel=1e-3)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_mixed_schedules(ctx, graphs, seed):
    rng = np.random.default_rng(seed)
    for name, (h, g, r, lv, cnt) in graphs.items():
        sched = rng.integers(0, 34, size=12).tolist()
        run = bw.bfs_schedule(ctx, g, sched, r)
        assert np.array_equal(run.levels.cpu().numpy(), lv), (name, sched)
        assert [s["frontier_vertices"] for s in run.level_stats] == list(cnt)


@pytest.mark.parametrize("fam", ["vertex-push-warp", "vertex-pull-warp"])
@pytest.mark.parametrize("w,c", [(1, 1), (2, 8), (4, 4), (8, 64), (16, 16), (32, 32), (32, 128)])
def test_warp_configs(ctx, graphs, fam, w, c):
    for name in ["rmat14", "grid", "star"]:
        h, g, r, lv, cnt = graphs[name]
        run = bw.bfs(ctx, g, fam, r, warp=w, chunk=c)
        assert np.array_equal(run.levels.cpu().numpy(), lv), (fam, w, c, name)


def test_launch_geometry_overrides(ctx, graphs):
    h, g, r, lv, cnt = graphs["er"]
    for v, blk, grd in [("edge-list-blockreduce", 64, 3), ("vertex-pull", 512, 1), ("vertex-push-bulk", 32, 7)]:
        run = bw.bfs(ctx, g, v, r, block=blk, grid=grd)
        assert np.array_equal(run.levels.cpu().numpy(), lv)


def test_level_api(ctx, graphs):
    """bw_bfs_init + bw_bfs_level, the reference's per-level host loop."""
    import torch
    lib = bw.library()
    h, g, r, lv, cnt = graphs["ba"]
    levels = torch.empty(h.vertex_count, dtype=torch.int32, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.bw_bfs_init(ctx.handle, h.vertex_count, r, C.c_void_p(levels.data_ptr()), st) == 0
    f = C.c_uint32()
    depth, seen = 0, []
    variants = [bw.bfs_variant_id(n) for n in ("vertex-push", "frontier-pull", "edge-list-warpreduce")]
    while True:
        rc = lib.bw_bfs_level(ctx.handle, C.byref(g.view), variants[depth % 3], C.c_void_p(levels.data_ptr()),
                              depth, None, C.byref(f), st)
        assert rc == 0
        seen.append(f.value)
        depth += 1
        if f.value == 0:
            break
    assert seen == list(cnt)
    assert np.array_equal(levels.cpu().numpy(), lv)


def test_errors(ctx, graphs):
    h, g, r, lv, cnt = graphs["chain"]
    with pytest.raises(bw.BwError) as e:
        bw.bfs(ctx, g, "vertex-push", r, max_levels=5)
    assert e.value.status == 6                         # BW_ERR_LEVEL_LIMIT
    with pytest.raises(bw.BwError) as e:
        bw.bfs(ctx, g, "vertex-push", r, loop="graph", max_levels=5)
    assert e.value.status == 6
    with pytest.raises(bw.BwError) as e:
        bw.bfs(ctx, g, "vertex-push", h.vertex_count)
    assert e.value.status == 1
    with pytest.raises(bw.BwError) as e:
        bw.bfs(ctx, g, "vertex-push-warp", r, warp=3)
    assert e.value.status == 1
    only_csr = bw.DeviceGraph(h, reps=bw.REP_FWD_CSR | bw.REP_REV_CSR)
    with pytest.raises(bw.BwError) as e:
        bw.bfs(ctx, only_csr, "struct-edge-list", r)
    assert e.value.status == 2                         # missing representation
    # the context stays usable after errors
    run = bw.bfs(ctx, g, "vertex-push", r)
    assert np.array_equal(run.levels.cpu().numpy(), lv)


def _two_stars(leaves):
    """Root 0 -> hubs 1 and 2 -> `leaves` leaves each, then every leaf ->
    one of 64 sinks: the frontier grows from 2 rows to 2 * leaves vertices
    in one level (more than one block of the cluster kernel lists) and
    shrinks again."""
    n = 3 + 2 * leaves + 64
    src = [0, 0]
    dst = [1, 2]
    for hub in (1, 2):
        base = 3 + (hub - 1) * leaves
        src += [hub] * leaves
        dst += list(range(base, base + leaves))
    lv = np.arange(3, 3 + 2 * leaves)
    src += list(lv)
    dst += list(3 + 2 * leaves + (lv % 64))
    return bw.HostGraph.from_edges(n, np.array(src, np.uint32), np.array(dst, np.uint32))


@pytest.mark.parametrize("leaves", [3000, 20000])
def test_cluster_path_overflow(ctx, leaves):
    """frontier-push's device loop keeps small frontiers in one cluster
    launch; a level that discovers more vertices than a block's list holds
    spills to the global queue and hands over to the full-GPU kernels.
    Depths and per-level counts match the oracle either way."""
    h = _two_stars(leaves)
    g = bw.DeviceGraph(h)
    want, cnt = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, 0)
    for loop in ("graph", "host"):
        run = bw.bfs(ctx, g, "frontier-push", 0, loop=loop, stats=True)
        assert np.array_equal(run.levels.cpu().numpy(), want), loop
        assert [s["frontier_vertices"] for s in run.level_stats] == list(cnt), loop


@pytest.mark.parametrize("variant", ["frontier-push", "frontier-pull", "edge-list-bulk", "vertex-pull-warp"])
@pytest.mark.parametrize("loop", ["host", "graph"])
def test_l2_window_leaves_depths_unchanged(ctx, graphs, variant, loop):
    """BW_LAUNCH_L2_WINDOW (the depth array persisting in L2): same depths."""
    import torch
    side = torch.cuda.Stream()                    # a window is an attribute of a created stream
    for name, (h, g, r, lv, cnt) in graphs.items():
        with torch.cuda.stream(side):
            run = bw.bfs(ctx, g, variant, r, loop=loop, l2_window=True)
            got = run.levels.cpu().numpy()
        assert np.array_equal(got, lv), (variant, name, loop)
    with pytest.raises(bw.BwError):               # the legacy default stream carries no window
        bw.bfs(ctx, graphs["rmat10"][1], variant, graphs["rmat10"][2], l2_window=True,
               stream=torch.cuda.default_stream())
