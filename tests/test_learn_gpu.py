"""Learned variant switching on the GPU: features, MLP forward/backward
against the float64 oracle, training, profiling, and the switched BFS
(bit-exact depths, device and host prediction)."""
import ctypes as C

import numpy as np
import pytest

import belewitte_gb300 as bw
import oracle
from belewitte_gb300 import learn
from oracle import mlp as mlp_oracle
from tests.graphs import catalog, root_of

pytestmark = pytest.mark.gpu
K = len(learn.CANDIDATES)


def _random_params(seed=3):
    rng = np.random.default_rng(seed)
    mu = rng.normal(size=12).astype(np.float32)
    sd = rng.uniform(0.5, 2.0, size=12).astype(np.float32)
    return learn.init_params(K, mu, sd, seed=seed)


def _data(n, seed=5):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, 12)).astype(np.float32) * 3
    T = rng.dirichlet(np.ones(K) * 0.3, size=n).astype(np.float32)
    W = rng.uniform(0.1, 3.0, size=n).astype(np.float32)
    return X, T, W


def test_forward_matches_oracle(ctx):
    p = _random_params()
    X, _, _ = _data(300)
    got = learn.predict(ctx, p, X, K)
    want, _ = mlp_oracle.forward(p.cpu().numpy(), X, K)
    assert np.abs(got - want).max() < 2e-5


def test_gradient_matches_oracle(ctx):
    """The hand-written backward pass against the float64 oracle."""
    p = _random_params(7)
    X, T, W = _data(257, seed=9)
    g, loss = learn.gradient(ctx, p, X, T, W)
    want_loss, want = mlp_oracle.loss_and_grad(p.cpu().numpy(), X, T, W, K)
    assert loss == pytest.approx(want_loss, rel=1e-4)
    scale = np.abs(want).max()
    assert np.abs(g - want).max() <= 1e-4 * scale + 1e-7
    # unweighted form
    g2, _ = learn.gradient(ctx, p, X, T, None)
    _, want2 = mlp_oracle.loss_and_grad(p.cpu().numpy(), X, T, None, K)
    assert np.abs(g2 - want2).max() <= 1e-4 * np.abs(want2).max() + 1e-7


def test_training_learns_separable_rule(ctx):
    """Labels that depend on two features: training must reach high accuracy."""
    rng = np.random.default_rng(1)
    X = rng.normal(size=(4000, 12)).astype(np.float32)
    cls = (X[:, 0] > 0).astype(int) * 2 + (X[:, 3] > 0.5).astype(int)
    T = np.zeros((len(X), K), np.float32)
    T[np.arange(len(X)), cls] = 1.0
    params, curve = learn.train(ctx, X, T, np.ones(len(X), np.float32), steps=3000, lr=3e-3)
    assert curve[-1] < curve[0] * 0.3
    acc = (learn.predict(ctx, params, X, K).argmax(1) == cls).mean()
    assert acc > 0.95


def test_features_host_equals_device(ctx):
    h = catalog()["rmat14"][0]()
    g = bw.DeviceGraph(h)
    r = h.max_out_degree_vertex()
    times, feats, levels = learn.profile_graph(ctx, g, r, sample_every=1)
    lv, cnt = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, r)
    assert np.array_equal(levels.cpu().numpy(), lv)
    assert len(times) == len(cnt)
    assert np.all(times > 0)
    # recompute features on the host from the oracle's levels
    deg = h.out_degrees().astype(np.float64)
    visited, ev = 1, deg[r]
    out = (C.c_float * 12)()
    for L in range(len(cnt)):
        front = lv == L
        lg = np.log2(1 + deg[front])
        bw.library().bw_bfs_features(int(front.sum()), int(deg[front].sum()), float(lg.sum()), float((lg * lg).sum()),
                                     float(lg.max()) if front.any() else 0.0, h.vertex_count, h.edge_count,
                                     visited, int(ev), L, out)
        assert np.allclose(np.array(out), feats[L], rtol=1e-4, atol=1e-4), L
        visited += int((lv == L + 1).sum())
        ev += deg[lv == L + 1].sum()


def _quick_predictor(ctx):
    """A predictor trained on a few small graphs (fast)."""
    recs = []
    for spec in learn.catalogue(8, seed=11, max_scale=15, max_side=600):
        g = spec.build()
        t, f, _ = learn.profile_graph(ctx, g, learn.pick_root(g, spec.seed))
        recs.append(learn.subsample_levels(t, f))
    X, T, W = learn.build_dataset(recs)
    params, _ = learn.train(ctx, X, T, W, steps=2000)
    return learn.Predictor(params, learn.CANDIDATES, learn.fallback_variant(recs), 0.3), recs


@pytest.mark.parametrize("loop", ["graph", "host"])
def test_learned_bfs_bitexact(ctx, loop):
    pred, _ = _quick_predictor(ctx)
    for name in ["rmat14", "grid", "ba", "er", "star", "tiny", "isolated"]:
        make, root = catalog()[name]
        h = make()
        g = bw.DeviceGraph(h)
        r = root_of(h, root)
        lv, cnt = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, r)
        run = learn.run_learned(ctx, g, pred, r, loop=loop)
        assert np.array_equal(run.levels.cpu().numpy(), lv), (name, loop)
        assert [s["frontier_vertices"] for s in run.level_stats] == list(cnt)
        allowed = {bw.bfs_variant_id(c) for c in learn.CANDIDATES}
        assert all(s["variant"] in allowed for s in run.level_stats)


def test_device_and_host_predictions_agree(ctx):
    pred, _ = _quick_predictor(ctx)
    h = catalog()["rmat14"][0]()
    g = bw.DeviceGraph(h)
    r = h.max_out_degree_vertex()
    a = learn.run_learned(ctx, g, pred, r, loop="graph", mlp_only=True)
    b = learn.run_learned(ctx, g, pred, r, loop="host")
    assert [s["variant"] for s in a.level_stats] == [s["variant"] for s in b.level_stats]


def test_learned_schedule_is_deterministic(ctx):
    """The level statistics are summed in fixed point, so every run on the
    same graph and root sees the same features and picks the same variant
    for every level, whichever order the threads added in."""
    pred = learn.load_predictor()
    for h in (bw.HostGraph.rmat(16, 16, seed=4, symmetrise=True), bw.HostGraph.barabasi_albert(60000, 4, seed=2)):
        g = bw.DeviceGraph(h)
        r = h.max_out_degree_vertex()
        # the device loop also sends cluster-sized frontiers to frontier-push,
        # which the host loop never does: each loop mode against itself
        for loop in ("graph", "host"):
            runs = [learn.run_learned(ctx, g, pred, r, loop=loop) for _ in range(3)]
            first = runs[0].level_stats
            for run in runs[1:]:
                assert [s["variant"] for s in run.level_stats] == [s["variant"] for s in first], loop
                assert [(s["log_degree_sum"], s["log_degree_sq_sum"]) for s in run.level_stats] == \
                    [(s["log_degree_sum"], s["log_degree_sq_sum"]) for s in first], loop


def test_cluster_sized_frontiers_run_frontier_push(ctx):
    """The device loop gives every level whose frontier the cluster kernel
    takes to frontier-push, and the MLP the rest; depths are unchanged."""
    pred = learn.load_predictor()
    fp = bw.bfs_variant_id("frontier-push")
    for name in ["grid", "rmat14", "chain"]:
        make, root = catalog()[name]
        h = make()
        g = bw.DeviceGraph(h)
        r = root_of(h, root)
        lv, cnt = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, r)
        run = learn.run_learned(ctx, g, pred, r, loop="graph")
        assert np.array_equal(run.levels.cpu().numpy(), lv), name
        deg = np.diff(h.fwd_vertices.astype(np.int64))
        frontier, fedges = 1, int(deg[r])
        for L, s in enumerate(run.level_stats):
            if frontier <= 32768 and fedges <= 65536:
                assert s["variant"] == fp, (name, L)
            frontier = int((lv == L + 1).sum())
            fedges = int(deg[lv == L + 1].sum())


def test_learned_graph_loop_without_level_log(ctx):
    """Without a level log the device loop's cluster kernel computes the
    statistics of a handed-over frontier at handover only; depths and the
    level count stay exact, on graphs whose frontiers outgrow the cluster
    kernel (R-MAT, BA) and on ones that stay in it (grid, chain)."""
    pred = learn.load_predictor()
    for name in ["rmat14", "rmat12_sym", "ba", "grid", "chain", "star"]:
        make, root = catalog()[name]
        h = make()
        g = bw.DeviceGraph(h)
        r = root_of(h, root)
        lv, cnt = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, r)
        for stats in (False, True):
            run = learn.run_learned(ctx, g, pred, r, loop="graph", stats=stats)
            assert np.array_equal(run.levels.cpu().numpy(), lv), (name, stats)
            assert run.level_count == len(cnt), (name, stats)


# ---------------------------------------------------------------------------
# PageRank: per-iteration variant choice
# ---------------------------------------------------------------------------
def _quick_pr_predictor(ctx):
    """A PageRank predictor trained on a few small graphs (fast)."""
    specs = learn.catalogue(8, seed=11, max_scale=15, max_side=600)
    recs = learn.collect_pagerank(ctx, specs, log=lambda *a: None)
    X, T, W = learn.build_dataset(recs)
    params, _ = learn.train(ctx, X, T, W, steps=1500)
    return learn.Predictor(params, learn.PR_CANDIDATES, learn.fallback_variant(recs), 0.3), recs


def test_pagerank_features_are_whole_graph_moments(ctx):
    h = catalog()["rmat14"][0]()
    g = bw.DeviceGraph(h)
    deg = np.diff(h.rev_vertices.astype(np.int64))
    l = np.log2(1.0 + deg)
    want = np.zeros(12, np.float32)
    lib = bw.library()
    for it in (0, 1, 7):
        f = learn.pagerank_features(ctx, g, it)
        x = (C.c_float * 12)()
        lib.bw_bfs_features(h.vertex_count, h.edge_count, float(l.sum()), float((l * l).sum()), float(l.max()),
                            h.vertex_count, h.edge_count, h.vertex_count, h.edge_count, min(it, 1), x)
        want[:] = np.frombuffer(x, np.float32)
        assert np.allclose(f, want, rtol=1e-4, atol=1e-5), (it, f, want)


def test_learned_pagerank_within_tolerance(ctx):
    """Ranks of the learned per-iteration schedule against the oracle of the
    div semantics: the same bar as every order-changing variant."""
    pred, _ = _quick_pr_predictor(ctx)
    allowed = set(learn.PR_CANDIDATES)
    for name in ["rmat14", "er", "grid", "ba", "star", "tiny", "isolated"]:
        h = catalog()[name][0]()
        g = bw.DeviceGraph(h)
        ref, _ = oracle.pagerank(oracle.PR_DIV, h.vertex_count, h.rev_vertices, h.rev_edges, 12)
        r64 = oracle.pagerank_f64(oracle.PR_DIV, h.vertex_count, h.rev_vertices, h.rev_edges, 12)
        for loop in ("host", "graph"):
            run, sched = learn.run_pagerank_learned(ctx, g, pred, 12, loop=loop)
            got = run.ranks.cpu().numpy().astype(np.float64)
            assert len(sched) == 12 and set(sched) <= allowed, sched
            assert float((np.abs(got - ref) / np.abs(ref)).max()) <= 1e-5, (name, loop)
            assert float((np.abs(got - r64) / np.abs(r64)).max()) <= 1e-4, (name, loop)


def test_learned_pagerank_choices_score(ctx):
    """On its recorded timings the trained network's schedule costs no more
    than the fixed fallback variant's (what the network adds to the plain
    method), and every schedule is scored against the oracle-best one."""
    pred, recs = _quick_pr_predictor(ctx)
    K = len(learn.PR_CANDIDATES)
    chosen = fallback = best = 0.0
    for times, feats in recs:
        probs = learn.predict(ctx, pred.params, feats, K)
        ch = learn.choose(probs, pred.fallback, pred.threshold)
        sc = learn.score_graph(times, ch)
        chosen += sc["chosen"]
        fallback += float(times[:, pred.fallback].sum())
        best += sc["oracle_best"]
    assert best <= chosen <= fallback * 1.02, (best, chosen, fallback)
