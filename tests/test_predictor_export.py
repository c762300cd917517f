"""The learned predictor exported as a reference-format predictor library
(predictorName, propNames, implNames, default_impl, lookup;
benchmark-analysis src/Predictor/Raw.hs:56-139).

CPU: a small C++ driver loads the library the way kernel-runner's switch
does (dlopen, properties set through propNames, lookup()), and its picks are
checked against bw_mlp_predict_host on bw_bfs_features and against the
float64 numpy MLP.  GPU: kernel-runner -k switch -m with the library picks,
level by level, what bw_bfs_run_learned's host loop picks."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

import belewitte_gb300 as bw
from belewitte_gb300 import _abi, build, predictor_export as pe
from oracle import mlp as omlp

PKG = Path(bw.__file__).resolve().parent

DRIVER = r'''
#include <dlfcn.h>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <iostream>
#include <map>
#include <string>
#include <tuple>
#include <vector>
using props_t = std::map<std::string, std::reference_wrapper<double>>;
using impls_t = std::vector<std::tuple<std::string, int64_t, size_t, size_t, size_t>>;
int main(int argc, char **argv)
{
    void *h = dlopen(argv[1], RTLD_NOW);
    if (!h) { std::fprintf(stderr, "%s\n", dlerror()); return 2; }
    auto lookup = reinterpret_cast<int32_t (*)()>(dlsym(h, "lookup"));
    auto &props = *reinterpret_cast<props_t *>(dlsym(h, "propNames"));
    auto &impls = *reinterpret_cast<impls_t *>(dlsym(h, "implNames"));
    const int32_t def = *reinterpret_cast<int32_t *>(dlsym(h, "default_impl"));
    const char *name = *reinterpret_cast<const char **>(dlsym(h, "predictorName"));
    std::printf("name %s default %d\n", name, def);
    for (auto &t : impls) std::printf("impl %s %lld %zu\n", std::get<0>(t).c_str(), (long long)std::get<1>(t), std::get<2>(t));
    std::vector<std::string> order;
    for (int i = 2; i < argc; i++) order.push_back(argv[i]);
    for (;;) {
        std::vector<double> v(order.size());
        for (auto &x : v) if (!(std::cin >> x)) return 0;
        for (size_t i = 0; i < order.size(); i++) props.at(order[i]).get() = v[i];
        std::printf("pick %d\n", lookup());
    }
}
'''


@pytest.fixture(scope="module")
def predictor_so():
    build.build_core()
    build.build_plugins()
    assert pe.DEFAULT_SO.exists()
    return pe.DEFAULT_SO


def _driver(tmp_path):
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "driver"
    subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-o", str(exe), "-ldl"], check=True)
    return exe


def _samples(rng, count):
    """Property rows (PROPERTIES order) spanning small to large frontiers."""
    rows = []
    for _ in range(count):
        n = int(2 ** rng.uniform(10, 24))
        m = int(n * 2 ** rng.uniform(1, 6))
        visited = int(rng.integers(0, n))
        fv = int(rng.integers(1, max(2, n - visited)))
        deg = 2 ** rng.uniform(0, 8, size=min(fv, 64))
        ld = np.log2(1 + deg).astype(np.float32)
        scale = fv / len(ld)
        fe = int(min(m, deg.sum() * scale))
        vedges = int(rng.integers(0, max(1, m - fe)))
        rows.append([fv, fe, float(np.float32(ld.sum() * scale)), float(np.float32((ld * ld).sum() * scale)),
                     float(ld.max()), n, m, visited, vedges, int(rng.integers(0, 40))])
    return rows


def test_exported_lookup_matches_host_forward(predictor_so, tmp_path):
    d = np.load(pe.DEFAULT_NPZ, allow_pickle=False)
    params = d["params"].astype(np.float32)
    cands = [str(c) for c in d["candidates"]]
    K, fb, thr = len(cands), int(d["fallback"]), float(d["threshold"])
    exe = _driver(tmp_path)
    rows = _samples(np.random.default_rng(7), 400)
    text = "\n".join(" ".join(repr(float(x)) for x in r) for r in rows) + "\n"
    out = subprocess.run([str(exe), str(predictor_so), *pe.PROPERTIES], input=text, capture_output=True,
                         text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.splitlines()
    assert lines[0] == f"name bfs-mlp default {fb}"
    assert [ln.split()[1:] for ln in lines[1:1 + K]] == [[c, str(k), str(k)] for k, c in enumerate(cands)]
    picks = [int(ln.split()[1]) for ln in lines[1 + K:]]
    assert len(picks) == len(rows)

    lib = bw.library()
    cp = params.ctypes.data_as(C.POINTER(C.c_float))
    X = np.zeros((len(rows), 12), np.float32)
    for i, r in enumerate(rows):
        fv, fe, ls, lq, lm, n, m, vis, ve, depth = r
        x = (C.c_float * 12)()
        lib.bw_bfs_features(int(fv), int(fe), ls, lq, lm, int(n), int(m), int(vis + fv), int(ve + fe), int(depth), x)
        X[i] = np.frombuffer(x, np.float32)
    probs = np.zeros((len(rows), K), np.float32)
    _abi.check(lib.bw_mlp_predict_host(cp, K, X.ctypes.data_as(C.POINTER(C.c_float)), len(rows),
                                       probs.ctypes.data_as(C.POINTER(C.c_float))), "bw_mlp_predict_host")
    expect = [fb if p.max() < thr else int(p.argmax()) for p in probs]
    assert picks == expect
    # the host forward pass is the MLP: float64 numpy within float32 rounding
    ref, _ = omlp.forward(params.astype(np.float64), X.astype(np.float64), K)
    assert np.allclose(probs, ref, atol=2e-5)
    assert len(set(picks)) >= 2          # the samples exercise more than one choice


def test_predict_host_rejects_bad_arguments():
    lib = bw.library()
    x = (C.c_float * 12)()
    p = (C.c_float * 16)()
    assert lib.bw_mlp_predict_host(None, 4, x, 1, p) != 0
    assert lib.bw_mlp_predict_host(p, 1, x, 1, p) != 0
    assert lib.bw_mlp_predict_host(p, 17, x, 1, p) != 0


def test_exported_pagerank_lookup_matches_host_forward(predictor_so, tmp_path):
    """The PageRank predictor library picks what bw_mlp_predict_host picks
    on the steady-state iteration's features of the given graph moments."""
    d = np.load(pe.PAGERANK_NPZ, allow_pickle=False)
    params = d["params"].astype(np.float32)
    cands = [str(c) for c in d["candidates"]]
    K, fb, thr = len(cands), int(d["fallback"]), float(d["threshold"])
    exe = _driver(tmp_path)
    rng = np.random.default_rng(3)
    rows = []
    for _ in range(200):
        n = int(2 ** rng.uniform(10, 24))
        m = int(n * 2 ** rng.uniform(1, 5))
        mean = rng.uniform(0.5, 6.0)
        ls = n * mean
        lq = n * (mean * mean + rng.uniform(0.0, 4.0))
        rows.append([n, m, ls, lq, mean + rng.uniform(1.0, 14.0)])
    text = "\n".join(" ".join(repr(float(x)) for x in r) for r in rows) + "\n"
    out = subprocess.run([str(exe), str(pe.PAGERANK_SO), *pe.PAGERANK_PROPERTIES], input=text, capture_output=True,
                         text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.splitlines()
    assert lines[0] == f"name pagerank-mlp default {fb}"
    picks = [int(ln.split()[1]) for ln in lines[1 + K:]]
    lib = bw.library()
    cp = params.ctypes.data_as(C.POINTER(C.c_float))
    expect = []
    for n, m, ls, lq, lm in rows:
        x = (C.c_float * 12)()
        lib.bw_bfs_features(int(n), int(m), ls, lq, lm, int(n), int(m), int(n), int(m), 1, x)
        p = (C.c_float * K)()
        _abi.check(lib.bw_mlp_predict_host(cp, K, x, 1, p), "bw_mlp_predict_host")
        p = np.frombuffer(p, np.float32)
        expect.append(fb if p.max() < thr else int(p.argmax()))
    assert picks == expect


@pytest.mark.gpu
def test_kernel_runner_pagerank_switch_with_exported_predictor(predictor_so, tmp_path):
    """kernel-runner -a pagerank -k switch -m libpagerank_mlp_predictor.so:
    ranks within the order-changing variants' tolerance, and the variant
    the learned run chooses for its steady-state iterations."""
    from belewitte_gb300 import learn
    import oracle
    for name, h in (("rmat", bw.HostGraph.rmat(14, 16, seed=9)), ("grid", bw.HostGraph.grid(300, 300))):
        p = tmp_path / f"{name}.graph"
        h.write(p)
        log = tmp_path / f"{name}.log"
        runner = PKG / "kernel-runner"
        out = subprocess.run([str(runner), "-L", str(PKG), "-a", "pagerank", "-k", "switch", "-m",
                              str(pe.PAGERANK_SO), "-l", str(log), "-i", "30", "--validate", "-o", str(tmp_path),
                              str(p)], capture_output=True, text=True, timeout=600)
        assert out.returncode == 0, out.stderr
        preds = [int(ln.split(":")[2]) for ln in log.read_text().splitlines() if ln.startswith("prediction:")]
        assert len(preds) == 1
        pred = learn.load_pagerank_predictor()
        run, sched = learn.run_pagerank_learned(ctx_of(), bw.DeviceGraph(h), pred, 30)
        assert pred.candidates[preds[0]] == sched[1], (name, pred.candidates[preds[0]], sched)
        ref, _ = oracle.pagerank(oracle.PR_DIV, h.vertex_count, h.rev_vertices, h.rev_edges, 30)
        got = np.loadtxt(tmp_path / f"{name}.output", dtype=np.float64)[:, 1]
        # the schedule may pick float-atomic variants (<= 1e-5 from the
        # reference); the --validate output rounds to 7 significant digits
        assert float((np.abs(got - ref) / np.abs(ref)).max()) <= 1e-5 + 5e-7, name


def ctx_of():
    return bw.Context()


@pytest.mark.gpu
def test_kernel_runner_switch_with_exported_predictor(predictor_so, tmp_path):
    import torch
    from belewitte_gb300 import learn
    import oracle
    h = bw.HostGraph.rmat(14, 16, seed=9, symmetrise=True)
    p = tmp_path / "g.graph"
    h.write(p)
    root = h.max_out_degree_vertex()
    log = tmp_path / "props.log"
    runner = PKG / "kernel-runner"
    out = subprocess.run([str(runner), "-L", str(PKG), "-a", "bfs", "-k", "switch", "-m", str(predictor_so),
                          "-l", str(log), "-r", str(root), "-o", str(tmp_path), str(p)],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lv, _ = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, root)
    rows = np.loadtxt(tmp_path / "g.output", dtype=np.int64)
    assert np.array_equal(rows[:, 1], lv.astype(np.int64))
    preds = {}
    for line in log.read_text().splitlines():
        if line.startswith("prediction:"):
            _, step, pid = line.split(":")
            preds[int(step)] = int(pid)
    ctx = bw.Context()
    g = bw.DeviceGraph(h)
    pred = learn.load_predictor()
    run = learn.run_learned(ctx, g, pred, root, loop="host")
    ids = [bw.bfs_variant_id(c) for c in pred.candidates]
    chosen = [ids.index(s["variant"]) for s in run.level_stats]
    got = [preds[L] for L in range(len(chosen))]
    # The level statistics are fixed-point sums (the same whatever order the
    # threads added in), the switch and the exported library both form the
    # features from them rounded to single precision, and both run the same
    # host network: every level's choice agrees.
    assert got == chosen, (got, chosen)
    torch.cuda.synchronize()
