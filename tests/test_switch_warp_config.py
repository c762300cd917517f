"""The switch honours the warp and chunk sizes of its predictor's
implementations.

A reference-format predictor library (benchmark-analysis
src/Predictor/Raw.hs:56-139) lists each implementation as (name, id, index,
warp, chunk); the reference's switch runs a picked warp kernel with that
warp and chunk size (setWarpConfig, ImplementationTemplate.hpp:806-816).
Here a fixed predictor that always picks vertex-pull-warp with w=8, c=64
drives kernel-runner's BFS and PageRank switch: the property log shows the
8/64 configuration for every step, and the results equal the oracle's.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import belewitte_gb300 as bw
import oracle
from belewitte_gb300 import build

PKG = Path(bw.__file__).resolve().parent

FIXED_PREDICTOR = r'''
#include <cstdint>
#include <functional>
#include <map>
#include <string>
#include <tuple>
#include <vector>
extern "C" const char *predictorName;
extern "C" const char *predictorName = "fixed-warp-8-64";
extern "C" const std::map<std::string, std::reference_wrapper<double>> propNames;
extern "C" const std::map<std::string, std::reference_wrapper<double>> propNames = {};
extern "C" const int32_t default_impl;
extern "C" const int32_t default_impl = 0;
extern "C" const std::vector<std::tuple<std::string, int64_t, size_t, size_t, size_t>> implNames;
extern "C" const std::vector<std::tuple<std::string, int64_t, size_t, size_t, size_t>> implNames = {
    {"edge-list", 11, 0, 32, 32},
    {"%(warp)s", 22, 1, 8, 64},
};
extern "C" int32_t lookup();
extern "C" int32_t lookup() { return 1; }
'''


def _predictor(tmp_path, warp_name):
    src = tmp_path / f"{warp_name}.cpp"
    so = tmp_path / f"lib{warp_name}-fixed.so"
    src.write_text(FIXED_PREDICTOR % {"warp": warp_name})
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", str(src), "-o", str(so)], check=True)
    return so


def _configs(log: Path):
    return [tuple(int(x) for x in ln.split(":")[1:]) for ln in log.read_text().splitlines()
            if ln.startswith("config:")]


@pytest.mark.gpu
def test_bfs_switch_runs_picked_warp_config(tmp_path):
    build.build_plugins()
    h = bw.HostGraph.rmat(13, 16, seed=6, symmetrise=True)
    graph = tmp_path / "g.graph"
    h.write(graph)
    root = h.max_out_degree_vertex()
    so = _predictor(tmp_path, "vertex-pull-warp")
    log = tmp_path / "props.log"
    out = subprocess.run([str(PKG / "kernel-runner"), "-L", str(PKG), "-a", "bfs", "-k", "switch", "-m", str(so),
                          "-l", str(log), "-r", str(root), "-o", str(tmp_path), str(graph)],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    want, counts = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, root)
    rows = np.loadtxt(tmp_path / "g.output", dtype=np.int64)
    assert np.array_equal(rows[:, 1], want.astype(np.int64))
    cfgs = _configs(log)
    # the first pick (step 0), then one per level that found vertices
    assert cfgs[0] == (0, 8, 64)
    assert all(c[1:] == (8, 64) for c in cfgs)
    preds = [ln for ln in log.read_text().splitlines() if ln.startswith("prediction:")]
    assert all(ln.endswith(":22") for ln in preds)


@pytest.mark.gpu
def test_pagerank_switch_runs_picked_warp_config(tmp_path):
    build.build_plugins()
    h = bw.HostGraph.rmat(12, 16, seed=2)
    graph = tmp_path / "p.graph"
    h.write(graph)
    so = _predictor(tmp_path, "vertex-pull-warp")
    log = tmp_path / "props.log"
    out = subprocess.run([str(PKG / "kernel-runner"), "-L", str(PKG), "-a", "pagerank", "-k", "switch", "-m",
                          str(so), "-l", str(log), "-i", "30", "--validate", "-o", str(tmp_path), str(graph)],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    assert _configs(log) == [(0, 8, 64)]
    ref, _ = oracle.pagerank(oracle.PR_DIV, h.vertex_count, h.rev_vertices, h.rev_edges, 30)
    got = np.loadtxt(tmp_path / "p.output", dtype=np.float64)[:, 1]
    # vertex-pull-warp adds with float atomics (<= 1e-5 from the reference);
    # the --validate output rounds to 7 significant digits
    assert float((np.abs(got - ref) / np.abs(ref)).max()) <= 1e-5 + 5e-7
