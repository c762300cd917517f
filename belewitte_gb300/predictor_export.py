"""Export a trained variant predictor as a predictor library in the
reference's format, so that kernel-runner's ``-a bfs|pagerank -k switch -m
FILE.so`` runs the learned switch through the plugin surface.

The reference's predictors are decision trees that benchmark-analysis writes
out as C++ and compiles (``src/Predictor/Raw.hs:56-139``). Each library
exports, unmangled and with C++ types:

- ``predictorName``;
- ``propNames``: property name -> storage that ``lookup`` reads;
- ``implNames``: (implementation name, id, index, warp, chunk) tuples;
- ``default_impl``;
- ``int32_t lookup()``: the index of the implementation for the next step.

This module writes the same symbols around the MLP. Its weights are embedded
as exact hexadecimal floats. ``lookup`` forms the 12 level features with
``bw_bfs_features`` and runs ``bw_mlp_predict_host``, both from
libbelewitte_gb300.so. A predictor library therefore picks exactly what
``bw_bfs_run_learned`` picks in its host loop (``BW_LOOP_HOST``).

The properties it reads are the BFS switch's step and graph properties:
``frontier abs``, ``visited abs``, ``frontier edges``,
``frontier log degree sum``, ``frontier log degree square sum``,
``frontier log degree max``, ``visited edges``, ``depth``, ``vertex count``
and ``edge count``.

The PageRank predictor (``algo="pagerank"``) picks once per run, as the
reference's PageRank switch does, from the PageRank switch's graph
properties ``vertex count``, ``edge count`` and the in-degree log moments
``in log degree sum``, ``in log degree square sum`` and
``in log degree max``; it evaluates the network at the steady-state
iteration's features (level 1).
"""
from __future__ import annotations

import subprocess
import tempfile
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
DEFAULT_NPZ = PKG / "data" / "bfs_predictor.npz"
DEFAULT_SO = PKG / "libbfs_mlp_predictor.so"
PAGERANK_NPZ = PKG / "data" / "pagerank_predictor.npz"
PAGERANK_SO = PKG / "libpagerank_mlp_predictor.so"

# property name -> slot of the predictor's property array
PROPERTIES = ["frontier abs", "frontier edges", "frontier log degree sum", "frontier log degree square sum",
              "frontier log degree max", "vertex count", "edge count", "visited abs", "visited edges", "depth"]
# PageRank's switch picks once per run from graph properties
# (pagerank/pagerank.cpp:98-100): the in-degree log moments its plugin
# publishes, and the counts
PAGERANK_PROPERTIES = ["vertex count", "edge count", "in log degree sum", "in log degree square sum",
                       "in log degree max"]


def _hex(v: float) -> str:
    return float(np.float32(v)).hex() + "f"


def predictor_source(params, candidates, fallback: int, threshold: float, name: str, algo: str = "bfs") -> str:
    """C++ source of a predictor library for these MLP parameters; algo
    "bfs" (per level) or "pagerank" (once per run, at the steady-state
    iteration's features)."""
    p = np.asarray(params, dtype=np.float32).ravel()
    K = len(candidates)
    if not 2 <= K <= 16:
        raise ValueError("a predictor has 2 to 16 candidates")
    if not 0 <= fallback < K:
        raise ValueError("fallback must index a candidate")
    props_list = PAGERANK_PROPERTIES if algo == "pagerank" else PROPERTIES
    slot = {n: i for i, n in enumerate(props_list)}
    props = "".join(f'    {{"{n}", std::ref(properties[{i}])}},\n' for n, i in slot.items())
    impls = "".join(f'    std::make_tuple(std::string("{c}"), int64_t({k}), size_t({k}), size_t(0), size_t(0)),\n'
                    for k, c in enumerate(candidates))
    rows = [", ".join(_hex(v) for v in p[i:i + 8]) for i in range(0, len(p), 8)]
    weights = ",\n    ".join(rows)
    what = "PageRank (one variant per run)" if algo == "pagerank" else "BFS (one variant per level)"
    return f'''// Generated by belewitte_gb300.predictor_export: learned {what}
// variant predictor ({K} candidates, {len(p)} parameters).
#include <cstdint>
#include <functional>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "belewitte_gb300.h"

extern "C" const char *predictorName;
extern "C" const char *predictorName = "{name}";

static double properties[{len(props_list)}];

extern "C" const std::map<std::string, std::reference_wrapper<double>> propNames;
extern "C" const std::map<std::string, std::reference_wrapper<double>> propNames = {{
{props}}};

extern "C" const int32_t default_impl;
extern "C" const int32_t default_impl = {int(fallback)};

extern "C" const std::vector<std::tuple<std::string, int64_t, size_t, size_t, size_t>> implNames;
extern "C" const std::vector<std::tuple<std::string, int64_t, size_t, size_t, size_t>> implNames = {{
{impls}}};

static const float params[{len(p)}] = {{
    {weights}
}};

extern "C" int32_t lookup();
extern "C" int32_t lookup()
{{
{_features(slot, algo)}
    float probs[{K}];
    if (bw_mlp_predict_host(params, {K}, x, 1, probs) != 0) return default_impl;
    int32_t best = 0;
    for (int32_t k = 1; k < {K}; k++)
        if (probs[k] > probs[best]) best = k;
    return probs[best] < {_hex(threshold)} ? default_impl : best;
}}
'''


def _features(slot, algo: str) -> str:
    """The lookup's feature computation (C++ statements filling x)."""
    if algo == "pagerank":
        # every vertex active, level 1: the steady-state iteration
        return f'''    const double n = properties[{slot["vertex count"]}], m = properties[{slot["edge count"]}];
    float x[BW_FEATURE_COUNT];
    bw_bfs_features(static_cast<uint64_t>(n), static_cast<uint64_t>(m),
                    static_cast<float>(properties[{slot["in log degree sum"]}]),
                    static_cast<float>(properties[{slot["in log degree square sum"]}]),
                    static_cast<float>(properties[{slot["in log degree max"]}]),
                    static_cast<uint64_t>(n), static_cast<uint64_t>(m), static_cast<uint64_t>(n),
                    static_cast<uint64_t>(m), 1u, x);'''
    return f'''    const double fv = properties[{slot["frontier abs"]}], fe = properties[{slot["frontier edges"]}];
    const double visited = properties[{slot["visited abs"]}] + fv;
    const double edges_visited = properties[{slot["visited edges"]}] + fe;
    float x[BW_FEATURE_COUNT];
    bw_bfs_features(static_cast<uint64_t>(fv), static_cast<uint64_t>(fe),
                    static_cast<float>(properties[{slot["frontier log degree sum"]}]),
                    static_cast<float>(properties[{slot["frontier log degree square sum"]}]),
                    static_cast<float>(properties[{slot["frontier log degree max"]}]),
                    static_cast<uint64_t>(properties[{slot["vertex count"]}]),
                    static_cast<uint64_t>(properties[{slot["edge count"]}]),
                    static_cast<uint64_t>(visited), static_cast<uint64_t>(edges_visited),
                    static_cast<uint32_t>(properties[{slot["depth"]}]), x);'''


def export_predictor(out=DEFAULT_SO, npz=DEFAULT_NPZ, name: str = "bfs-mlp", algo: str = "bfs") -> Path:
    """Compile the predictor in `npz` into the library `out`."""
    d = np.load(npz, allow_pickle=False)
    src = predictor_source(d["params"], [str(c) for c in d["candidates"]], int(d["fallback"]),
                           float(d["threshold"]), name, algo)
    out = Path(out)
    with tempfile.TemporaryDirectory() as tmp:
        cpp = Path(tmp) / "predictor.cpp"
        cpp.write_text(src)
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{PKG.parent / 'include'}", str(cpp),
               "-o", str(out), f"-L{PKG}", "-lbelewitte_gb300", f"-Wl,-rpath,{PKG}"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError("predictor build failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)
    return out
