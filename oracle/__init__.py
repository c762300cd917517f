"""Python access to the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``, always as the checker or the timed CPU
baseline, never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
PR_DIV, PR_NODIV = 0, 1
INF = 2147483647

_lib = None


class OrGraph(C.Structure):
    _fields_ = [("n", C.c_uint64), ("m", C.c_uint64),
                ("fwd_off", C.POINTER(C.c_uint32)), ("fwd_edges", C.POINTER(C.c_uint32)),
                ("rev_off", C.POINTER(C.c_uint32)), ("rev_edges", C.POINTER(C.c_uint32))]


def build(force: bool = False) -> Path:
    src, hdr = HERE / "oracle.c", HERE / "oracle.h"
    if force or not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        subprocess.run(["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                        str(src), "-o", str(LIB), "-lm"], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(str(LIB))
        u32p, i32p = C.POINTER(C.c_uint32), C.POINTER(C.c_int32)
        f32p, f64p = C.POINTER(C.c_float), C.POINTER(C.c_double)
        l.or_bfs.restype = C.c_int64
        l.or_bfs.argtypes = [C.c_uint64, u32p, u32p, C.c_uint32, i32p, u32p, C.c_uint64]
        l.or_bfs_parallel.restype = C.c_int64
        l.or_bfs_parallel.argtypes = [C.c_uint64, u32p, u32p, C.c_uint32, i32p, C.c_int]
        l.or_out_degrees.restype = None
        l.or_out_degrees.argtypes = [C.c_uint64, u32p, u32p, u32p]
        l.or_pagerank.restype = None
        l.or_pagerank.argtypes = [C.c_int, C.c_uint64, u32p, u32p, u32p, C.c_uint32, f32p, f64p]
        l.or_pagerank_f64.restype = None
        l.or_pagerank_f64.argtypes = [C.c_int, C.c_uint64, u32p, u32p, u32p, C.c_uint32, f64p]
        l.or_pagerank_parallel.restype = None
        l.or_pagerank_parallel.argtypes = [C.c_uint64, u32p, u32p, u32p, C.c_uint32, f32p, C.c_int]
        l.or_generate_rmat.restype = C.c_int
        l.or_generate_rmat.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                       C.c_int, C.POINTER(OrGraph)]
        l.or_graph_free.restype = None
        l.or_graph_free.argtypes = [C.POINTER(OrGraph)]
        l.or_format_rank.restype = C.c_int
        l.or_format_rank.argtypes = [C.c_float, C.c_char_p, C.c_int]
        _lib = l
    return _lib


def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(C.POINTER(C.c_uint32))


def bfs(n, off, edges, root, max_levels=None):
    """Exact BFS depths (int32, INF unreached) and per-level visit counts."""
    off, po = _u32(off)
    edges, pe = _u32(edges if len(edges) else np.zeros(1, np.uint32))
    levels = np.empty(n, dtype=np.int32)
    counts = np.zeros(n + 2, dtype=np.uint32)
    r = lib().or_bfs(n, po, pe, root, levels.ctypes.data_as(C.POINTER(C.c_int32)),
                     counts.ctypes.data_as(C.POINTER(C.c_uint32)), max_levels or (n + 2))
    if r < 0:
        raise RuntimeError("oracle BFS hit the level cap")
    return levels, counts[:r].copy()


def bfs_parallel(n, off, edges, root, threads=0):
    off, po = _u32(off)
    edges, pe = _u32(edges if len(edges) else np.zeros(1, np.uint32))
    levels = np.empty(n, dtype=np.int32)
    lv = lib().or_bfs_parallel(n, po, pe, root, levels.ctypes.data_as(C.POINTER(C.c_int32)), threads)
    return levels, lv


def out_degrees(n, rev_off, rev_edges):
    ro, pro = _u32(rev_off)
    re, pre = _u32(rev_edges if len(rev_edges) else np.zeros(1, np.uint32))
    deg = np.empty(n, dtype=np.uint32)
    lib().or_out_degrees(n, pro, pre, deg.ctypes.data_as(C.POINTER(C.c_uint32)))
    return deg


def pagerank(semantics, n, rev_off, rev_edges, iterations, deg=None):
    """FP32 PageRank with the reference arithmetic; returns (ranks, diffs)."""
    ro, pro = _u32(rev_off)
    re, pre = _u32(rev_edges if len(rev_edges) else np.zeros(1, np.uint32))
    if deg is None:
        deg = out_degrees(n, rev_off, rev_edges)
    deg, pd = _u32(deg)
    pr = np.empty(n, dtype=np.float32)
    diffs = np.zeros(max(iterations, 1), dtype=np.float64)
    lib().or_pagerank(semantics, n, pro, pre, pd, iterations, pr.ctypes.data_as(C.POINTER(C.c_float)),
                      diffs.ctypes.data_as(C.POINTER(C.c_double)))
    return pr, diffs[:iterations]


def pagerank_f64(semantics, n, rev_off, rev_edges, iterations, deg=None):
    ro, pro = _u32(rev_off)
    re, pre = _u32(rev_edges if len(rev_edges) else np.zeros(1, np.uint32))
    if deg is None:
        deg = out_degrees(n, rev_off, rev_edges)
    deg, pd = _u32(deg)
    pr = np.empty(n, dtype=np.float64)
    lib().or_pagerank_f64(semantics, n, pro, pre, pd, iterations, pr.ctypes.data_as(C.POINTER(C.c_double)))
    return pr


def pagerank_parallel(n, rev_off, rev_edges, iterations, deg=None, threads=0):
    ro, pro = _u32(rev_off)
    re, pre = _u32(rev_edges if len(rev_edges) else np.zeros(1, np.uint32))
    if deg is None:
        deg = out_degrees(n, rev_off, rev_edges)
    deg, pd = _u32(deg)
    pr = np.empty(n, dtype=np.float32)
    lib().or_pagerank_parallel(n, pro, pre, pd, iterations, pr.ctypes.data_as(C.POINTER(C.c_float)), threads)
    return pr


def generate_rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, symmetrise=False) -> dict:
    """The library's seeded R-MAT graph, made here without the library:
    {"fwd_vertices", "fwd_edges", "rev_vertices", "rev_edges"} (uint32)."""
    g = OrGraph()
    if lib().or_generate_rmat(scale, edge_factor, a, b, c, seed, int(symmetrise), C.byref(g)) != 0:
        raise MemoryError("or_generate_rmat failed")
    try:
        n, m = int(g.n), int(g.m)

        def grab(ptr, count):
            return np.ctypeslib.as_array(ptr, shape=(count,)).copy() if count else np.zeros(0, np.uint32)
        out = {"fwd_vertices": grab(g.fwd_off, n + 1), "fwd_edges": grab(g.fwd_edges, m)}
        if symmetrise:
            out["rev_vertices"], out["rev_edges"] = out["fwd_vertices"], out["fwd_edges"]
        else:
            out["rev_vertices"], out["rev_edges"] = grab(g.rev_off, n + 1), grab(g.rev_edges, m)
        return out
    finally:
        lib().or_graph_free(C.byref(g))


def format_rank(value: float) -> str:
    buf = C.create_string_buffer(64)
    lib().or_format_rank(float(value), buf, 64)
    return buf.value.decode()


def build_ref(reference_root: str | None = None, force: bool = False) -> list[Path]:
    """Compile the reference's CUDA kernels, unmodified, into cubins under
    oracle/_ref/ (the parity pin run by oracle/ref_runner.py).  Only runs
    where the reference tree exists; elsewhere the prebuilt cubins are used.

    The tree is `reference_root`, else the BELEWITTE_REFERENCE environment
    variable; with neither, nothing is compiled.
    """
    reference_root = reference_root or os.environ.get("BELEWITTE_REFERENCE", "")
    if not reference_root:
        out_dir = HERE / "_ref"
        return sorted(out_dir.glob("*.cubin")) if out_dir.exists() else []
    root = Path(reference_root)
    out_dir = HERE / "_ref"
    units = {"ref_bfs": "ref_bfs_unity.cu", "ref_pagerank": "ref_pagerank_unity.cu",
             "ref_pagerank_pull_warp": "ref_pagerank_pull_warp_unity.cu"}
    built = []
    if not root.exists():
        return [out_dir / f"{k}.cubin" for k in units if (out_dir / f"{k}.cubin").exists()]
    out_dir.mkdir(exist_ok=True)
    for key, unit in units.items():
        target = out_dir / f"{key}.cubin"
        if force or not target.exists() or target.stat().st_mtime < (HERE / unit).stat().st_mtime:
            subprocess.run(["nvcc", "-std=c++17", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                            "-O3", f"-I{root}", "-o", str(target), str(HERE / unit)], check=True,
                           capture_output=True)
        built.append(target)
    return built
