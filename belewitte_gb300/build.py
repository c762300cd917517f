"""Build recipe for the in-tree native libraries.

Compiles, in parallel, every translation unit of libbelewitte_gb300.so
(hand-written CUDA for sm_103a plus the host C++ graph substrate) and links
the shared library next to this file.  Used by ``__graft_entry__.build()``
and by the package import when the library is missing.  Also builds the C++
plugin libraries (``libbfskernel.so``, ``libpagerankkernel.so``), the
``kernel-runner`` driver from ``belewitte_gb300/plugin`` and the shipped BFS
predictor as a reference-format predictor library
(``libbfs_mlp_predictor.so``).
"""
from __future__ import annotations

import concurrent.futures as _cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
PLUGIN = PKG / "plugin"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
LIB = PKG / "libbelewitte_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["bw_context.cu", "bfs.cu", "bfs_edge.cu", "bfs_vertex.cu", "pagerank.cu", "bw_gen.cu", "bw_learn.cu", "bw_noalloc.cu", "bw_batch.cu", "bw_probe.cu", "bw_stats.cu"]
CXX_SOURCES = ["bw_graph.cpp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build belewitte_gb300")
    return cand


def _version() -> str:
    try:
        out = subprocess.run(["git", "-C", str(ROOT), "rev-parse", "--short", "HEAD"],
                             capture_output=True, text=True, timeout=10)
        if out.returncode == 0 and out.stdout.strip():
            return "belewitte-gb300-" + out.stdout.strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "belewitte-gb300-local"


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_core(force: bool = False, jobs: int | None = None) -> Path:
    """Compile and link libbelewitte_gb300.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    version = _version()
    steps = []
    objs = []
    for src in CUDA_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            steps.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                          f"-I{INCLUDE}", f"-DBW_VERSION_STRING=\"{version}\"",
                          "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            steps.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", f"-I{INCLUDE}",
                          "-c", str(CSRC / src), "-o", str(obj)])
    if steps:
        with _cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
            list(ex.map(_run, steps))
    if force or steps or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs),
              "-Xcompiler", "-fopenmp", "-lgomp"])
    return LIB


def build_plugins(force: bool = False) -> list[Path]:
    """Build the reference-compatible plugin libraries and kernel-runner.

    The framework (Algorithm, options, timers) is linked into kernel-runner
    and exported with -rdynamic; the plugin libraries resolve against it, so
    the timer registry and the implementation registry are shared.
    """
    if not PLUGIN.exists():
        return []
    cuda_inc = "/usr/local/cuda/include"
    common = ["g++", "-O2", "-std=c++17", "-fPIC", f"-I{INCLUDE}", f"-I{PLUGIN}", f"-I{cuda_inc}"]
    rt = [f"-L{PKG}", "-lbelewitte_gb300", f"-Wl,-rpath,{PKG}", "-Wl,-rpath,$ORIGIN",
          "-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64", "-ldl"]
    headers = list(PLUGIN.glob("*.hpp")) + list(INCLUDE.glob("*.h")) + [LIB]
    targets = [
        (PKG / "libbfskernel.so", [PLUGIN / "bfs_plugin.cpp"], ["-shared"]),
        (PKG / "libpagerankkernel.so", [PLUGIN / "pagerank_plugin.cpp"], ["-shared"]),
        (PKG / "kernel-runner", [PLUGIN / "kernel_runner.cpp", PLUGIN / "framework_core.cpp"], ["-rdynamic"]),
    ]
    steps, out = [], []
    for target, srcs, extra in targets:
        if force or _stale(target, srcs + headers):
            steps.append(common + extra + [*map(str, srcs), "-o", str(target)] + rt)
        out.append(target)
    with _cf.ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(_run, steps))
    # the shipped learned predictors as reference-format predictor libraries
    # (kernel-runner -a bfs|pagerank -k switch -m lib{bfs,pagerank}_mlp_predictor.so)
    import importlib.util
    spec = importlib.util.spec_from_file_location("_bw_predictor_export", PKG / "predictor_export.py")
    pe = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pe)
    for npz, so, name, algo in ((pe.DEFAULT_NPZ, pe.DEFAULT_SO, "bfs-mlp", "bfs"),
                                (pe.PAGERANK_NPZ, pe.PAGERANK_SO, "pagerank-mlp", "pagerank")):
        if npz.exists():
            if force or _stale(so, [npz, Path(pe.__file__), LIB] + list(INCLUDE.glob("*.h"))):
                pe.export_predictor(so, npz, name, algo)
            out.append(so)
    return out


def build_oracle(force: bool = False) -> Path:
    """Build the CPU oracle (test infrastructure) as oracle/liboracle.so."""
    src = ROOT / "oracle" / "oracle.c"
    lib = ROOT / "oracle" / "liboracle.so"
    if force or _stale(lib, [src, ROOT / "oracle" / "oracle.h"]):
        _run(["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              str(src), "-o", str(lib), "-lm"])
    return lib


def build_all(force: bool = False) -> None:
    build_core(force)
    build_plugins(force)
    build_oracle(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", LIB)
