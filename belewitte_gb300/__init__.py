"""belewitte_gb300 -- GB300 (sm_103a) BFS and PageRank kernel libraries.

Python host mirror of the reference's kernel-runner plugin surface for the
BFS and PageRank algorithms.  All compute goes through the C ABI of
``libbelewitte_gb300.so`` (include/belewitte_gb300.h); PyTorch is used only
to own device memory and streams.  There is no CPU fallback: every entry
point that computes raises when the CUDA library cannot run.

Reference surface mirrored here:
  * implementation names   bfs/bfs.cpp:121-223, pagerank/pagerank.cpp:205-357
  * graph representations  GraphLoader.hpp:123-211 (CSR, reverse CSR,
                           EdgeList, StructEdgeList, forward and reverse)
  * BFS result             int32 depth per vertex, INT_MAX when unreached
                           (bfs/bfs.cpp:69-117)
  * PageRank result        float32 rank per vertex after a fixed number of
                           iterations (pagerank/pagerank.cpp:74-131)
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Iterable, Sequence

import numpy as np

from . import _abi
from ._abi import BwError, check

__all__ = [
    "HostGraph", "DeviceGraph", "Context", "BfsRun", "PageRankRun",
    "bfs_variant_names", "pagerank_variant_names", "bfs_variant_id", "pagerank_variant_id",
    "BwError", "INF", "compute_division", "library",
]

INF = 2147483647
REP_FWD_CSR, REP_REV_CSR, REP_FWD_EL, REP_REV_EL, REP_FWD_ST, REP_REV_ST = 1, 2, 4, 8, 16, 32


def library() -> C.CDLL:
    return _abi.load()


def bfs_variant_names() -> list[str]:
    lib = library()
    return [lib.bw_bfs_variant_name(i).decode() for i in range(lib.bw_bfs_variant_count())]


def pagerank_variant_names() -> list[str]:
    lib = library()
    return [lib.bw_pagerank_variant_name(i).decode() for i in range(lib.bw_pagerank_variant_count())]


def bfs_variant_id(name: str | int) -> int:
    if isinstance(name, int):
        return name
    v = library().bw_bfs_variant_lookup(name.encode())
    if v < 0:
        raise KeyError(f'No kernel named "{name}" exists!')
    return v


def pagerank_variant_id(name: str | int) -> int:
    if isinstance(name, int):
        return name
    v = library().bw_pagerank_variant_lookup(name.encode())
    if v < 0:
        raise KeyError(f'No kernel named "{name}" exists!')
    return v


def compute_division(count: int, sm_count: int, max_threads: int = 1024) -> tuple[int, int]:
    """Reference Backend::computeDivision (Backend.cpp:52-70): (block, grid)."""
    b, g = C.c_uint32(), C.c_uint32()
    library().bw_compute_division(count, sm_count, max_threads, C.byref(b), C.byref(g))
    return b.value, g.value


# ---------------------------------------------------------------------------
# Host graphs
# ---------------------------------------------------------------------------
class HostGraph:
    """Forward + reverse CSR on the host (uint32), owned by the C library."""

    def __init__(self, raw: _abi.HostGraphC):
        self._raw = raw
        n, m = raw.vertex_count, raw.edge_count
        self.vertex_count = int(n)
        self.edge_count = int(m)
        self.undirected = bool(raw.undirected)

        def view(ptr, count):
            if count == 0:
                return np.zeros(0, dtype=np.uint32)
            return np.ctypeslib.as_array(ptr, shape=(count,))
        self.fwd_vertices = view(raw.fwd_vertices, n + 1)
        self.fwd_edges = view(raw.fwd_edges, m)
        self.rev_vertices = view(raw.rev_vertices, n + 1)
        self.rev_edges = view(raw.rev_edges, m)

    def __del__(self):
        raw = getattr(self, "_raw", None)
        if raw is not None and _abi._lib is not None:
            _abi._lib.bw_host_graph_free(C.byref(raw))
            self._raw = None

    # -- construction ------------------------------------------------------
    @staticmethod
    def _make(fn, *args, what: str) -> "HostGraph":
        raw = _abi.HostGraphC()
        check(fn(*args, C.byref(raw)), what)
        return HostGraph(raw)

    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
             c: float = 0.19, seed: int = 1, symmetrise: bool = False) -> "HostGraph":
        return cls._make(library().bw_generate_rmat, scale, edge_factor, a, b, c, seed,
                         int(symmetrise), what="bw_generate_rmat")

    @classmethod
    def rmat_n(cls, n: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
               c: float = 0.19, seed: int = 1, symmetrise: bool = False) -> "HostGraph":
        """R-MAT over `n` vertices (any n >= 2; bw_generate_rmat_n)."""
        return cls._make(library().bw_generate_rmat_n, n, edge_factor, a, b, c, seed,
                         int(symmetrise), what="bw_generate_rmat_n")

    @classmethod
    def erdos_renyi(cls, n: int, m: int, seed: int = 1, symmetrise: bool = False) -> "HostGraph":
        return cls._make(library().bw_generate_er, n, m, seed, int(symmetrise), what="bw_generate_er")

    @classmethod
    def grid(cls, h: int, w: int) -> "HostGraph":
        return cls._make(library().bw_generate_grid, h, w, what="bw_generate_grid")

    @classmethod
    def barabasi_albert(cls, n: int, m: int, seed: int = 1) -> "HostGraph":
        return cls._make(library().bw_generate_ba, n, m, seed, what="bw_generate_ba")

    @classmethod
    def from_edges(cls, vertex_count: int, src: Sequence[int], dst: Sequence[int],
                   dedupe: bool = True, drop_self_loops: bool = True,
                   symmetrise: bool = False) -> "HostGraph":
        s = np.ascontiguousarray(np.asarray(src, dtype=np.uint32))
        d = np.ascontiguousarray(np.asarray(dst, dtype=np.uint32))
        if s.shape != d.shape:
            raise ValueError("src and dst differ in length")
        flags = (1 if drop_self_loops else 0) | (2 if dedupe else 0) | (4 if symmetrise else 0)
        return cls._make(library().bw_graph_from_edges, vertex_count, s.size,
                         s.ctypes.data_as(_abi.u32p), d.ctypes.data_as(_abi.u32p), flags,
                         what="bw_graph_from_edges")

    @classmethod
    def read(cls, path: str) -> "HostGraph":
        """Read a reference .graph file (utils/Graph.hpp format v0/v1)."""
        return cls._make(library().bw_graph_file_read, str(path).encode(), what=f"read {path}")

    def write(self, path: str) -> None:
        check(library().bw_graph_file_write(str(path).encode(), C.byref(self._raw)), f"write {path}")

    # -- queries -----------------------------------------------------------
    def out_degrees(self) -> np.ndarray:
        return np.diff(self.fwd_vertices.astype(np.int64)).astype(np.uint32)

    def degree_statistics(self, kind: str = "out") -> dict[str, float]:
        """graph-details statistics (graph-details.cpp:36-61)."""
        k = {"abs": 0, "in": 1, "out": 2}[kind]
        out = (C.c_double * 7)()
        check(library().bw_degree_statistics(C.byref(self._raw), k, out), "bw_degree_statistics")
        keys = ["min", "lower", "mean", "median", "upper", "max", "stddev"]
        return dict(zip(keys, list(out)))

    def max_out_degree_vertex(self) -> int:
        return int(np.argmax(self.out_degrees())) if self.vertex_count else 0


# ---------------------------------------------------------------------------
# Device side
# ---------------------------------------------------------------------------
def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("belewitte_gb300 needs a CUDA device (no CPU fallback)")
    return torch


def _ptr(t) -> int:
    return 0 if t is None else int(t.data_ptr())


class Context:
    """A device context (scratch, events); replaces CUDABackend::setDevice."""

    def __init__(self, device: int = 0):
        _torch()
        self._lib = library()
        h = C.c_void_p()
        check(self._lib.bw_context_create(device, C.byref(h)), "bw_context_create")
        self.handle = h
        self.device = device
        self.sm_count = self._lib.bw_context_sm_count(h)

    def close(self) -> None:
        if self.handle:
            self._lib.bw_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _CudaArray:
    """Zero-copy __cuda_array_interface__ view of library-owned memory."""

    def __init__(self, ptr: int, count: int, typestr: str = "<i4"):
        self.__cuda_array_interface__ = {"shape": (max(count, 1),), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3}


class DeviceGraph:
    """A graph resident in HBM in the representations the variants read.

    Built from a HostGraph (uploaded) or generated directly on the device
    (``DeviceGraph.generate``).  ``reps`` selects which derived arrays to
    build (REP_* bit mask); reverse arrays alias the forward ones for
    undirected graphs.
    """

    def __init__(self, host: HostGraph | None = None, device: int = 0, reps: int = 63, stream=None,
                 _dev: "_abi.DeviceGraphC | None" = None):
        torch = _torch()
        self.host = host
        self._dev = _dev
        dev = torch.device("cuda", device)
        self.device = dev
        lib = library()
        st = stream or torch.cuda.current_stream(dev)
        sp = C.c_void_p(st.cuda_stream)
        if host is not None:
            self.vertex_count, self.edge_count, self.undirected = host.vertex_count, host.edge_count, host.undirected

            def up(a):
                a = np.ascontiguousarray(a)
                if a.size == 0:
                    return torch.zeros(1, dtype=torch.int32, device=dev)
                return torch.from_numpy(a.view(np.int32)).to(dev)
            self.fwd_vertices = up(host.fwd_vertices)
            self.fwd_edges = up(host.fwd_edges)
            if host.undirected:
                self.rev_vertices, self.rev_edges = self.fwd_vertices, self.fwd_edges
            else:
                self.rev_vertices = up(host.rev_vertices)
                self.rev_edges = up(host.rev_edges)
        else:
            d = _dev
            self.vertex_count, self.edge_count, self.undirected = int(d.vertex_count), int(d.edge_count), bool(d.undirected)
            n, m = self.vertex_count, self.edge_count
            self.fwd_vertices = torch.as_tensor(_CudaArray(d.fwd_vertices, n + 1), device=dev)
            self.fwd_edges = torch.as_tensor(_CudaArray(d.fwd_edges, m), device=dev)
            self.rev_vertices = torch.as_tensor(_CudaArray(d.rev_vertices, n + 1), device=dev)
            self.rev_edges = torch.as_tensor(_CudaArray(d.rev_edges, m), device=dev)
        m = max(self.edge_count, 1)
        self.fwd_in_edges = self.rev_in_edges = None
        self.fwd_struct = self.rev_struct = None
        if reps & (REP_FWD_EL | REP_FWD_ST):
            self.fwd_in_edges = torch.empty(m, dtype=torch.int32, device=dev)
            check(lib.bw_expand_edge_list(_ptr(self.fwd_vertices), self.vertex_count, self.edge_count,
                                          _ptr(self.fwd_in_edges), sp), "bw_expand_edge_list")
        if reps & (REP_REV_EL | REP_REV_ST):
            if self.undirected and self.fwd_in_edges is not None:
                self.rev_in_edges = self.fwd_in_edges
            else:
                self.rev_in_edges = torch.empty(m, dtype=torch.int32, device=dev)
                check(lib.bw_expand_edge_list(_ptr(self.rev_vertices), self.vertex_count, self.edge_count,
                                              _ptr(self.rev_in_edges), sp), "bw_expand_edge_list")
        if reps & REP_FWD_ST:
            self.fwd_struct = torch.empty(2 * m, dtype=torch.int32, device=dev)
            check(lib.bw_build_struct_edges(_ptr(self.fwd_in_edges), _ptr(self.fwd_edges), self.edge_count,
                                            _ptr(self.fwd_struct), sp), "bw_build_struct_edges")
        if reps & REP_REV_ST:
            if self.undirected and self.fwd_struct is not None:
                self.rev_struct = self.fwd_struct
            else:
                self.rev_struct = torch.empty(2 * m, dtype=torch.int32, device=dev)
                check(lib.bw_build_struct_edges(_ptr(self.rev_in_edges), _ptr(self.rev_edges), self.edge_count,
                                                _ptr(self.rev_struct), sp), "bw_build_struct_edges")
        st.synchronize()
        self.reps = reps
        self.view = _abi.GraphView(
            self.vertex_count, self.edge_count,
            _ptr(self.fwd_vertices), _ptr(self.fwd_edges), _ptr(self.rev_vertices), _ptr(self.rev_edges),
            _ptr(self.fwd_in_edges) if reps & REP_FWD_EL else 0,
            _ptr(self.rev_in_edges) if reps & REP_REV_EL else 0,
            _ptr(self.fwd_struct), _ptr(self.rev_struct))

    @classmethod
    def generate(cls, kind: str, *, scale: int = 0, edge_factor: int = 16, n: int = 0, m: int = 0,
                 h: int = 0, w: int = 0, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 1,
                 symmetrise: bool = False, device: int = 0, reps: int = REP_FWD_CSR | REP_REV_CSR,
                 stream=None) -> "DeviceGraph":
        """Generate on the GPU; identical to the HostGraph generator of the same kind."""
        torch = _torch()
        dev = torch.device("cuda", device)
        st = stream or torch.cuda.current_stream(dev)
        kinds = {"rmat": (0, scale, edge_factor), "er": (1, n, m), "grid": (2, h, w), "ba": (3, n, m),
                 "rmat_n": (4, n, edge_factor)}
        k, p0, p1 = kinds[kind]
        raw = _abi.DeviceGraphC()
        check(library().bw_generate_device(k, p0, p1, a, b, c, seed, int(symmetrise), C.byref(raw),
                                           C.c_void_p(st.cuda_stream)), f"generate {kind}")
        return cls(None, device=device, reps=reps, stream=st, _dev=raw)

    def __del__(self):
        raw = getattr(self, "_dev", None)
        if raw is not None and _abi._lib is not None:
            try:
                import torch
                torch.cuda.synchronize()
            except Exception:
                pass
            _abi._lib.bw_device_graph_free(C.byref(raw))
            self._dev = None

    def degree_statistics(self, ctx: "Context", kind: str = "out", stream=None) -> dict[str, float]:
        """graph-details statistics (graph-details.cpp:36-61) computed on the
        device (bw_degree_statistics_device)."""
        torch = _torch()
        k = {"abs": 0, "in": 1, "out": 2}[kind]
        out = (C.c_double * 7)()
        st = stream or torch.cuda.current_stream(self.device)
        check(library().bw_degree_statistics_device(ctx.handle, C.byref(self.view), int(self.undirected), k, out,
                                                    C.c_void_p(st.cuda_stream)), "bw_degree_statistics_device")
        keys = ["min", "lower", "mean", "median", "upper", "max", "stddev"]
        return dict(zip(keys, list(out)))

    def to_host_arrays(self) -> dict:
        """Copy the forward and reverse CSR back to numpy (uint32)."""
        n, m = self.vertex_count, self.edge_count
        out = {"fwd_vertices": self.fwd_vertices[: n + 1].cpu().numpy().view(np.uint32),
               "fwd_edges": self.fwd_edges[:m].cpu().numpy().view(np.uint32)}
        if self.undirected:
            out["rev_vertices"], out["rev_edges"] = out["fwd_vertices"], out["fwd_edges"]
        else:
            out["rev_vertices"] = self.rev_vertices[: n + 1].cpu().numpy().view(np.uint32)
            out["rev_edges"] = self.rev_edges[:m].cpu().numpy().view(np.uint32)
        return out

    def nbytes(self) -> int:
        seen, total = set(), 0
        for t in (self.fwd_vertices, self.fwd_edges, self.rev_vertices, self.rev_edges,
                  self.fwd_in_edges, self.rev_in_edges, self.fwd_struct, self.rev_struct):
            if t is not None and t.data_ptr() not in seen:
                seen.add(t.data_ptr())
                total += t.numel() * t.element_size()
        return total


@dataclass
class BfsRun:
    levels: object            # torch.int32 tensor (device)
    level_count: int
    visited: int
    traversed_edges: int
    device_ms: float
    level_stats: list = field(default_factory=list)

    @property
    def gteps(self) -> float:
        return self.traversed_edges / (self.device_ms * 1e-3) / 1e9 if self.device_ms > 0 else 0.0


@dataclass
class PageRankRun:
    ranks: object             # torch.float32 tensor (device)
    iterations: int
    device_ms: float
    diffs: list = field(default_factory=list)
    iteration_ms: list = field(default_factory=list)
    kernel_launches: int = 0  # this library's kernels the run launched


L2_WINDOW = 4      # BW_LAUNCH_L2_WINDOW


def _relabel_flags(relabel):
    """None: the library decides; True / False force the hub-first order."""
    return 0 if relabel is None else (_abi.LAUNCH_RELABEL if relabel else _abi.LAUNCH_NO_RELABEL)


def _cfg(block=0, grid=0, warp=0, chunk=0, flags=0):
    return _abi.LaunchConfig(block, grid, warp, chunk, flags)


def _stats_list(arr, count):
    out = []
    for i in range(count):
        s = arr[i]
        out.append(dict(frontier_vertices=s.frontier_vertices, variant=s.variant,
                        frontier_edges=s.frontier_edges, log_degree_sum=s.log_degree_sum,
                        log_degree_sq_sum=s.log_degree_sq_sum, log_degree_max=s.log_degree_max,
                        device_ms=s.device_ms))
    return out


def _tuned(algorithm: str, variant, g, block, grid, warp, chunk, tuned: bool):
    """The caller's geometry, or -- when none is given and `tuned` -- the
    autotuner's configuration for this variant and graph shape class."""
    if not tuned or block or grid or warp or chunk:
        return block, grid, warp, chunk
    from . import autotune
    name = variant if isinstance(variant, str) else (
        bfs_variant_names() if algorithm == "bfs" else pagerank_variant_names())[variant]
    c = autotune.tuned_config(algorithm, name, g)
    return c.get("block", 0), c.get("grid", 0), c.get("warp", 0), c.get("chunk", 0)


def bfs(ctx: Context, g: DeviceGraph, variant: str | int, root: int, *, levels=None,
        loop: str = "host", max_levels: int = 0, stats: bool = False, block: int = 0,
        grid: int = 0, warp: int = 0, chunk: int = 0, tuned: bool = True, l2_window: bool = False,
        stream=None) -> BfsRun:
    """BFS from `root` with a fixed variant (BFS::runImplementation).  With
    no geometry given, the autotuner's configuration for the graph's shape
    class is used (tuned=False: the library default)."""
    torch = _torch()
    lib = library()
    block, grid, warp, chunk = _tuned("bfs", variant, g, block, grid, warp, chunk, tuned)
    if levels is None:
        levels = torch.empty(g.vertex_count, dtype=torch.int32, device=f"cuda:{ctx.device}")
    st = stream or torch.cuda.current_stream(levels.device)
    res = _abi.BfsResult()
    cap = (max_levels or g.vertex_count + 1) if stats else 0
    cap = min(cap, 1 << 20)
    arr = (_abi.BfsLevelStats * cap)() if cap else None
    rc = lib.bw_bfs_run(ctx.handle, C.byref(g.view), bfs_variant_id(variant), root, _ptr(levels),
                        C.byref(_cfg(block, grid, warp, chunk, L2_WINDOW if l2_window else 0)),
                        1 if loop == "graph" else 0,
                        max_levels, C.byref(res), arr, cap, C.c_void_p(st.cuda_stream))
    check(rc, f"bfs {variant}")
    run = BfsRun(levels, res.level_count, res.visited, res.traversed_edges, res.device_ms)
    if arr is not None:
        run.level_stats = _stats_list(arr, min(res.level_count, cap))
    return run


def bfs_schedule(ctx: Context, g: DeviceGraph, schedule: Iterable[str | int], root: int, *,
                 levels=None, max_levels: int = 0, time_levels: bool = False,
                 block: int = 0, grid: int = 0, warp: int = 0, chunk: int = 0, stream=None) -> BfsRun:
    """BFS with a per-level variant schedule (last entry repeats)."""
    torch = _torch()
    lib = library()
    sched = [bfs_variant_id(v) for v in schedule]
    arr_s = (C.c_int32 * len(sched))(*sched)
    if levels is None:
        levels = torch.empty(g.vertex_count, dtype=torch.int32, device=f"cuda:{ctx.device}")
    st = stream or torch.cuda.current_stream(levels.device)
    res = _abi.BfsResult()
    cap = min(max_levels or g.vertex_count + 1, 1 << 20)
    arr = (_abi.BfsLevelStats * cap)()
    rc = lib.bw_bfs_run_schedule(ctx.handle, C.byref(g.view), arr_s, len(sched), root, _ptr(levels),
                                 C.byref(_cfg(block, grid, warp, chunk)), max_levels, int(time_levels),
                                 C.byref(res), arr, cap, C.c_void_p(st.cuda_stream))
    check(rc, "bfs schedule")
    run = BfsRun(levels, res.level_count, res.visited, res.traversed_edges, res.device_ms)
    run.level_stats = _stats_list(arr, min(res.level_count, cap))
    return run


def pagerank(ctx: Context, g: DeviceGraph, variant: str | int, iterations: int = 30, *,
             ranks=None, block: int = 0, grid: int = 0, warp: int = 0, chunk: int = 0,
             relabel: bool | None = None, loop: str = "host", tuned: bool = True, l2_window: bool = False,
             stream=None) -> PageRankRun:
    """PageRank, damping 0.85, 1/N init, exactly `iterations` iterations.
    With no geometry given, the autotuner's configuration for the graph's
    shape class is used (tuned=False: the library default)."""
    torch = _torch()
    lib = library()
    block, grid, warp, chunk = _tuned("pagerank", variant, g, block, grid, warp, chunk, tuned)
    if ranks is None:
        ranks = torch.empty(g.vertex_count, dtype=torch.float32, device=f"cuda:{ctx.device}")
    st = stream or torch.cuda.current_stream(ranks.device)
    res = _abi.PagerankResult()
    diffs = (C.c_float * max(iterations, 1))()
    rc = lib.bw_pagerank_run(ctx.handle, C.byref(g.view), pagerank_variant_id(variant), iterations,
                             _ptr(ranks), C.byref(_cfg(block, grid, warp, chunk,
                                                       _relabel_flags(relabel) | (L2_WINDOW if l2_window else 0))),
                             1 if loop == "graph" else 0, C.byref(res), diffs, C.c_void_p(st.cuda_stream))
    check(rc, f"pagerank {variant}")
    return PageRankRun(ranks, res.iterations, res.device_ms, list(diffs)[:iterations],
                       kernel_launches=res.kernel_launches)


def gather_ceiling(ctx: Context, src, idx, *, warmup: int = 3, repeats: int = 10, stream=None) -> float:
    """Scattered 4-byte loads per second that the device sustains: the time
    of bw_gather_probe gathering src[idx] (float32 and uint32/int32 device
    tensors), timed with CUDA events on `stream` after `warmup` launches,
    median of `repeats`.  The bound of the PageRank pull kernels when their
    gathered vector fits in L2."""
    torch = _torch()
    lib = library()
    st = stream or torch.cuda.current_stream(src.device)
    partial = torch.empty(ctx.sm_count, dtype=torch.float32, device=src.device)

    def launch():
        check(lib.bw_gather_probe(ctx.handle, C.c_void_p(_ptr(src)), src.numel(), C.c_void_p(_ptr(idx)),
                                  idx.numel(), C.c_void_p(_ptr(partial)), C.c_void_p(st.cuda_stream)),
              "bw_gather_probe")

    for _ in range(warmup):
        launch()
    times = []
    for _ in range(repeats):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        launch()
        b.record(st)
        b.synchronize()
        times.append(a.elapsed_time(b) * 1e-3)
    return idx.numel() / float(np.median(times))


def gather_probe_sum(ctx: Context, src, idx, stream=None) -> float:
    """The probe's total (sum of the gathered values, in any order)."""
    torch = _torch()
    lib = library()
    st = stream or torch.cuda.current_stream(src.device)
    partial = torch.zeros(ctx.sm_count, dtype=torch.float32, device=src.device)
    check(lib.bw_gather_probe(ctx.handle, C.c_void_p(_ptr(src)), src.numel(), C.c_void_p(_ptr(idx)),
                              idx.numel(), C.c_void_p(_ptr(partial)), C.c_void_p(st.cuda_stream)),
          "bw_gather_probe")
    st.synchronize()
    return float(partial.double().sum().item())


def pagerank_schedule(ctx: Context, g: DeviceGraph, schedule: Iterable[str | int], iterations: int = 30,
                      *, ranks=None, time_iterations: bool = False, block: int = 0, grid: int = 0,
                      warp: int = 0, chunk: int = 0, relabel: bool | None = None, tuned: bool = True,
                      l2_window: bool = False, stream=None) -> PageRankRun:
    """PageRank with a per-iteration variant schedule (last entry repeats).
    A one-variant schedule with no geometry given runs the autotuner's
    configuration, as pagerank() does."""
    torch = _torch()
    lib = library()
    sched = [pagerank_variant_id(v) for v in schedule]
    if len(set(sched)) == 1:
        block, grid, warp, chunk = _tuned("pagerank", sched[0], g, block, grid, warp, chunk, tuned)
    arr_s = (C.c_int32 * len(sched))(*sched)
    if ranks is None:
        ranks = torch.empty(g.vertex_count, dtype=torch.float32, device=f"cuda:{ctx.device}")
    st = stream or torch.cuda.current_stream(ranks.device)
    res = _abi.PagerankResult()
    it_ms = (C.c_float * max(iterations, 1))()
    rc = lib.bw_pagerank_run_schedule(ctx.handle, C.byref(g.view), arr_s, len(sched), iterations,
                                      _ptr(ranks), C.byref(_cfg(block, grid, warp, chunk,
                                                                _relabel_flags(relabel) |
                                                                (L2_WINDOW if l2_window else 0))),
                                      int(time_iterations), it_ms, C.byref(res), C.c_void_p(st.cuda_stream))
    check(rc, "pagerank schedule")
    run = PageRankRun(ranks, res.iterations, res.device_ms, kernel_launches=res.kernel_launches)
    if time_iterations:
        run.iteration_ms = list(it_ms)[:iterations]
    return run
