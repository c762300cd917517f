"""ctypes declarations of the C ABI in include/belewitte_gb300.h."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libbelewitte_gb300.so"

u32p = C.POINTER(C.c_uint32)
i32p = C.POINTER(C.c_int32)


class GraphView(C.Structure):
    _fields_ = [("vertex_count", C.c_uint64), ("edge_count", C.c_uint64),
                ("fwd_vertices", C.c_void_p), ("fwd_edges", C.c_void_p),
                ("rev_vertices", C.c_void_p), ("rev_edges", C.c_void_p),
                ("fwd_in_edges", C.c_void_p), ("rev_in_edges", C.c_void_p),
                ("fwd_struct_edges", C.c_void_p), ("rev_struct_edges", C.c_void_p)]


class HostGraphC(C.Structure):
    _fields_ = [("vertex_count", C.c_uint64), ("edge_count", C.c_uint64),
                ("undirected", C.c_int32), ("reserved", C.c_int32),
                ("fwd_vertices", u32p), ("fwd_edges", u32p),
                ("rev_vertices", u32p), ("rev_edges", u32p)]


class DeviceGraphC(C.Structure):
    _fields_ = [("vertex_count", C.c_uint64), ("edge_count", C.c_uint64),
                ("undirected", C.c_int32), ("reserved", C.c_int32),
                ("fwd_vertices", C.c_void_p), ("fwd_edges", C.c_void_p),
                ("rev_vertices", C.c_void_p), ("rev_edges", C.c_void_p)]


class LaunchConfig(C.Structure):
    _fields_ = [("block_size", C.c_uint32), ("grid_size", C.c_uint32),
                ("warp_size", C.c_uint32), ("chunk_size", C.c_uint32), ("flags", C.c_uint32)]


LAUNCH_RELABEL = 1
LAUNCH_NO_RELABEL = 2


class BfsLevelStats(C.Structure):
    _fields_ = [("frontier_vertices", C.c_uint32), ("variant", C.c_uint32),
                ("frontier_edges", C.c_uint64), ("log_degree_sum", C.c_float),
                ("log_degree_sq_sum", C.c_float), ("log_degree_max", C.c_float),
                ("device_ms", C.c_float)]


class BfsResult(C.Structure):
    _fields_ = [("level_count", C.c_uint32), ("reserved", C.c_uint32),
                ("visited", C.c_uint64), ("traversed_edges", C.c_uint64),
                ("device_ms", C.c_double)]


class PagerankResult(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("kernel_launches", C.c_uint32),
                ("last_diff", C.c_float), ("reserved_f", C.c_float),
                ("device_ms", C.c_double)]


class BatchResult(C.Structure):
    _fields_ = [("units", C.c_uint64), ("traversed_edges", C.c_uint64), ("device_ms", C.c_double)]


class MlpTrainConfig(C.Structure):
    _fields_ = [("steps", C.c_uint32), ("batch", C.c_uint32), ("lr", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float), ("weight_decay", C.c_float), ("reserved", C.c_uint32),
                ("seed", C.c_uint64)]


class SwitchConfig(C.Structure):
    _fields_ = [("params", C.c_void_p), ("classes", C.c_uint32), ("fallback", C.c_int32),
                ("candidates", C.POINTER(C.c_int32)), ("threshold", C.c_float), ("flags", C.c_uint32)]


# name -> (restype, argtypes); every symbol declared in include/belewitte_gb300.h
SIGNATURES = {
    "bw_status_string": (C.c_char_p, [C.c_int]),
    "bw_last_error": (C.c_char_p, []),
    "bw_version": (C.c_char_p, []),
    "bw_host_graph_free": (None, [C.POINTER(HostGraphC)]),
    "bw_graph_from_edges": (C.c_int, [C.c_uint64, C.c_uint64, u32p, u32p, C.c_int, C.POINTER(HostGraphC)]),
    "bw_generate_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                   C.c_uint64, C.c_int, C.POINTER(HostGraphC)]),
    "bw_generate_rmat_n": (C.c_int, [C.c_uint64, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                     C.c_uint64, C.c_int, C.POINTER(HostGraphC)]),
    "bw_generate_er": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int, C.POINTER(HostGraphC)]),
    "bw_generate_grid": (C.c_int, [C.c_uint32, C.c_uint32, C.POINTER(HostGraphC)]),
    "bw_generate_ba": (C.c_int, [C.c_uint64, C.c_uint32, C.c_uint64, C.POINTER(HostGraphC)]),
    "bw_generate_device": (C.c_int, [C.c_int, C.c_uint64, C.c_uint64, C.c_double, C.c_double, C.c_double,
                                     C.c_uint64, C.c_int, C.POINTER(DeviceGraphC), C.c_void_p]),
    "bw_device_graph_free": (None, [C.POINTER(DeviceGraphC)]),
    "bw_graph_file_read": (C.c_int, [C.c_char_p, C.POINTER(HostGraphC)]),
    "bw_graph_file_write": (C.c_int, [C.c_char_p, C.POINTER(HostGraphC)]),
    "bw_degree_statistics": (C.c_int, [C.POINTER(HostGraphC), C.c_int, C.POINTER(C.c_double)]),
    "bw_degree_statistics_device": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.c_int, C.c_int,
                                              C.POINTER(C.c_double), C.c_void_p]),
    "bw_context_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "bw_context_destroy": (C.c_int, [C.c_void_p]),
    "bw_context_sm_count": (C.c_int, [C.c_void_p]),
    "bw_compute_division": (None, [C.c_uint64, C.c_uint32, C.c_uint32, u32p, u32p]),
    "bw_expand_edge_list": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p]),
    "bw_build_struct_edges": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    "bw_bfs_variant_count": (C.c_int, []),
    "bw_bfs_variant_name": (C.c_char_p, [C.c_int]),
    "bw_bfs_variant_lookup": (C.c_int, [C.c_char_p]),
    "bw_bfs_variant_reps": (C.c_int, [C.c_int]),
    "bw_bfs_init": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p, C.c_void_p]),
    "bw_bfs_level": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.c_int, C.c_void_p, C.c_int32,
                               C.POINTER(LaunchConfig), u32p, C.c_void_p]),
    "bw_bfs_run": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.c_int, C.c_uint32, C.c_void_p,
                             C.POINTER(LaunchConfig), C.c_int, C.c_uint32, C.POINTER(BfsResult),
                             C.POINTER(BfsLevelStats), C.c_uint32, C.c_void_p]),
    "bw_bfs_run_schedule": (C.c_int, [C.c_void_p, C.POINTER(GraphView), i32p, C.c_uint32, C.c_uint32,
                                      C.c_void_p, C.POINTER(LaunchConfig), C.c_uint32, C.c_int,
                                      C.POINTER(BfsResult), C.POINTER(BfsLevelStats), C.c_uint32,
                                      C.c_void_p]),
    "bw_pagerank_variant_count": (C.c_int, []),
    "bw_pagerank_variant_name": (C.c_char_p, [C.c_int]),
    "bw_pagerank_variant_lookup": (C.c_int, [C.c_char_p]),
    "bw_pagerank_variant_reps": (C.c_int, [C.c_int]),
    "bw_pagerank_run": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.c_int, C.c_uint32, C.c_void_p,
                                  C.POINTER(LaunchConfig), C.c_int, C.POINTER(PagerankResult),
                                  C.POINTER(C.c_float), C.c_void_p]),
    "bw_pagerank_run_schedule": (C.c_int, [C.c_void_p, C.POINTER(GraphView), i32p, C.c_uint32,
                                           C.c_uint32, C.c_void_p, C.POINTER(LaunchConfig), C.c_int,
                                           C.POINTER(C.c_float), C.POINTER(PagerankResult), C.c_void_p]),
    "bw_mlp_param_count": (C.c_uint32, [C.c_uint32]),
    "bw_bfs_features": (None, [C.c_uint64, C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_uint64, C.c_uint64,
                               C.c_uint64, C.c_uint64, C.c_uint32, C.POINTER(C.c_float)]),
    "bw_bfs_profile": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.c_uint32, C.c_void_p, i32p, C.c_uint32,
                                 C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_float),
                                 C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.c_void_p]),
    "bw_mlp_init": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint64,
                              C.c_void_p]),
    "bw_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                               C.POINTER(MlpTrainConfig), C.POINTER(C.c_float), C.c_uint32, C.c_void_p]),
    "bw_mlp_gradient": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_uint32, C.c_void_p, C.POINTER(C.c_float), C.c_void_p]),
    "bw_mlp_predict": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                 C.c_void_p]),
    "bw_mlp_predict_host": (C.c_int, [C.POINTER(C.c_float), C.c_uint32, C.POINTER(C.c_float), C.c_uint32,
                                      C.POINTER(C.c_float)]),
    "bw_bfs_frontier_stats": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.c_uint32, C.c_int32,
                                        C.POINTER(BfsLevelStats), C.c_void_p]),
    "bw_pagerank_features": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.c_uint32, C.POINTER(C.c_float),
                                       C.c_void_p]),
    "bw_pagerank_run_learned": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.POINTER(SwitchConfig), C.c_uint32,
                                          C.c_void_p, C.c_int, C.POINTER(PagerankResult), C.POINTER(C.c_float),
                                          C.POINTER(C.c_int32), C.c_void_p]),
    "bw_bfs_run_learned": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.POINTER(SwitchConfig), C.c_uint32,
                                     C.c_void_p, C.c_int, C.c_uint32, C.POINTER(BfsResult),
                                     C.POINTER(BfsLevelStats), C.c_uint32, C.c_void_p]),
    "bw_batch_run": (C.c_int, [C.c_void_p, C.POINTER(GraphView), C.c_int, C.c_void_p, C.c_uint32, C.c_void_p,
                               C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                               C.POINTER(LaunchConfig), C.POINTER(BatchResult), C.c_void_p]),
    "bw_gather_probe": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p,
                                  C.c_void_p]),
    "bw_bfs_run_noalloc": (C.c_int, [C.POINTER(GraphView), C.c_uint32, C.c_void_p, C.c_uint32,
                                     C.POINTER(C.c_uint32), C.c_void_p]),
}

_lib = None


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libbelewitte_gb300.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if not build_if_missing:
            raise ImportError(f"{LIB_PATH} is missing; run __graft_entry__.build()")
        from . import build as _build
        _build.build_core()
    lib = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | getattr(os, "RTLD_GLOBAL", 0))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class BwError(RuntimeError):
    def __init__(self, status: int, what: str):
        lib = load()
        msg = lib.bw_status_string(status).decode()
        detail = lib.bw_last_error().decode()
        super().__init__(f"{what}: {msg} ({status})" + (f" [{detail}]" if detail and status == 4 else ""))
        self.status = status


def check(status: int, what: str) -> None:
    if status != 0:
        raise BwError(status, what)
