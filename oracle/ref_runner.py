"""Run the reference's own CUDA kernels on the GPU (parity pin).

TEST INFRASTRUCTURE ONLY.  The reference kernels (bfs/*.cu, pagerank/*.cu)
are compiled unmodified into cubins under oracle/_ref/ by
``oracle.build_ref()`` (this container, where the reference tree exists);
the cubins travel to the GPU machine and are loaded here with the CUDA
driver API.  The reference's host loops are restated around them:

  * BFS::runImplementation        bfs/bfs.cpp:51-118 (INT_MAX fill, root 0,
    resetFrontier / kernel / getFrontier until the frontier is empty)
  * PageRank::runImplementation   pagerank/pagerank.cpp:74-131 (1/N init,
    zero accumulator, zeroInitDegrees + computeDegrees, then per iteration
    resetDiff / kernel / consolidate(notLast) / getDiff)
  * launch geometry                Backend::computeDivision (Backend.cpp:52-70)
    over vertices or edges, warp kernels with (block / warp) * chunkMemory
    bytes of dynamic shared memory (ImplementationTemplate.hpp:166-167)
  * device graph structs           GraphRep.hpp:20-73 built as in
    GraphLoader.hpp:123-211

Nothing here touches the product library.
"""
from __future__ import annotations

import ctypes as C
import struct
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
INT_MAX = 2147483647

BFS_FAMILIES = ["edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list",
                "vertex-push", "vertex-pull", "vertex-push-warp", "vertex-pull-warp"]
BFS_SUFFIX = ["", "-bulk", "-warpreduce", "-blockreduce"]
_BFS_KERNEL = {
    "edge-list": ("11edgeListBfs", "P8EdgeListIjEPii", "EL", 0, "edge", False),
    "rev-edge-list": ("14revEdgeListBfs", "P8EdgeListIjEPii", "EL", 1, "edge", False),
    "struct-edge-list": ("17structEdgeListBfs", "P14StructEdgeListIjEPii", "SEL", 0, "edge", False),
    "rev-struct-edge-list": ("20revStructEdgeListBfs", "P14StructEdgeListIjEPii", "SEL", 1, "edge", False),
    "vertex-push": ("13vertexPushBfs", "P3CSRIjjEPii", "CSR", 0, "vertex", False),
    "vertex-pull": ("13vertexPullBfs", "P3CSRIjjEPii", "CSR", 1, "vertex", False),
    "vertex-push-warp": ("17vertexPushWarpBfs", "mmP3CSRIjjEPii", "CSR", 0, "vertex", True),
    "vertex-pull-warp": ("17vertexPullWarpBfs", "mmP3CSRIjjEPii", "CSR", 1, "vertex", True),
}

# name -> (kernel, rep, dir, division, warp smem per chunk fn | None,
#          consolidate, degree kernel | None, degree rep, degree dir, degree division)
_PR_VARIANTS = {
    "edge-list": ("_Z16edgeListPageRankP8EdgeListIjEPjPfS3_", "EL", 0, "edge", None, "div",
                  "_Z22edgeListComputeDegreesP8EdgeListIjEPj", "EL", 0, "edge"),
    "rev-edge-list": ("_Z19revEdgeListPageRankP8EdgeListIjEPjPfS3_", "EL", 1, "edge", None, "div",
                      "_Z29reverseEdgeListComputeDegreesP8EdgeListIjEPj", "EL", 1, "edge"),
    "struct-edge-list": ("_Z22structEdgeListPageRankP14StructEdgeListIjEPjPfS3_", "SEL", 0, "edge", None, "div",
                         "_Z28structEdgeListComputeDegreesP14StructEdgeListIjEPj", "SEL", 0, "edge"),
    "rev-struct-edge-list": ("_Z25revStructEdgeListPageRankP14StructEdgeListIjEPjPfS3_", "SEL", 1, "edge", None,
                             "div", "_Z35reverseStructEdgeListComputeDegreesP14StructEdgeListIjEPj", "SEL", 1, "edge"),
    "vertex-push": ("_Z18vertexPushPageRankP3CSRIjjEPjPfS3_", "CSR", 0, "vertex", None, "div",
                    None, None, None, None),
    "vertex-pull": ("_Z18vertexPullPageRankP3CSRIjjEPjPfS3_", "CSR", 1, "vertex", None, "div",
                    "_Z24reverseCSRComputeDegreesP3CSRIjjEPj", "CSR", 1, "vertex"),
    "vertex-push-warp": ("_Z22vertexPushWarpPageRankmmP3CSRIjjEPjPfS3_", "CSR", 0, "vertex",
                         lambda c: c * 4 + (1 + c) * 4, "div", None, None, None, None),
    "vertex-pull-warp": ("_Z22vertexPullWarpPageRankmmP3CSRIjjEPjPfS3_", "CSR", 1, "vertex",
                         lambda c: (1 + c) * 4, "div",
                         "_Z24reverseCSRComputeDegreesP3CSRIjjEPj", "CSR", 1, "vertex"),
    "vertex-pull-nodiv": ("_Z23vertexPullNoDivPageRankP3CSRIjjEPjPfS3_", "CSR", 1, "vertex", None, "nodiv",
                          "_Z24reverseCSRComputeDegreesP3CSRIjjEPj", "CSR", 1, "vertex"),
    "vertex-pull-warp-nodiv": ("_Z27vertexPullWarpNoDivPageRankmmP3CSRIjjEPjPfS3_", "CSR", 1, "vertex",
                               lambda c: (1 + c) * 4, "nodiv",
                               "_Z24reverseCSRComputeDegreesP3CSRIjjEPj", "CSR", 1, "vertex"),
}
PR_VARIANTS = list(_PR_VARIANTS)
_CONSOLIDATE = {"div": "_Z15consolidateRankmPjPfS0_b", "nodiv": "_Z20consolidateRankNoDivmPjPfS0_b"}
_ZERO_INIT = "_Z21zeroInitDegreesKernelmPj"


def bfs_variant_names():
    return [f + s for s in BFS_SUFFIX for f in BFS_FAMILIES]


def cubins_present() -> bool:
    return all((REF_DIR / n).exists() for n in ("ref_bfs.cubin", "ref_pagerank.cubin",
                                                "ref_pagerank_pull_warp.cubin"))


def compute_division(count: int, sm: int, max_tpb: int = 1024):
    """Backend::computeDivision (Backend.cpp:52-70)."""
    def cdiv(x, y):
        return (x + y - 1) // y
    i = 1
    b = cdiv(count, sm)
    while b > max_tpb:
        i += 1
        b = cdiv(count, i * sm)
    adj = b % 32
    b += 32 - adj if adj else 0
    b = max(b, 32)
    g = max(1, min(i * sm, cdiv(count, b)))
    return b, g


class _Driver:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        for name, res, args in [
            ("cuModuleLoad", C.c_int, [C.POINTER(C.c_void_p), C.c_char_p]),
            ("cuModuleUnload", C.c_int, [C.c_void_p]),
            ("cuModuleGetFunction", C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]),
            ("cuModuleGetGlobal_v2", C.c_int, [C.POINTER(C.c_uint64), C.POINTER(C.c_size_t), C.c_void_p,
                                               C.c_char_p]),
            ("cuLaunchKernel", C.c_int, [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                         C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
            ("cuMemcpyHtoD_v2", C.c_int, [C.c_uint64, C.c_void_p, C.c_size_t]),
            ("cuMemcpyDtoH_v2", C.c_int, [C.c_void_p, C.c_uint64, C.c_size_t]),
            ("cuCtxSynchronize", C.c_int, []),
        ]:
            f = getattr(self.cu, name)
            f.restype, f.argtypes = res, args

    def ok(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")


class ReferenceKernels:
    """Loads the reference cubins into the current (torch) CUDA context."""

    def __init__(self):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("reference kernels need a GPU")
        if not cubins_present():
            raise FileNotFoundError("reference cubins missing under oracle/_ref (oracle.build_ref())")
        self.torch = torch
        torch.zeros(1, device="cuda")        # make the primary context current
        self.sm = torch.cuda.get_device_properties(0).multi_processor_count
        self.drv = _Driver()
        self.mods = {}
        for key in ("ref_bfs", "ref_pagerank", "ref_pagerank_pull_warp"):
            m = C.c_void_p()
            self.drv.ok(self.drv.cu.cuModuleLoad(C.byref(m), str(REF_DIR / f"{key}.cubin").encode()), "cuModuleLoad")
            self.mods[key] = m
        self._fn_cache = {}

    def fn(self, module, name):
        key = (module, name)
        if key not in self._fn_cache:
            f = C.c_void_p()
            self.drv.ok(self.drv.cu.cuModuleGetFunction(C.byref(f), self.mods[module], name.encode()),
                        f"cuModuleGetFunction {name}")
            self._fn_cache[key] = f
        return self._fn_cache[key]

    def global_ptr(self, module, name):
        p, sz = C.c_uint64(), C.c_size_t()
        self.drv.ok(self.drv.cu.cuModuleGetGlobal_v2(C.byref(p), C.byref(sz), self.mods[module], name.encode()),
                    f"cuModuleGetGlobal {name}")
        return p.value

    def launch(self, f, grid, block, smem, args):
        holders = []
        ptrs = (C.c_void_p * len(args))()
        for i, (kind, val) in enumerate(args):
            h = {"u64": C.c_uint64, "i32": C.c_int32, "bool": C.c_bool}[kind](val)
            holders.append(h)
            ptrs[i] = C.cast(C.byref(h), C.c_void_p)
        stream = C.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        self.drv.ok(self.drv.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, stream, ptrs, None),
                    "cuLaunchKernel")

    def sync(self):
        self.torch.cuda.synchronize()

    # -- device graph structs (GraphRep.hpp, GraphLoader.hpp:123-211) -------
    def upload_graph(self, n, fwd_v, fwd_e, rev_v, rev_e):
        torch = self.torch
        m = int(len(fwd_e))

        def dev(a, dtype=np.uint32):
            a = np.ascontiguousarray(np.asarray(a, dtype=dtype))
            if a.size == 0:
                a = np.zeros(1, dtype=dtype)
            return torch.from_numpy(a.view(np.uint8).copy()).cuda()
        fv = np.asarray(fwd_v, np.uint32)
        rv = np.asarray(rev_v, np.uint32)
        fwd_src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(fv.astype(np.int64)))
        rev_dst = np.repeat(np.arange(n, dtype=np.uint32), np.diff(rv.astype(np.int64)))
        keep = {}
        keep["fv"], keep["fe"] = dev(fv), dev(fwd_e)
        keep["rv"], keep["re"] = dev(rv), dev(rev_e)
        keep["fin"], keep["fout"] = dev(fwd_src), dev(fwd_e)
        keep["rin"], keep["rout"] = dev(rev_dst), dev(rev_e)
        keep["fst"] = dev(np.stack([fwd_src, np.asarray(fwd_e, np.uint32)], 1).reshape(-1))
        keep["rst"] = dev(np.stack([rev_dst, np.asarray(rev_e, np.uint32)], 1).reshape(-1))
        p = {k: v.data_ptr() for k, v in keep.items()}
        structs = {
            ("CSR", 0): struct.pack("<QQQQ", n, m, p["fv"], p["fe"]),
            ("CSR", 1): struct.pack("<QQQQ", n, m, p["rv"], p["re"]),
            ("EL", 0): struct.pack("<QQQQ", n, m, p["fin"], p["fout"]),
            ("EL", 1): struct.pack("<QQQQ", n, m, p["rin"], p["rout"]),
            ("SEL", 0): struct.pack("<QQQ", n, m, p["fst"]),
            ("SEL", 1): struct.pack("<QQQ", n, m, p["rst"]),
        }
        g = {"n": n, "m": m, "keep": keep, "struct": {}}
        for key, blob in structs.items():
            t = torch.from_numpy(np.frombuffer(blob, dtype=np.uint8).copy()).cuda()
            g["struct"][key] = t
            g["keep"][("s",) + key] = t
        return g

    # -- BFS ---------------------------------------------------------------
    def _event(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.torch.cuda.current_stream())
        return e

    def bfs(self, g, variant: str, root: int, warp: int = 32, chunk: int = 32, max_levels: int = 1 << 20,
            times: list | None = None):
        """Depths and per-level visit counts; with `times`, each level's
        kernel time (CUDA events around the launch, host round trips
        excluded) is appended in ms."""
        torch = self.torch
        fam = variant
        red = 0
        for i, s in enumerate(BFS_SUFFIX):
            if s and variant.endswith(s):
                fam, red = variant[: -len(s)], i
        prefix, tail, rep, direction, div, warpk = _BFS_KERNEL[fam]
        name = f"_Z{prefix}I9ReductionIL11bfs_variant{red}EEE v{tail}".replace(" ", "")
        f = self.fn("ref_bfs", name)
        n, m = g["n"], g["m"]
        count = m if div == "edge" else n
        block, grid = compute_division(count, self.sm)
        smem = (block // warp) * (chunk * 4 + (chunk + 1) * 4) if warpk else 0
        levels = torch.full((n,), INT_MAX, dtype=torch.int32, device="cuda")
        levels[root] = 0
        fptr = self.global_ptr("ref_bfs", "frontier")
        zero = C.c_uint32(0)
        out = C.c_uint32(0)
        counts = []
        curr = 0
        while True:
            self.sync()
            self.drv.ok(self.drv.cu.cuMemcpyHtoD_v2(fptr, C.byref(zero), 4), "resetFrontier")
            args = []
            if warpk:
                args += [("u64", warp), ("u64", chunk)]
            args += [("u64", g["struct"][(rep, direction)].data_ptr()), ("u64", levels.data_ptr()), ("i32", curr)]
            e0 = self._event() if times is not None else None
            self.launch(f, grid, block, smem, args)
            e1 = self._event() if times is not None else None
            self.sync()
            if times is not None:
                times.append(e0.elapsed_time(e1))
            self.drv.ok(self.drv.cu.cuMemcpyDtoH_v2(C.byref(out), fptr, 4), "getFrontier")
            counts.append(out.value)
            curr += 1
            if out.value == 0 or curr >= max_levels:
                break
        return levels.cpu().numpy(), np.array(counts, dtype=np.uint32)

    # -- PageRank ----------------------------------------------------------
    def pagerank(self, g, variant: str, iterations: int, warp: int = 32, chunk: int = 32,
                 times: list | None = None):
        """Ranks and per-iteration diffs; with `times`, each iteration's
        kernel + consolidation time (CUDA events, host round trips excluded)
        is appended in ms."""
        torch = self.torch
        (kname, rep, direction, div, mem, cons, dname, drep, ddir, ddiv) = _PR_VARIANTS[variant]
        module = "ref_pagerank_pull_warp" if "PullWarp" in kname else "ref_pagerank"
        n, m = g["n"], g["m"]
        vb, vg = compute_division(n, self.sm)
        eb, eg = compute_division(m, self.sm)

        def geo(d):
            return (vb, vg) if d == "vertex" else (eb, eg)
        pr = torch.full((n,), np.float32(1.0) / np.float32(n), dtype=torch.float32, device="cuda")
        newpr = torch.zeros(n, dtype=torch.float32, device="cuda")
        deg = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda") if dname else None
        degp = deg.data_ptr() if deg is not None else 0
        vc = g["struct"][("CSR", 0)]   # VertexCount rep: the count itself is passed
        del vc
        if dname:
            b, gr = geo("vertex")
            self.launch(self.fn("ref_pagerank", _ZERO_INIT), gr, b, 0, [("u64", n), ("u64", degp)])
            b, gr = geo(ddiv)
            self.launch(self.fn("ref_pagerank", dname), gr, b, 0,
                        [("u64", g["struct"][(drep, ddir)].data_ptr()), ("u64", degp)])
        kf = self.fn(module, kname)
        cf = self.fn("ref_pagerank", _CONSOLIDATE[cons])
        dptr = self.global_ptr("ref_pagerank", "diff")
        zero = C.c_float(0.0)
        diffs = []
        b, gr = geo(div)
        smem = (b // warp) * mem(chunk) if mem else 0
        for j in range(1, iterations + 1):
            self.sync()
            self.drv.ok(self.drv.cu.cuMemcpyHtoD_v2(dptr, C.byref(zero), 4), "resetDiff")
            args = [("u64", warp), ("u64", chunk)] if mem else []
            args += [("u64", g["struct"][(rep, direction)].data_ptr()), ("u64", degp),
                     ("u64", pr.data_ptr()), ("u64", newpr.data_ptr())]
            e0 = self._event() if times is not None else None
            self.launch(kf, gr, b, smem, args)
            cb, cg = geo("vertex")
            self.launch(cf, cg, cb, 0, [("u64", n), ("u64", degp), ("u64", pr.data_ptr()),
                                        ("u64", newpr.data_ptr()), ("bool", iterations > j)])
            e1 = self._event() if times is not None else None
            self.sync()
            if times is not None:
                times.append(e0.elapsed_time(e1))
            out = C.c_float(0.0)
            self.drv.ok(self.drv.cu.cuMemcpyDtoH_v2(C.byref(out), dptr, 4), "getDiff")
            diffs.append(out.value)
        return pr.cpu().numpy(), np.array(diffs, dtype=np.float32)
