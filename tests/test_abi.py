"""The C-ABI library loads and exports every symbol include/*.h declares;
host-side helpers that need no GPU.  CPU only (no compute calls)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

import belewitte_gb300 as bw
from belewitte_gb300 import _abi

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(bw_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_exported():
    lib = _abi.load()
    declared = _declared()
    assert len(declared) >= 30
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding covers all of them
    assert declared <= set(_abi.SIGNATURES), declared - set(_abi.SIGNATURES)


def test_exports_are_c_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_abi.LIB_PATH)], capture_output=True, text=True)
    exported = set(re.findall(r"\bT (bw_[a-z0-9_]+)$", out.stdout, flags=re.M))
    assert _declared() <= exported


def test_reference_variant_names():
    # bfs/bfs.cpp:121-207: 8 families x {"", -bulk, -warpreduce, -blockreduce}
    fams = ["edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list",
            "vertex-push", "vertex-pull", "vertex-push-warp", "vertex-pull-warp"]
    names = bw.bfs_variant_names()
    for f in fams:
        for s in ["", "-bulk", "-warpreduce", "-blockreduce"]:
            assert f + s in names
    assert names[:32] == [f + s for f in fams for s in ["", "-bulk", "-warpreduce", "-blockreduce"]]
    # pagerank/pagerank.cpp:205-351
    pr = bw.pagerank_variant_names()
    assert pr[:10] == ["edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list",
                       "vertex-push", "vertex-pull", "vertex-push-warp", "vertex-pull-warp",
                       "vertex-pull-nodiv", "vertex-pull-warp-nodiv"]
    with pytest.raises(KeyError):
        bw.bfs_variant_id("no-such-kernel")
    assert bw.library().bw_bfs_variant_name(999) is None


def test_compute_division_matches_reference_rule():
    # Backend.cpp:52-70 restated
    def ref(count, sm, mt=1024):
        cdiv = lambda x, y: (x + y - 1) // y
        i, b = 1, cdiv(count, sm)
        while b > mt:
            i += 1
            b = cdiv(count, i * sm)
        b += (32 - b % 32) if b % 32 else 0
        return b, min(i * sm, cdiv(count, b))
    for count in [1, 31, 32, 1000, 65536, 954639, 67108864, 536870912]:
        assert bw.compute_division(count, 152) == ref(count, 152)


def test_status_strings():
    lib = bw.library()
    assert lib.bw_status_string(0) == b"ok"
    assert b"representation" in lib.bw_status_string(2)
    assert lib.bw_version().startswith(b"belewitte-gb300")


def test_context_without_gpu_reports_no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert bw.library().bw_context_create(0, C.byref(h)) == 10     # BW_ERR_NO_DEVICE
    with pytest.raises(RuntimeError):
        bw.Context(0)


def test_reps_bits():
    # edge-list reads the forward EdgeList, vertex-pull the reverse CSR, ...
    lib = bw.library()
    assert lib.bw_bfs_variant_reps(bw.bfs_variant_id("edge-list")) == bw.REP_FWD_EL
    assert lib.bw_bfs_variant_reps(bw.bfs_variant_id("vertex-pull-bulk")) == bw.REP_REV_CSR
    assert lib.bw_pagerank_variant_reps(bw.pagerank_variant_id("rev-struct-edge-list")) == bw.REP_REV_ST
