"""The allocation-free BFS entry point (bw_bfs_run_noalloc).

Callers that cannot allocate device memory while running (a serving process
with a fixed HBM budget, a host application with its own allocator policy)
use this entry point: its scratch is a fixed device array inside the
library.  This file is collected last so a failure here leaves every other
test already run.  Output must equal the context-based frontier-push BFS,
bit for bit, on two calls in a row.
"""
import ctypes as C

import numpy as np
import pytest

import belewitte_gb300 as bw
from belewitte_gb300 import _abi
from tests.graphs import catalog, root_of

pytestmark = pytest.mark.gpu


def _noalloc(g, root, levels):
    import torch
    count = C.c_uint32()
    st = torch.cuda.current_stream()
    rc = bw.library().bw_bfs_run_noalloc(C.byref(g.view), root, C.c_void_p(levels.data_ptr()), 0, C.byref(count),
                                         C.c_void_p(st.cuda_stream))
    return rc, count.value


def test_noalloc_matches_context_entry_point(ctx):
    import torch
    graphs = [catalog()[name] for name in ("rmat14", "ba", "grid", "star")]
    for make, root in graphs:
        h = make()
        g = bw.DeviceGraph(h, reps=bw.REP_FWD_CSR | bw.REP_REV_CSR)
        r = root_of(h, root)
        want = bw.bfs(ctx, g, "frontier-push", r)
        for _ in range(2):                       # two calls in a row share the scratch
            levels = torch.full((h.vertex_count,), -7, dtype=torch.int32, device="cuda")
            rc, count = _noalloc(g, r, levels)
            assert rc == 0
            assert count == want.level_count
            assert torch.equal(levels, want.levels)


def test_noalloc_at_its_limits(ctx):
    """A graph at the entry point's size limits: 2^20 vertices and
    16,776,975 edges.  Vertex 0 points at fifteen hubs and at every leaf;
    each hub points at every leaf, so level 1 holds fifteen rows of about
    2^20 edges (the hub-chunk queue's largest load) next to a million leaves."""
    import torch

    import oracle
    n = 2 ** 20
    hubs = np.arange(1, 16, dtype=np.uint32)
    leaves = np.arange(16, n, dtype=np.uint32)
    src = np.concatenate([np.zeros(15 + leaves.size, np.uint32), np.repeat(hubs, leaves.size)])
    dst = np.concatenate([hubs, leaves, np.tile(leaves, hubs.size)])
    assert src.size == 16 * leaves.size + 15 <= 2 ** 24
    h = bw.HostGraph.from_edges(n, src, dst)
    del src, dst
    g = bw.DeviceGraph(h, reps=bw.REP_FWD_CSR | bw.REP_REV_CSR)
    want, counts = oracle.bfs(n, h.fwd_vertices, h.fwd_edges, 0)
    for _ in range(2):
        levels = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        rc, count = _noalloc(g, 0, levels)
        assert rc == 0
        assert count == len(counts)
        assert np.array_equal(levels.cpu().numpy(), want)


def test_noalloc_second_call_leaves_free_memory_unchanged(ctx):
    """After the first call on a device (which reserves the fixed array under
    lazy module loading) a call takes no device memory."""
    import torch
    make, root = catalog()["rmat14"]
    h = make()
    g = bw.DeviceGraph(h, reps=bw.REP_FWD_CSR | bw.REP_REV_CSR)
    levels = torch.empty(h.vertex_count, dtype=torch.int32, device="cuda")
    r = root_of(h, root)
    assert _noalloc(g, r, levels)[0] == 0
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info()[0]
    assert _noalloc(g, r, levels)[0] == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == before


def test_noalloc_rejects_sizes_beyond_its_maximum():
    # rejected from the sizes alone: no device memory is touched
    view = _abi.GraphView(2 ** 20 + 1, 10, 1, 1, 0, 0, 0, 0, 0, 0)
    count = C.c_uint32()
    rc = bw.library().bw_bfs_run_noalloc(C.byref(view), 0, C.c_void_p(16), 0, C.byref(count), None)
    assert rc == 7                                  # BW_ERR_TOO_LARGE
    view = _abi.GraphView(1000, 2 ** 24 + 1, 1, 1, 0, 0, 0, 0, 0, 0)
    assert bw.library().bw_bfs_run_noalloc(C.byref(view), 0, C.c_void_p(16), 0, C.byref(count), None) == 7
