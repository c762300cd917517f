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


def test_noalloc_rejects_sizes_beyond_its_maximum():
    # rejected from the sizes alone: no device memory is touched
    view = _abi.GraphView(2 ** 20 + 1, 10, 1, 1, 0, 0, 0, 0, 0, 0)
    count = C.c_uint32()
    rc = bw.library().bw_bfs_run_noalloc(C.byref(view), 0, C.c_void_p(16), 0, C.byref(count), None)
    assert rc == 7                                  # BW_ERR_TOO_LARGE
    view = _abi.GraphView(1000, 2 ** 24 + 1, 1, 1, 0, 0, 0, 0, 0, 0)
    assert bw.library().bw_bfs_run_noalloc(C.byref(view), 0, C.c_void_p(16), 0, C.byref(count), None) == 7
