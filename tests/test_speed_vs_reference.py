"""Speed of every variant against the reference's own CUDA kernel of the
same name, on the same GPU and the same graph (the reference kernels are
compiled unmodified into cubins and driven by oracle/ref_runner.py around a
restatement of its host loops).

The reference is timed generously: CUDA events around its kernel launches
only, so its per-level and per-iteration host round trips (frontier and
diff read-backs) are not counted.  Ours is timed as shipped: PageRank
iterations with CUDA events per iteration; BFS as the whole device-side
traversal (one CUDA graph with a conditional loop).

Graphs: R-MAT scale 20, edge factor 16 (PageRank, directed), and its
symmetrised version (BFS from the highest-out-degree vertex).  Set
BW_SPEED_REPORT to a path to write the table as JSON."""
import json
import os

import numpy as np
import pytest

import belewitte_gb300 as bw
from oracle import ref_runner

pytestmark = pytest.mark.gpu

PR_VARIANTS = ["edge-list", "rev-edge-list", "struct-edge-list", "rev-struct-edge-list", "vertex-push",
               "vertex-pull", "vertex-push-warp", "vertex-pull-warp", "vertex-pull-nodiv", "vertex-pull-warp-nodiv"]
PR_ITERATIONS = 6


@pytest.fixture(scope="module")
def setup(ctx):
    if not ref_runner.cubins_present():
        pytest.skip("reference cubins not present (built from the reference tree)")
    ref = ref_runner.ReferenceKernels()
    hp = bw.HostGraph.rmat(20, 16, seed=20)
    hb = bw.HostGraph.rmat(20, 16, seed=20, symmetrise=True)
    out = {"ref": ref, "pr": (hp, bw.DeviceGraph(hp, reps=63),
                              ref.upload_graph(hp.vertex_count, hp.fwd_vertices, hp.fwd_edges, hp.rev_vertices,
                                               hp.rev_edges)),
           "bfs": (hb, bw.DeviceGraph(hb, reps=63),
                   ref.upload_graph(hb.vertex_count, hb.fwd_vertices, hb.fwd_edges, hb.rev_vertices,
                                    hb.rev_edges))}
    yield out
    report = os.environ.get("BW_SPEED_REPORT")
    if report and "table" in out:
        with open(report, "w") as f:
            json.dump(out["table"], f, indent=1)


def _record(setup, kind, variant, ours_ms, ref_ms):
    setup.setdefault("table", {}).setdefault(kind, {})[variant] = {
        "ours_ms": round(ours_ms, 4), "reference_ms": round(ref_ms, 4), "speedup": round(ref_ms / ours_ms, 2)}
    print(f"{kind} {variant:28s} ours {ours_ms:9.4f} ms  reference {ref_ms:9.4f} ms  x{ref_ms / ours_ms:7.2f}")


@pytest.mark.parametrize("variant", PR_VARIANTS)
def test_pagerank_iteration_faster_than_reference(ctx, setup, variant):
    """Median per-iteration time (iterations 2..6): ours below the
    reference kernel's."""
    h, g, rg = setup["pr"]
    ref = setup["ref"]
    times = []
    ref.pagerank(rg, variant, PR_ITERATIONS, times=times)
    ref_ms = float(np.median(times[1:]))
    bw.pagerank(ctx, g, variant, 2)
    run = bw.pagerank_schedule(ctx, g, [variant], PR_ITERATIONS, time_iterations=True)
    ours_ms = float(np.median(run.iteration_ms[1:]))
    _record(setup, "pagerank", variant, ours_ms, ref_ms)
    assert ours_ms < ref_ms


@pytest.mark.parametrize("variant", ref_runner.bfs_variant_names())
def test_bfs_traversal_faster_than_reference(ctx, setup, variant):
    """Whole traversal: ours (device loop) below the sum of the reference
    kernel's level times."""
    h, g, rg = setup["bfs"]
    ref = setup["ref"]
    root = h.max_out_degree_vertex()
    ref_ms = []
    for _ in range(2):
        times = []
        ref.bfs(rg, variant, root, times=times)
        ref_ms.append(sum(times))
    ours = [bw.bfs(ctx, g, variant, root, loop="graph").device_ms for _ in range(3)]
    _record(setup, "bfs", variant, min(ours), min(ref_ms))
    assert min(ours) < min(ref_ms)
