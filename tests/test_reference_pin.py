"""Pin the oracle against the reference's OWN kernels on the GPU.

The reference's bfs/*.cu and pagerank/*.cu are compiled unmodified into
cubins (oracle/_ref, built where the reference tree exists) and run by
oracle/ref_runner.py around a restatement of the reference host loops.
"""
import numpy as np
import pytest

import oracle
from oracle import ref_runner
from tests.graphs import catalog, root_of

pytestmark = pytest.mark.gpu

GRAPHS = ["rmat10", "rmat12_sym", "er", "grid", "ba", "star", "tiny", "isolated"]


@pytest.fixture(scope="module")
def ref():
    if not ref_runner.cubins_present():
        pytest.skip("reference cubins not present (built from the reference tree)")
    return ref_runner.ReferenceKernels()


@pytest.fixture(scope="module")
def graphs(ref):
    out = {}
    for name in GRAPHS:
        make, root = catalog()[name]
        h = make()
        out[name] = (h, ref.upload_graph(h.vertex_count, h.fwd_vertices, h.fwd_edges, h.rev_vertices,
                                         h.rev_edges), root_of(h, root))
    return out


@pytest.mark.parametrize("variant", ref_runner.bfs_variant_names())
def test_reference_bfs_equals_oracle(ref, graphs, variant):
    for name, (h, dg, r) in graphs.items():
        lv, cnt = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, r)
        rl, rc = ref.bfs(dg, variant, r)
        assert np.array_equal(rl, lv), (variant, name)
        assert np.array_equal(rc, cnt), (variant, name)


@pytest.mark.parametrize("variant", ref_runner.PR_VARIANTS)
def test_reference_pagerank_equals_oracle(ref, graphs, variant):
    for name, (h, dg, r) in graphs.items():
        it = 30
        got, _ = ref.pagerank(dg, variant, it)
        sem = oracle.PR_NODIV if "nodiv" in variant else oracle.PR_DIV
        want, _ = oracle.pagerank(sem, h.vertex_count, h.rev_vertices, h.rev_edges, it)
        if variant in ("vertex-pull", "vertex-pull-nodiv"):
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (variant, name)
        else:
            rel = np.abs(got.astype(np.float64) - want) / np.abs(want.astype(np.float64))
            assert rel.max() <= 1e-5, (variant, name, rel.max())
