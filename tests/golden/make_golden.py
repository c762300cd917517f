"""Record golden fixtures from the reference's OWN CUDA kernels.

Runs on a machine with a GPU and the reference cubins under oracle/_ref
(compiled, unmodified, from the reference's bfs/*.cu and pagerank/*.cu by
oracle.build_ref()).  For each small seeded graph it stores the graph (CSR +
reverse CSR), the BFS depths and per-level frontier counts every one of the
32 reference BFS implementations produced (they must all agree), and the
final ranks of each of the 10 reference PageRank implementations after 30
iterations.  tests/test_oracle.py checks the CPU oracle against them with no
GPU.

    python tests/golden/make_golden.py [OUT_DIR]
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import belewitte_gb300 as bw  # noqa: E402  (graph generation only)
from oracle import ref_runner  # noqa: E402

ITERATIONS = 30
GRAPHS = {
    "rmat10_s11": (lambda: bw.HostGraph.rmat(10, 16, seed=11), None),
    "rmat11_sym_s5": (lambda: bw.HostGraph.rmat(11, 8, seed=5, symmetrise=True), None),
    "er2000_s4": (lambda: bw.HostGraph.erdos_renyi(2000, 16000, seed=4), None),
    "grid30x33": (lambda: bw.HostGraph.grid(30, 33), 0),
    "ba3000_m3_s8": (lambda: bw.HostGraph.barabasi_albert(3000, 3, seed=8), None),
}


def main(out_dir: Path) -> None:
    out_dir.mkdir(parents=True, exist_ok=True)
    ref = ref_runner.ReferenceKernels()
    for name, (make, root) in GRAPHS.items():
        h = make()
        r = h.max_out_degree_vertex() if root is None else root
        dg = ref.upload_graph(h.vertex_count, h.fwd_vertices, h.fwd_edges, h.rev_vertices, h.rev_edges)
        levels, counts = None, None
        for v in ref_runner.bfs_variant_names():
            lv, cnt = ref.bfs(dg, v, r)
            if levels is None:
                levels, counts = lv, cnt
            elif not (np.array_equal(lv, levels) and np.array_equal(cnt, counts)):
                raise AssertionError(f"reference BFS variants disagree on {name}: {v}")
        arrays = dict(n=np.int64(h.vertex_count), root=np.int64(r), iterations=np.int64(ITERATIONS),
                      fwd_vertices=h.fwd_vertices.copy(), fwd_edges=h.fwd_edges.copy(),
                      rev_vertices=h.rev_vertices.copy(), rev_edges=h.rev_edges.copy(),
                      bfs_levels=levels, bfs_counts=counts)
        for v in ref_runner.PR_VARIANTS:
            pr, _ = ref.pagerank(dg, v, ITERATIONS)
            arrays["pr_" + v] = pr
        np.savez_compressed(out_dir / f"{name}.npz", **arrays)
        print("recorded", name, h.vertex_count, h.edge_count, len(counts), "levels")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent)
