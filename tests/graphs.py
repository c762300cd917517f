"""Small seeded test graphs shared by the CPU and GPU tests."""
import numpy as np

import belewitte_gb300 as bw


def chain(n):
    """evolve/gen-graph.cpp:72-82 chain (directed i -> i+1)."""
    src = np.arange(n - 1, dtype=np.uint32)
    return bw.HostGraph.from_edges(n, src, src + 1)


def star(n):
    """evolve/gen-graph.cpp:84-94 star (directed 0 -> i)."""
    dst = np.arange(1, n, dtype=np.uint32)
    return bw.HostGraph.from_edges(n, np.zeros(n - 1, np.uint32), dst)


def star_in(n):
    """Every leaf points at vertex 0: one in-row of n - 1 equal terms."""
    src = np.arange(1, n, dtype=np.uint32)
    return bw.HostGraph.from_edges(n, src, np.zeros(n - 1, np.uint32))


def catalog():
    """name -> (constructor, root) of the small parity graphs."""
    return {
        "rmat10": (lambda: bw.HostGraph.rmat(10, 16, seed=11), None),
        "rmat12_sym": (lambda: bw.HostGraph.rmat(12, 8, seed=5, symmetrise=True), None),
        "rmat14": (lambda: bw.HostGraph.rmat(14, 16, seed=2), None),
        "er": (lambda: bw.HostGraph.erdos_renyi(5000, 40000, seed=4), None),
        "grid": (lambda: bw.HostGraph.grid(40, 37), 0),
        "ba": (lambda: bw.HostGraph.barabasi_albert(6000, 3, seed=8), None),
        "chain": (lambda: chain(300), 0),
        "star": (lambda: star(2000), 0),
        "tiny": (lambda: bw.HostGraph.from_edges(5, [0, 1, 2, 3, 0], [1, 2, 3, 0, 4]), 0),
        "isolated": (lambda: bw.HostGraph.from_edges(7, [1, 2], [2, 3]), 0),
    }


def root_of(g, root):
    return g.max_out_degree_vertex() if root is None else root
