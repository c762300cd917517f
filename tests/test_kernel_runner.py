"""kernel-runner and the plugin libraries (libbfskernel.so,
libpagerankkernel.so): discovery and registry on the CPU, end-to-end runs on
the GPU with the reference's file formats."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import belewitte_gb300 as bw
import oracle
from belewitte_gb300 import build

PKG = Path(bw.__file__).resolve().parent
RUNNER = PKG / "kernel-runner"


@pytest.fixture(scope="module", autouse=True)
def plugins():
    build.build_core()
    build.build_plugins()
    assert RUNNER.exists()


def run(*args, stdin=None, cwd=None):
    return subprocess.run([str(RUNNER), "-L", str(PKG), *args], capture_output=True, text=True, input=stdin,
                          cwd=cwd, timeout=600)


def test_list_and_query():
    out = run("list", "algorithms")
    assert out.returncode == 0 and out.stdout.split() == ["bfs", "pagerank"]
    impls = run("list", "implementations", "-a", "bfs").stdout.split()
    assert len(impls) == 35 and "switch" in impls and "vertex-pull-warp-blockreduce" in impls
    impls = run("list", "implementations", "-a", "pagerank").stdout.split()
    assert {"edge-list", "vertex-pull-nodiv", "vertex-pull-warp-nodiv", "switch"} <= set(impls)
    ver = run("query", "algorithm-version", "-a", "bfs")
    assert ver.returncode == 0 and ver.stdout.strip().startswith("belewitte-gb300")


def test_unknown_kernel_is_reported():
    out = run("-a", "bfs", "-k", "no-such-kernel", "x.graph")
    assert out.returncode != 0


def _write_graph(tmp_path, h, name="g"):
    p = tmp_path / f"{name}.graph"
    h.write(p)
    return p


@pytest.mark.gpu
def test_bfs_end_to_end(tmp_path):
    h = bw.HostGraph.rmat(12, 16, seed=21)
    p = _write_graph(tmp_path, h)
    root = h.max_out_degree_vertex()
    lv, cnt = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, root)
    for kernel in ["edge-list", "vertex-pull-warp-bulk", "frontier-push"]:
        out = run("-a", "bfs", "-k", kernel, "-r", str(root), "-o", str(tmp_path), str(p))
        assert out.returncode == 0, out.stderr
        rows = np.loadtxt(tmp_path / "g.output", dtype=np.int64)
        assert np.array_equal(rows[:, 0], np.arange(h.vertex_count))
        assert np.array_equal(rows[:, 1], lv.astype(np.int64)), kernel
        timings = (tmp_path / "g.timings").read_text().splitlines()
        names = {line.split(":")[0] if not line[0].isdigit() else ":".join(line.split(":")[:2])
                 for line in timings}
        assert "computation" in names and "0:bfsLevel" in names
        for line in timings:       # name:min mean max stddev (ns)
            vals = line.rsplit(":", 1)[1].split()
            assert len(vals) == 4 and all(v.isdigit() for v in vals)


@pytest.mark.gpu
def test_pagerank_end_to_end(tmp_path):
    h = bw.HostGraph.rmat(11, 16, seed=4)
    p = _write_graph(tmp_path, h)
    want, _ = oracle.pagerank(oracle.PR_DIV, h.vertex_count, h.rev_vertices, h.rev_edges, 100)
    out = run("-a", "pagerank", "-k", "vertex-pull", "--validate", "-o", str(tmp_path), str(p))
    assert out.returncode == 0, out.stderr
    lines = (tmp_path / "g.output").read_text().splitlines()
    assert lines[5] == f"5\t{oracle.format_rank(want[5])}"
    got = np.array([float(x.split("\t")[1]) for x in lines])
    assert np.allclose(got, want, rtol=1e-6)
    # default output: ids ordered by masked rank, 1000-entry buckets re-sorted by id
    out = run("-a", "pagerank", "-k", "vertex-pull", "-i", "30", "-o", str(tmp_path), str(p))
    ids = [int(x) for x in (tmp_path / "g.output").read_text().split()]
    assert sorted(ids) == list(range(h.vertex_count))


@pytest.mark.gpu
def test_stdin_jobs_and_switch_log(tmp_path):
    h = bw.HostGraph.grid(20, 25)
    p = _write_graph(tmp_path, h, "grid")
    log = tmp_path / "props.log"
    jobs = f"job1 -a bfs -k vertex-push -r 3 {p}\njob2 -a bfs -k switch -r 3 -l {log} {p}\n"
    out = run("-S", "-o", str(tmp_path), stdin=jobs)
    assert out.returncode == 0, out.stderr
    assert [line.rsplit(":", 1)[1] for line in out.stdout.split()] == ["job1", "job2"]
    lv, cnt = oracle.bfs(h.vertex_count, h.fwd_vertices, h.fwd_edges, 3)
    for job in ("job1", "job2"):
        rows = np.loadtxt(tmp_path / f"{job}.output", dtype=np.int64)
        assert np.array_equal(rows[:, 1], lv.astype(np.int64))
    text = log.read_text().splitlines()
    assert any(t.startswith("graph:vertex count:") for t in text)
    assert any(t.startswith("step:1:frontier abs:") for t in text)
    assert any(t.startswith("prediction:0:") for t in text)
