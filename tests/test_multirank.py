"""The N > 1 path of bench.py on CPU: two gloo ranks, as the driver launches
one rank per GPU.  The path does not shard a graph (independent replicas,
weak scaling): the only collectives are the barrier and the max-over-ranks
of the timings, and the reference arm runs on rank 0 alone."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        slowest = bench.max_over_ranks(1.5 + rank, world)          # rank 1 is the slow one
        gteps = bench.replica_throughput(world, 1_000_000, 30, slowest * 1e-3)
        out.put((rank, slowest, gteps))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_report_the_slowest_and_the_whole_job():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slowest, gteps in got:
        assert slowest == pytest.approx(2.5)
        # two replicas of 30 M edge-iterations in 2.5 ms
        assert gteps == pytest.approx(2 * 30e6 / 2.5e-3 / 1e9)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class Args:
        steps, warmup = 1, 3
    bench.run_reference(Args())               # rank 1: no work, no output
    assert capsys.readouterr().out == ""
