"""bench.py's multi-GPU form is replicas only (a build does not shard): each rank
builds its own dataset and the only collectives are the barrier around the
timed region and the max over ranks of the timing.  Cover that host logic with
two gloo ranks on CPU (127.0.0.1 rendezvous)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    g = bench.Group("gloo")
    assert (g.ws, g.rank) == (world, rank)
    g.barrier()
    t = g.max(1.5 + rank)  # each replica's own time; the job's time is the slowest
    g.barrier()
    g.close()
    out.put((rank, t))


def test_two_rank_barrier_and_max():
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 2.5, 1: 2.5}


def test_single_rank_group_is_a_no_op(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "1")
    sys.path.insert(0, ROOT)
    import bench

    g = bench.Group("gloo")
    g.barrier()
    assert g.max(3.0) == 3.0
    g.close()


def test_reference_arm_other_ranks_exit_without_work(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    sys.path.insert(0, ROOT)
    import bench

    class A:
        gpus, steps, warmup, config = 2, 1, 0, "full"

    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""
