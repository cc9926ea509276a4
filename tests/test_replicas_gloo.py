"""The multi-GPU form of the bench is replicas (the path has no cross-GPU
exchange in this form): every rank reconstructs its own copy, the
step time is the max over ranks and the value counts every rank's
iterations.  The cross-rank part runs here on two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    # rank r's replica took (1 + r) s per step and (2 + r / 2) s end to end
    tmax, rates = bench.aggregate_replicas((1.0 + rank, 2.0 + 0.5 * rank), 20, world, dist, "cpu")
    q.put((rank, tmax, rates))
    dist.destroy_process_group()


def test_replicas_time_is_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = [q.get(timeout=120) for _ in procs]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    for rank, tmax, rates in out:
        assert tmax == [2.0, 2.5]                      # the slower replica
        assert rates == [2 * 20 / 2.0, 2 * 20 / 2.5]   # both ranks' iterations


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    bench.reference_arm(bench.parse())  # returns at once: no work, no output
    assert capsys.readouterr().out == ""
