"""The multi-GPU form of bench.py is replicas: every rank casts its own copy of the batch and the
job's time is the slowest rank's.  The host-side reduction runs here as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        dist.barrier()
        out[rank] = bench.max_over_ranks(times[rank], dist)
    finally:
        dist.destroy_process_group()


def test_job_time_is_the_slowest_replica():
    world = 2
    times = [0.25, 0.75]
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, _free_port(), times, out), nprocs=world, join=True)
        assert dict(out) == {0: 0.75, 1: 0.75}


def test_single_process_keeps_its_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5, None) == 1.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        steps, warmup = 1, 1
    bench.run_reference(Args(), bench.WORKLOADS["heightfield128"])  # rank 1 returns without work
    assert capsys.readouterr().out == ""
