"""Multi-GPU is replicas only: N ranks each solve their own right-hand sides,
with no collective in the data path; the only exchange is the max over ranks
of the timed totals. Checked here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local = 100.0 + 50.0 * rank  # the second replica is slower
    total = bench.aggregate_replicas(local, dist, device="cpu")
    out[rank] = (total, bench.replica_value(32, 5, world, total))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    world = 2
    out = mp.get_context("spawn").Manager().dict()  # no fork of this (threaded) process
    mp.spawn(_rank, args=(world, _port(), out), nprocs=world, join=True)
    for r in range(world):
        total, value = out[r]
        assert total == 150.0                              # the slowest replica
        assert value == pytest.approx(2 * 32 * 5 / 0.150)  # all replicas' solves over that time


def test_reference_arm_prints_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")

    class Args:
        gpus, steps, warmup = 2, 1, 0
    bench.run_reference(Args())
    assert capsys.readouterr().out == ""
