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


def test_reference_arm_json_line(monkeypatch, capsys):
    """bench.py --impl reference: one JSON line with the arm's metric, the
    steps and warm-up it was given, the CPU baseline it measured and an e2e
    block without host-device copies. Run in-process on a smaller sphere
    (M = 3, P = 1, n_p = 6) so that it takes seconds; the line's structure is
    what is checked."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.setattr(bench, "M", 3)
    monkeypatch.setattr(bench, "P", 1)
    monkeypatch.setattr(bench, "NP", 6)

    class Args:
        gpus, steps, warmup = 1, 2, 1
    bench.run_reference(Args())
    out = capsys.readouterr().out
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["unit"] == "solves/s" and j["higher_is_better"] is True
    assert j["steps"] == 2 and j["warmup"] == 1 and j["value"] > 0
    assert j["cpu_baseline"]["value"] == j["value"] and j["cpu_baseline"]["cores"] >= 1
    assert j["cpu_baseline"]["kind"] == "port" and j["cpu_baseline"]["sample"]
    assert j["e2e"] == {"value": j["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert j["config"]["workload"] == "laplace_sl_h2_sphere_M5_P2_np9_32rhs"
    assert j["full_solve"]["iterations"] > 0 and j["full_solve"]["final_relres"] <= 1e-8
    assert "measured" in j["cpu_baseline"]["sample"]


def test_bench_column_errors():
    """The accuracy figures of the bench line: largest column-wise relative error."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    ref = np.array([[1.0, 0.0], [0.0, 2.0]])
    a = np.array([[1.0, 0.0], [0.1, 2.0]])
    assert abs(bench.col_rel_err(a, ref) - 0.1) < 1e-15
    assert bench.col_rel_err(ref, ref) == 0.0
    assert abs(bench.col_rel_err(np.array([2.0, 0.0]), np.array([1.0, 0.0])) - 1.0) < 1e-15
