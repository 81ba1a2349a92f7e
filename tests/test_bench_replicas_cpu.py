"""bench.py's replica bookkeeping on two gloo ranks on the CPU: the job's
time per step is the slowest rank's, the whole-job throughput counts every
rank's sweep, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [700.0, 725.5][rank]
        slow = bench.slowest_replica_ms(ms, world, "cpu")
        out[rank] = (slow, bench.job_sweeps_per_s(slow, world))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world = 2
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True,
                       start_method="spawn")
    for r in range(world):
        slow, value = out[r]
        assert slow == 725.5
        assert value == pytest.approx(2 * 1e3 / 725.5)


def test_single_process_needs_no_collective():
    assert bench.slowest_replica_ms(700.0, 1, "cpu") == 700.0
    assert bench.job_sweeps_per_s(700.0, 1) == pytest.approx(1e3 / 700.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")
    called = []
    monkeypatch.setattr(bench, "cpu_sweep_estimate", lambda *a, **k: called.append(1))
    assert bench.run_reference(None, bench.CONFIGS["c5"]) == 0
    assert not called
