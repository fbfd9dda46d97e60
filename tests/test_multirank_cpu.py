"""The N > 1 path of bench.py (replicas: one map instance per GPU, no data
exchange) on CPU with world size 2 over gloo: the whole-job reduction takes
the slowest rank's time and every rank's points; rank and world come from
the launcher's environment; the reference arm runs on rank 0 only."""
import os
import socket

import pytest

from conftest import REPO


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, REPO)
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    import bench
    t, p = bench._reduce_max_sum(torch, dist, 1.0 + rank, 100 * (rank + 1))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, p))


def test_whole_job_reduction_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for pr in procs:
        pr.join(60)
        assert pr.exitcode == 0
    assert out == [(0, 2.0, 300.0), (1, 2.0, 300.0)]


def test_rank_and_world_from_the_launcher_environment(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "3")
    monkeypatch.setenv("WORLD_SIZE", "4")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.env_rank() == (3, 4, 1)
    monkeypatch.delenv("LOCAL_RANK")
    assert bench.env_rank() == (3, 4, 3)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import types

    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = types.SimpleNamespace(workload="os1_64_veg", steps=1, warmup=0)
    assert bench.run_reference(args) == 0  # returns before building any workload
