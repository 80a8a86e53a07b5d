"""The multi-GPU form of the benchmark is independent replicas (the operator
does not shard without a halo exchange): each rank times its own sweep, the
job's time is the max over ranks, the rate counts every rank's work.  The
aggregation runs here on CPU with two gloo ranks; the reference arm does its
work on rank 0 only."""

from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_s = 1.0 + rank                      # rank 1 finishes last
        job_s = bench.max_over_ranks(local_s, "cpu")
        out[rank] = (job_s, bench.replica_rate(100.0, job_s, world))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_aggregate_by_the_slowest_rank():
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (2.0, 100.0)       # 2 x 100 units in 2 s


def test_single_process_is_unchanged():
    import bench
    assert bench.max_over_ranks(3.5, "cpu") == 3.5
    assert bench.replica_rate(10.0, 2.0, 1) == 5.0


def test_reference_arm_does_no_work_off_rank_zero(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    calls = []
    monkeypatch.setattr(bench, "run_oracle_sweep", lambda *a, **k: calls.append(a))

    class Args:
        cpu_scale, warmup, steps = 4, 1, 1
    bench.reference_arm(Args())
    assert not calls and capsys.readouterr().out == ""
