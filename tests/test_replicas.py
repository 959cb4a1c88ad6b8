"""The replica mode of bench.py (one independent channel per rank, no
collective on the data path): the job's time is the slowest rank's, the
job's rate counts every rank's steps, and the reference arm runs on rank 0
only.  Two gloo ranks on the CPU (127.0.0.1)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist
import torch.multiprocessing as mp


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank  # rank 1 is the slow replica
        t = bench.max_over_ranks(ms, tdist, "cpu")
        out[rank] = (t, bench.replica_rate(world, 100, t / 1e3), bench.dist_env())
    finally:
        tdist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    world = 2
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        t, rate, env = res[rank]
        assert t == 15.0  # the max over the ranks
        assert rate == pytest.approx(2 * 100 / 0.015)  # both ranks' steps over the slowest time
        assert env == (rank, world, rank)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    called = []
    monkeypatch.setattr(bench, "cpu_reference_rate", lambda *a, **k: called.append(a))
    import argparse
    ns = argparse.Namespace(config="c1_poiseuille_32", grid=None, warmup=1, steps=1, impl="reference")
    assert bench.run_reference(ns) == 0
    assert not called


def test_max_over_ranks_without_a_group():
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.replica_rate(1, 50, 0.5) == 100.0
