"""The multi-GPU form of the benchmark runs one replica of the lattice per rank (the path has
no exchange step at one lattice per GPU): the job time is the slowest rank's and the job
MLUPS counts every replica.  Checked here with two gloo ranks on the CPU."""
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
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = 1.0 + 0.5 * rank  # rank 1 is the slow one
        t = bench.max_over_ranks(seconds, world, "cpu")
        out[rank] = (t, bench.job_mlups(4096 * 4096 * 10, t, world))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        t, mlups = res[r]
        assert t == 1.5
        assert mlups == pytest.approx(4096 * 4096 * 10 * 2 / 1.5 / 1e6, rel=1e-15)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(2.5, 1, "cpu") == 2.5
    assert bench.job_mlups(1e6, 2.0, 1) == 0.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun the reference arm's other ranks exit 0 without work or output."""
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class A:
        gpus, steps, warmup = 2, 3, 3
    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""
