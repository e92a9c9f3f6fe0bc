"""Multi-rank plumbing of bench.py on CPU: two gloo ranks (replicas) aggregate
units and take the slowest rank's time, as the GPU benchmark does under
torchrun; the reference arm runs on rank 0 only."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, results):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units, seconds = 1000 * (rank + 1), 0.5 + rank
    total, slowest = bench.aggregate_over_ranks(units, seconds, dist, "cpu")
    dist.barrier()
    results[rank] = (total, slowest)
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_the_benchmark():
    import torch.multiprocessing as mp

    port = _free_port()
    with mp.Manager() as manager:
        results = manager.dict()
        mp.spawn(_rank_main, args=(2, port, results), nprocs=2, join=True)
        assert dict(results) == {0: (3000.0, 1.5), 1: (3000.0, 1.5)}


def test_single_process_aggregate_is_identity():
    import bench

    assert bench.aggregate_over_ranks(7, 0.25) == (7, 0.25)


def test_reference_arm_prints_only_on_rank_zero(capsys, monkeypatch):
    import argparse

    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(gpus=2, steps=1, warmup=0)
    assert bench.run_reference(args) == 0
    assert capsys.readouterr().out == ""
