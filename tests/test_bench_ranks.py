"""bench.py's multi-GPU aggregation (replicas: one rank per GPU, no collective on the data path)
on CPU with gloo, world size 2: the job's time is the slowest rank's, its rate counts every rank's
frames."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, results):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        local_ms = 100.0 + 25.0 * rank           # rank 1 is the slow one
        ms = bench.reduce_max(local_ms, device="cpu")
        rate = bench.job_throughput(50, world, ms)
        dist.barrier()
        results[rank] = (ms, rate)
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_count_all_frames():
    import torch.multiprocessing as mp
    world = 2
    manager = mp.get_context("spawn").Manager()
    results = manager.dict()
    mp.spawn(_rank, args=(world, _free_port(), results), nprocs=world, join=True)
    for rank in range(world):
        ms, rate = results[rank]
        assert ms == 125.0
        assert rate == pytest.approx(world * 50 / 0.125)


def test_single_process_is_the_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(42.5, device="cpu") == 42.5
    assert bench.job_throughput(10, 1, 1000.0) == pytest.approx(10.0)
