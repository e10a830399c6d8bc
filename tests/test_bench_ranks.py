"""bench.py's multi-GPU path (one replica per GPU, the slowest replica's step
time, the whole job's throughput) on two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms = bench.max_over_ranks(100.0 + 50.0 * rank, world, "cpu")  # rank 1 is the slower replica
    out[rank] = (ms, bench.replicas_value(60582677, world, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_step_and_sum_the_work():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    for r in range(world):
        ms, value = out[r]
        assert ms == 150.0
        assert value == pytest.approx(60582677 * 2 / 0.150)


def test_one_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
    assert bench.replicas_value(1000, 1, 500.0) == 2000.0
