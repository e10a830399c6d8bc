"""bench.py's multi-GPU path on two gloo ranks on the CPU: each rank takes a
round-robin shard of the roots, the job's count and hash are the sums of the
ranks' shares (the hash a wrapping sum), the step time is the slowest
rank's, and the whole job's throughput is the total count over that time.
The shards' results are checked with the oracle: together they are exactly
the whole graph's."""
import os
import socket
import sys

import numpy as np
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
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import oracle
    csr = oracle.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1)
    shard = bench.shard_of(rank, world)
    r = oracle.ref_enumerate_roots(*csr, root_begin=shard["root_begin"], root_stride=shard["root_stride"],
                                   threads=2)
    ms = bench.max_over_ranks(100.0 + 50.0 * rank, world, "cpu")  # rank 1 is the slower rank
    count = bench.sum_over_ranks(r.count, world, "cpu")
    h = r.hash - (1 << 64) if r.hash >= (1 << 63) else r.hash
    hsum = bench.sum_over_ranks(h, world, "cpu") % (1 << 64)
    out[rank] = (ms, count, hsum, bench.sharded_value(count, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_the_roots_and_sum_to_the_whole_graph():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    full = oracle.ref_enumerate(*oracle.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1), threads=4)
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    for r in range(world):
        ms, count, h, value = out[r]
        assert ms == 150.0
        assert (count, h) == (full.count, full.hash)
        assert value == pytest.approx(full.count / 0.150)


def test_one_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
    assert bench.sum_over_ranks(7, 1, "cpu") == 7
    assert bench.shard_of(0, 1) == {}
    assert bench.sharded_value(1000, 500.0) == 2000.0
