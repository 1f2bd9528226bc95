"""Multi-replica aggregation of bench.py on CPU: two gloo ranks with different step
times; the job time is the slowest rank's and the throughput counts both replicas."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [0.004, 0.006][rank]  # seconds per step on this rank
        t = bench.max_over_ranks(local, world, "cpu")
        out[rank] = (t, bench.replica_throughput(1e12, t, world))
    finally:
        dist.destroy_process_group()


def test_two_replicas_max_time_and_summed_throughput():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork of a process with OpenMP threads
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        t, v = res[rank]
        assert t == pytest.approx(0.006)
        assert v == pytest.approx(2 * 1e12 / 0.006)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(0.5, 1, "cpu") == 0.5
    assert bench.replica_throughput(10.0, 2.0, 1) == 5.0
