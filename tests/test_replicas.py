"""Multi-GPU form of the benchmark: independent replicas, one per rank, no
data-path collective; the job's time is the slowest rank's.  Exercised with
two gloo ranks on the CPU (the aggregation is the only cross-rank step)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t, value = bench.replica_throughput(times[rank], 10, world, dist, device="cpu")
        out[rank] = (t, value)
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    times = [0.5, 0.8]
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(2, _free_port(), times, out), nprocs=2, join=True)
    for r in range(2):
        t, value = out[r]
        assert t == pytest.approx(0.8)
        assert value == pytest.approx(10 * 2 / 0.8)


def test_single_replica_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(0.25, 5, 1) == (0.25, 20.0)
