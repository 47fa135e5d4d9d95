"""The multi-GPU path is replicas only: each rank proves its own proofs and
rank 0 reports world * steps / (slowest rank's time).  The cross-rank part
of bench.py runs here on two gloo processes on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        slowest = bench.max_over_ranks(times[rank], world, "cpu")
        dist.barrier()
        out[rank] = (slowest, bench.replica_throughput(world, 10, slowest))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world, times = 2, [0.25, 0.4]
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), times, out), nprocs=world, join=True)
    for r in range(world):
        slowest, value = out[r]
        assert slowest == pytest.approx(0.4)
        assert value == pytest.approx(2 * 10 / 0.4)


def test_single_rank_is_a_no_op():
    import bench
    assert bench.max_over_ranks(1.5, 1, "cpu") == 1.5
    assert bench.replica_throughput(1, 30, 0.5) == 60
