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


def _prove_rank(rank, world, port, out):
    # each replica proves its own polynomials (the oracle stands in for the
    # GPU prover on the CPU), times them, and the job is accounted as
    # bench.py accounts it: the slowest rank's time, every rank's proofs
    import time
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from oracle import oracle as O
        O.lib().wo_set_threads(1)
        params, steps = (10, 4, 1, 1, 1, 100), 3
        dist.barrier()
        t0 = time.perf_counter()
        proofs = [O.prove(params, [O.rand_fe(100 * rank + s, 1 << 10)], [10], [[0]])
                  for s in range(steps)]
        el = time.perf_counter() - t0
        slowest = bench.max_over_ranks(el, world, "cpu")
        # every rank's proofs reach rank 0 (a replica's proofs are its own)
        gathered = [None] * world
        dist.all_gather_object(gathered, [p[0] for p in proofs])
        out[rank] = (el, slowest, bench.replica_throughput(world, steps, slowest), gathered)
    finally:
        dist.destroy_process_group()


def test_two_replicas_prove_independently():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_prove_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    from oracle import oracle as O
    els = [out[r][0] for r in range(world)]
    for r in range(world):
        el, slowest, value, gathered = out[r]
        assert slowest == pytest.approx(max(els))
        assert value == pytest.approx(world * 3 / max(els))
        # the same proofs on every rank, and each is the oracle's for its seed
        assert gathered == out[0][3]
    for rank in range(world):
        for s in range(3):
            want = O.prove((10, 4, 1, 1, 1, 100), [O.rand_fe(100 * rank + s, 1 << 10)], [10],
                           [[0]])[0]
            assert out[0][3][rank][s] == want
    assert out[0][3][0][0] != out[0][3][1][0]  # the replicas' work differs
