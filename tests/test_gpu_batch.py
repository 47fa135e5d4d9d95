"""Batched and served proving (whir_batch_prove / whir_serve) on the GPU.

Every job's proof must be byte-identical to the same job proved alone by
the plain prover (and, for the small ones, to the oracle), whichever worker
ran it and whatever ran beside it.
"""
import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


def mixed_jobs(oracle, seed, n, ks=(10, 12, 14, 16), arrival_gap=0.0):
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(n):
        k = int(rng.choice(ks))
        rate = int(rng.choice([1, 2]))
        claims = int(rng.integers(1, 5))
        commit_only = bool(i % 7 == 3)
        poly = oracle.rand_fe(1000 + seed * 100 + i, 1 << k)
        jobs.append(W.Job((k, 4, rate, 1, 1, 100), poly, claims=claims,
                          commit_only=commit_only, arrival_s=i * arrival_gap))
    return jobs


def alone(ctx, job):
    p = job.params
    params = (p.k, p.folding, p.rate, p.initial_reduction, p.soundness, p.security_level)
    if job.commit_only:
        w = W.Whir(ctx, *params)
        t = W.PoseidonWriter()
        w.commit(t, [job.poly], [p.k])
        cp = t.draw_base()
        return t.finalize(), cp
    return W.prove_harness(ctx, params, [job.poly], [p.k], [[0]] * job.claims)


def test_batch_matches_alone(ctx, oracle):
    jobs = mixed_jobs(oracle, 1, 24)
    W.prove_jobs(jobs, workers=4)
    for j in jobs:
        assert j.status == 0
        proof, cp = alone(ctx, j)
        assert j.proof == proof
        assert j.checkpoint == cp
        if not j.commit_only:
            p = j.params
            params = (p.k, p.folding, p.rate, p.initial_reduction, p.soundness, p.security_level)
            assert W.verify(params, [p.k], [[0]] * j.claims, j.proof) == (0, cp)


def test_batch_matches_oracle(oracle):
    jobs = mixed_jobs(oracle, 2, 6, ks=(10, 12))
    W.prove_jobs(jobs, workers=3)
    for j in jobs:
        if j.commit_only:
            continue
        p = j.params
        want, wcp = oracle.prove((p.k, p.folding, p.rate, 1, 1, 100), [j.poly], [p.k],
                                 [[0]] * j.claims)
        assert j.proof == want and j.checkpoint == wcp


def test_batch_mixed_parameters(oracle):
    # jobs of different foldings (1..6), initial reductions, soundness modes
    # and security levels share the pool's provers, whose buffers are grown
    # to the union of the shapes before the run
    shapes = [(12, 5, 1, 3, 1, 100), (11, 3, 2, 2, 0, 32), (13, 6, 1, 1, 2, 64),
              (10, 1, 1, 1, 1, 32), (14, 4, 2, 1, 1, 100), (12, 2, 3, 2, 2, 80)]
    jobs = [W.Job(p, oracle.rand_fe(50 + i, 1 << p[0]), claims=1 + i % 3)
            for i, p in enumerate(shapes * 2)]
    W.prove_jobs(jobs, workers=3)
    for j in jobs:
        p = j.params
        params = (p.k, p.folding, p.rate, p.initial_reduction, p.soundness, p.security_level)
        want, wcp = oracle.prove(params, [j.poly], [p.k], [[0]] * j.claims)
        assert j.status == 0
        assert j.proof == want and j.checkpoint == wcp


def test_served_stream_same_as_batch(oracle):
    a = mixed_jobs(oracle, 3, 16, arrival_gap=0.004)
    b = mixed_jobs(oracle, 3, 16)
    W.prove_jobs(a, workers=4, serve=True)
    W.prove_jobs(b, workers=2)
    for x, y in zip(a, b):
        assert x.status == 0 and y.status == 0
        assert x.start_s >= x.arrival_s - 1e-3
        assert x.proof == y.proof and x.checkpoint == y.checkpoint


def test_device_resident_inputs(ctx, oracle):
    jobs = mixed_jobs(oracle, 4, 6, ks=(12, 14))
    dev = [ctx.to_device(j.poly) for j in jobs]
    host_proofs = []
    W.prove_jobs(jobs, workers=2)
    host_proofs = [(j.proof, j.checkpoint) for j in jobs]
    for j, d in zip(jobs, dev):
        j.poly = d
    W.prove_jobs(jobs, workers=3)
    for j, hp in zip(jobs, host_proofs):
        assert (j.proof, j.checkpoint) == hp


def test_budget_too_small_fails_job_only(oracle):
    jobs = mixed_jobs(oracle, 5, 3, ks=(12,))
    need = W.workspace_bytes(jobs[0].params)
    big = W.Job((16, 4, 2, 1, 1, 100), oracle.rand_fe(9, 1 << 16), claims=1)
    W.prove_jobs(jobs + [big], workers=2, budget_bytes=need + (1 << 20))
    assert all(j.status == 0 for j in jobs)
    assert big.status == -4


def test_server_reuse_across_runs(oracle):
    srv = W.Server(workers=3)
    try:
        a = mixed_jobs(oracle, 6, 10)
        srv.run(a)
        b = mixed_jobs(oracle, 6, 10)
        srv.run(b, serve=True)   # warm workers, arrivals all at 0
        c = mixed_jobs(oracle, 7, 8, ks=(16, 10))
        srv.run(c)
        for x, y in zip(a, b):
            assert x.status == 0 and x.proof == y.proof and x.checkpoint == y.checkpoint
        d = mixed_jobs(oracle, 7, 8, ks=(16, 10))
        W.prove_jobs(d, workers=1)
        for x, y in zip(c, d):
            assert x.proof == y.proof and x.checkpoint == y.checkpoint
    finally:
        srv.close()


def test_server_reuse_with_growing_folding(ctx, oracle):
    # one pool, three runs whose foldings grow (2, then 6, then 5) and mix
    # commit-only jobs in: every proof equals the oracle's (full proofs) or
    # the plain prover's (commitments)
    srv = W.Server(workers=2)
    try:
        runs = [[(11, 2, 1, 1, 1, 100), (10, 2, 2, 2, 0, 32)],
                [(13, 6, 1, 1, 1, 100), (12, 6, 1, 3, 2, 64)],
                [(12, 5, 2, 1, 1, 100), (11, 5, 1, 5, 0, 32)]]
        for r, shapes in enumerate(runs):
            jobs = [W.Job(p, oracle.rand_fe(70 + 10 * r + i, 1 << p[0]), claims=1 + i % 2,
                          commit_only=(i == 2))
                    for i, p in enumerate(shapes + shapes[:1])]
            srv.run(jobs)
            for j in jobs:
                assert j.status == 0
                if j.commit_only:
                    proof, cp = alone(ctx, j)
                else:
                    p = j.params
                    params = (p.k, p.folding, p.rate, p.initial_reduction, p.soundness,
                              p.security_level)
                    proof, cp = oracle.prove(params, [j.poly], [p.k], [[0]] * j.claims)
                assert j.proof == proof and j.checkpoint == cp
    finally:
        srv.close()


def test_run_with_parameters_the_reference_cannot_run_is_refused(oracle):
    # initial_reduction 5 > rate + folding: the whole run is refused before
    # any job starts, and the pool still works afterwards
    good = W.Job((10, 2, 1, 1, 1, 32), oracle.rand_fe(1, 1 << 10))
    bad = W.Job((10, 2, 1, 5, 1, 32), oracle.rand_fe(2, 1 << 10))
    with pytest.raises(W.WhirError):
        W.prove_jobs([good, bad], workers=2)
    W.prove_jobs([good], workers=2)
    want, wcp = oracle.prove((10, 2, 1, 1, 1, 32), [good.poly], [10], [[0]])
    assert good.status == 0 and good.proof == want and good.checkpoint == wcp


@pytest.mark.parametrize("params,n", [((16, 4, 2, 1, 1, 100), 4), ((14, 4, 1, 1, 0, 1200), 2),
                                      ((16, 8, 1, 1, 1, 100), 2), ((12, 3, 1, 1, 1, 32), 20),
                                      ((18, 6, 2, 2, 1, 100), 3), ((12, 4, 0, 1, 1, 100), 2)])
def test_workspace_plan_covers_a_proof(oracle, params, n):
    # admission charges a job whir_workspace_bytes; the device memory its
    # worker holds after the proof (many queries, many claims, large
    # foldings, rate 1 included) must not exceed it
    j = W.Job(params, oracle.rand_fe(3, 1 << params[0]), claims=n)
    _, peak = W.prove_jobs([j], workers=1)
    assert j.status == 0
    assert peak <= W.workspace_bytes(params)


@pytest.mark.parametrize("lockstep", [1, 3, 0])
def test_server_lockstep_groups_match_alone(ctx, oracle, lockstep):
    # many jobs of a few shapes released together: with lock step the server
    # proves same-shape jobs as groups (at most 3 per group, or the default),
    # without it one at a time; every proof equals the job proved alone
    rng = np.random.default_rng(40 + lockstep)
    jobs = []
    for i in range(20):
        k = int(rng.choice([10, 12]))
        claims = int(rng.choice([1, 2]))
        jobs.append(W.Job((k, 4, 1, 1, 1, 100), oracle.rand_fe(5000 + i, 1 << k), claims=claims,
                          commit_only=(i % 9 == 4)))
    srv = W.Server(workers=3, lockstep=lockstep)
    try:
        srv.run(jobs)
    finally:
        srv.close()
    for j in jobs:
        assert j.status == 0
        assert (j.proof, j.checkpoint) == alone(ctx, j)
