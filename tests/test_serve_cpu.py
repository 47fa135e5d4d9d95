"""Admission of the batched/served job runner, on the CPU.

whir_serve_simulate runs the same scheduler as whir_serve (arrival order,
free workers, a device-memory budget over grow-only worker buffers) with a
host sleep standing in for each proof, so the ordering and memory rules are
checked without a GPU.
"""
import numpy as np
import pytest

import whir_gb300 as W


def held_at_starts(start, need, worker, n_workers):
    """Total bytes held right after each job starts (buffers only grow)."""
    order = np.argsort(start, kind="stable")
    held = np.zeros(n_workers, dtype=np.int64)
    totals = []
    for j in order:
        held[worker[j]] = max(held[worker[j]], need[j])
        totals.append(held.sum())
    return totals


def test_fifo_and_arrival():
    rng = np.random.default_rng(3)
    n = 24
    arrival = np.sort(rng.uniform(0, 0.05, n))
    need = rng.integers(1, 10, n)
    dur = rng.uniform(0.001, 0.01, n)
    s, e, wk, st = W.serve_simulate(arrival, need, dur, 4, 10 ** 9)
    assert (st == 0).all()
    assert (s >= arrival - 1e-4).all()           # nothing starts before it arrives
    assert (np.diff(s[np.argsort(arrival, kind="stable")]) >= -1e-4).all()  # FIFO
    assert (e >= s + dur - 1e-4).all()
    assert set(wk) <= set(range(4))


def test_workers_overlap():
    n = 8
    s, e, wk, st = W.serve_simulate([0.0] * n, [1] * n, [0.02] * n, 4, 10 ** 9)
    assert (st == 0).all()
    # four at a time: the last four start after the first four end
    assert e.max() < 0.02 * n / 4 + 0.05
    assert len(set(wk)) == 4


def test_budget_bounds_held_bytes():
    rng = np.random.default_rng(7)
    n = 30
    arrival = np.zeros(n)
    need = rng.integers(10, 60, n)
    budget = 100
    s, e, wk, st = W.serve_simulate(arrival, need, [0.002] * n, 6, budget)
    assert (st == 0).all()
    assert max(held_at_starts(s, need, wk, 6)) <= budget


def test_budget_serialises_when_one_job_fills_it():
    n = 5
    s, e, wk, st = W.serve_simulate([0.0] * n, [100] * n, [0.01] * n, 3, 100)
    assert (st == 0).all()
    order = np.argsort(s)
    for a, b in zip(order[:-1], order[1:]):
        assert s[b] >= e[a] - 1e-4          # never two at once
    assert len(set(wk)) == 1                 # the first worker keeps the budget


def test_job_larger_than_budget_fails_alone():
    s, e, wk, st = W.serve_simulate([0.0, 0.0, 0.0], [5, 500, 5], [0.001] * 3, 2, 100)
    assert st[1] == -4                       # WHIR_ERR_CAPACITY
    assert st[0] == 0 and st[2] == 0


def test_workspace_and_proof_bounds():
    small = W.workspace_bytes((14, 4, 1, 1, 1, 100))
    big = W.workspace_bytes((24, 4, 2, 1, 1, 100))
    assert 0 < small < big < 4 << 30
    assert W.proof_bound((24, 4, 2, 1, 1, 100), 4) > W.proof_bound((24, 4, 2, 1, 1, 100), 1)
    with pytest.raises(W.WhirError):
        W.workspace_bytes((3, 4, 1, 1, 1, 100))   # k < folding


def test_proof_bound_covers_oracle_proofs(oracle):
    for (k, f, r, n) in [(10, 4, 1, 1), (12, 2, 1, 3), (13, 3, 2, 4)]:
        poly = oracle.rand_fe(k, 1 << k)
        proof, _ = oracle.prove((k, f, r, 1, 1, 100), [poly], [k], [[0]] * n)
        assert len(proof) <= W.proof_bound((k, f, r, 1, 1, 100), n)
    # other foldings, rates, reductions and soundness modes (a served job's
    # proof buffer is sized by this bound)
    for params in [(12, 5, 1, 5, 2, 32), (15, 6, 1, 1, 1, 100), (12, 7, 1, 2, 0, 32),
                   (16, 8, 1, 1, 1, 100), (12, 4, 0, 1, 1, 100), (12, 3, 1, 4, 1, 32),
                   (14, 4, 3, 1, 2, 100), (9, 1, 1, 1, 0, 32)]:
        k = params[0]
        for n in (1, 4):
            proof, _ = oracle.prove(params, [oracle.rand_fe(k, 1 << k)], [k], [[0]] * n)
            assert len(proof) <= W.proof_bound(params, n)


def test_short_polynomial_buffers_are_refused_before_the_library():
    # the C ABI reads 2^k words from the pointers it is given; the binding
    # checks the buffers' sizes first (no GPU needed: the check comes first)
    class FakeDev(W.DeviceArray):
        def __init__(self, nbytes):
            self.nbytes, self.ptr, self.ctx = nbytes, 0, None

        def close(self):
            pass

    with pytest.raises(W.WhirError):
        W.Whir._polys([np.zeros(100, np.uint32)], [7])
    with pytest.raises(W.WhirError):
        W.Whir._polys(np.zeros(100, np.uint32), [7])
    with pytest.raises(W.WhirError):
        W.Whir._polys(FakeDev(4 * 127), [7])
    assert W.Whir._polys([np.zeros(128, np.uint32), np.zeros(64, np.uint32)], [7, 6])[1] == 0
    with pytest.raises(W.WhirError):
        W._jobs_in([W.Job((12, 4, 1, 1, 1, 100), FakeDev(4 << 11))])


# ---- lock-step groups (whir_server_set_lockstep's admission) ----

def test_groups_take_arrived_jobs_of_one_shape():
    # eight jobs at t = 0: shapes 0,1,0,1,...; two workers, groups up to 4
    n = 8
    shape = [i % 2 for i in range(n)]
    s, e, wk, st = W.serve_simulate([0.0] * n, [1] * n, [0.03] * n, 2, 10 ** 9,
                                    shape=shape, max_group=4)
    assert (st == 0).all()
    for sh in (0, 1):
        members = [i for i in range(n) if shape[i] == sh]
        assert len({wk[i] for i in members}) == 1          # one worker per group
        assert np.ptp(s[members]) < 1e-3                   # started together
        assert np.ptp(e[members]) < 1e-3
    assert e.max() < 0.03 + 0.02                            # two groups side by side


def test_groups_respect_max_group_and_arrival():
    # 6 same-shape jobs at t = 0, one worker, groups of at most 4: the first
    # four together, then the last two; a job arriving later is not pulled in
    arrival = [0.0] * 6 + [0.2]
    s, e, wk, st = W.serve_simulate(arrival, [1] * 7, [0.02] * 7, 1, 10 ** 9,
                                    shape=[0] * 7, max_group=4)
    assert (st == 0).all()
    assert np.ptp(s[:4]) < 1e-3 and np.ptp(s[4:6]) < 1e-3
    assert s[4] >= e[0] - 1e-3
    assert s[6] >= 0.2 - 1e-4 and s[6] > e[5] - 1e-3


def test_groups_halve_to_fit_the_budget():
    # a group of 4 would hold 4 units; the budget holds 2: groups of 2
    n = 4
    s, e, wk, st = W.serve_simulate([0.0] * n, [1] * n, [0.02] * n, 1, 2,
                                    shape=[0] * n, max_group=4)
    assert (st == 0).all()
    assert np.ptp(s[:2]) < 1e-3 and np.ptp(s[2:]) < 1e-3
    assert s[2] >= e[0] - 1e-3


def test_groups_keep_heads_in_arrival_order():
    rng = np.random.default_rng(11)
    n = 40
    arrival = np.sort(rng.uniform(0, 0.05, n))
    shape = rng.integers(0, 3, n)
    s, e, wk, st = W.serve_simulate(arrival, [1] * n, rng.uniform(0.001, 0.005, n), 3, 10 ** 9,
                                    shape=shape, max_group=8)
    assert (st == 0).all()
    assert (s >= arrival - 1e-4).all()
    # a job never starts before an earlier-arrived job of another group
    # starts, except when it is grouped with a head that arrived first
    starts = {}
    for j in range(n):
        starts.setdefault(round(s[j], 4), []).append(j)
    heads = sorted(min(g) for g in starts.values())
    assert (np.diff([s[h] for h in heads]) >= -1e-4).all()


def test_job_that_no_idle_worker_can_hold_fails_instead_of_waiting():
    # two workers each keep 60 units after their first jobs (buffers only
    # grow); a later job needing 80 fits the budget of 130 alone, but on
    # either worker it would add 20 to 120: with nothing running no release
    # can make room, so it fails with the capacity status instead of waiting
    s, e, wk, st = W.serve_simulate([0.0, 0.0, 0.05], [60, 60, 80], [0.02, 0.02, 0.01], 2, 130)
    assert list(st[:2]) == [0, 0]
    assert st[2] == -4   # WHIR_ERR_CAPACITY
    assert e[2] < 1.0


def test_job_waits_for_the_worker_that_can_hold_it():
    # the same budget, but one worker keeps 80 units: a second 80-unit job
    # must wait for that worker (adding nothing there) and succeed
    s, e, wk, st = W.serve_simulate([0.0, 0.0], [80, 80], [0.03, 0.01], 2, 100)
    assert (st == 0).all()
    assert wk[0] == wk[1]
    assert s[1] >= e[0] - 1e-3


INTERNAL = -5  # WHIR_ERR_INTERNAL


def test_failed_proof_fails_only_its_job():
    # job 2 fails 5 ms into its proof (a transcript or I/O error, injected by
    # a negative duration); the other jobs finish, and its worker goes on
    # with later jobs
    n = 10
    dur = [0.005] * n
    dur[2] = -0.005
    s, e, wk, st = W.serve_simulate([0.0] * n, [10] * n, dur, 2, 10 ** 9)
    assert st[2] == INTERNAL
    assert all(st[j] == 0 for j in range(n) if j != 2)
    assert e[2] >= s[2] + 0.005 - 1e-4
    assert any(wk[j] == wk[2] and s[j] >= e[2] - 1e-4 for j in range(3, n))


def test_failed_proof_keeps_its_buffers_in_the_budget():
    # worker buffers only grow, and a proof that fails has grown its
    # worker's buffers first (admission reserved them when it handed the
    # job out): job 0 (need 60) fails on one worker, which then holds 60;
    # with a budget of 100 a second 60-byte job cannot start on the other
    # worker beside it, so every later job runs where the 60 bytes already are
    n = 5
    need = [60] * n
    dur = [0.004] * n
    dur[0] = -0.004
    s, e, wk, st = W.serve_simulate([0.0] * n, need, dur, 2, 100)
    assert st[0] == INTERNAL
    assert all(st[j] == 0 for j in range(1, n))
    assert len(set(wk)) == 1
    assert max(held_at_starts(s, need, wk, 2)) <= 100


def test_failures_in_groups():
    # a group's proof fails: every job of the group reports it, the next
    # group of the same shape proves
    n = 8
    shape = [1] * n
    dur = [0.004] * n
    dur[0] = -0.004  # the head of the first group
    s, e, wk, st = W.serve_simulate([0.0] * n, [5] * n, dur, 1, 10 ** 9, shape=shape,
                                    max_group=4)
    assert list(st[:4]) == [INTERNAL] * 4
    assert (st[4:] == 0).all()

