"""Seeded random statements on the GPU, each proof equal to the oracle's.

The hand-picked parity cases cover each parameter on its own; this sweep
draws whole statements at random (folding 1-6, rates 0-3, the three
soundness modes, security 32-100, any initial reduction the round shapes
allow, one to four polynomials of mixed sizes stacked with selector bits,
claim groups over equal-size polynomials) and checks every GPU proof
byte for byte against the oracle's, and against the verifier.  Lock-step
batches of random shapes and sizes are checked against the plain prover.
Statements the reference cannot run are refused before any work (the
library's WhirError) and skipped.
"""
import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


def draw_statement(rng):
    f = int(rng.integers(1, 7))
    k = int(rng.integers(f + 1, 15))
    rate = int(rng.integers(0, 4))
    soundness = int(rng.integers(0, 3))
    sec = int(rng.choice([32, 64, 100]))
    ir = int(rng.integers(1, rate + f + 1))
    params = (k, f, rate, ir, soundness, sec)
    n_polys = int(rng.integers(1, 5))
    if n_polys == 1:
        ks = [k]
    else:
        # sizes from k - 3 to k - 1, packed into 2^k words (largest first)
        ks, room = [], 1 << k
        for _ in range(n_polys):
            kp = int(rng.integers(max(1, k - 3), k))
            if (1 << kp) <= room:
                ks.append(kp)
                room -= 1 << kp
        ks = ks or [k]
    groups = []
    for _ in range(int(rng.integers(0, 4))):
        kp = ks[int(rng.integers(0, len(ks)))]
        same = [i for i, x in enumerate(ks) if x == kp]
        take = rng.choice(same, size=int(rng.integers(1, len(same) + 1)), replace=False)
        groups.append(sorted(int(i) for i in take))
    return params, ks, groups


@pytest.mark.parametrize("seed", range(96))
def test_random_statement(ctx, oracle, seed):
    rng = np.random.default_rng(1000 + seed)
    params, ks, groups = draw_statement(rng)
    polys = [oracle.rand_fe(seed * 16 + i, 1 << kp) for i, kp in enumerate(ks)]
    try:
        got = W.prove_harness(ctx, params, polys, ks, groups)
    except W.WhirError:
        # refused before any work: the oracle refuses the same statement
        with pytest.raises(RuntimeError):
            oracle.prove(params, polys, ks, groups)
        return
    assert got == oracle.prove(params, polys, ks, groups), (params, ks, groups)
    assert W.verify(params, ks, groups, got[0]) == (0, got[1])


@pytest.mark.parametrize("seed", range(16))
def test_random_lockstep_batch(ctx, oracle, seed):
    rng = np.random.default_rng(2000 + seed)
    f = int(rng.integers(1, 6))
    k = int(rng.integers(f + 2, 15))
    rate = int(rng.integers(0, 4))
    params = (k, f, rate, int(rng.integers(1, rate + f + 1)), int(rng.integers(0, 3)),
              int(rng.choice([32, 64, 100])))
    n = int(rng.integers(1, 13))
    claims = int(rng.integers(0, 4))
    polys = [oracle.rand_fe(3000 + 31 * seed + i, 1 << k) for i in range(n)]
    try:
        got = W.prove_batch(ctx, params, polys, claims=claims)
    except W.WhirError:
        with pytest.raises(W.WhirError):
            W.prove_harness(ctx, params, polys[:1], [k], [[0]] * claims)
        return
    for i, (proof, cp) in enumerate(got):
        assert (proof, cp) == W.prove_harness(ctx, params, [polys[i]], [k], [[0]] * claims), \
            (params, n, claims, i)
    assert got[0] == oracle.prove(params, [polys[0]], [k], [[0]] * claims)
