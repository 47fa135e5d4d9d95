"""whir_verify_batch on the GPU equals whir_verify on each proof.

The batch reads every proof on host threads with the Merkle openings
deferred and hashes all openings of all proofs in one launch; each proof's
(result, checkpoint) must be what whir_verify gives for it alone: accepted
proofs with their checkpoints, and every rejection code (Merkle, transcript,
final openings, sumcheck) for corrupted, truncated and random proofs mixed
into the same batch.  Shapes cover foldings 2 and 4 (rows of 4, 16 and 64
words), a stacked layout, rate 1 (no openings at all) and a batch of 256.
"""
import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


def alone(params, ks, groups, proofs):
    return [W.verify(params, ks, groups, p) for p in proofs]


def corrupted(proof, rng, n):
    out = []
    for t in range(n):
        b = bytearray(proof)
        kind = t % 4
        if kind == 0:
            b[int(rng.integers(0, len(b)))] ^= 1 << int(rng.integers(0, 7))
        elif kind == 1:
            p = int(rng.integers(0, len(b)))
            b[p] ^= 1
            b = b[:int(rng.integers(p + 1, len(b) + 1))]
        elif kind == 2:
            b = b[:int(rng.integers(0, len(b)))]
        else:
            b = bytearray(rng.integers(0, 256, len(b), dtype=np.uint8).tobytes())
        out.append(bytes(b))
    return out


@pytest.mark.parametrize("params,n", [
    ((12, 4, 1, 1, 1, 100), 6),
    ((14, 2, 1, 1, 1, 64), 4),
    ((16, 4, 2, 1, 1, 100), 5),
])
def test_batch_equals_alone(ctx, oracle, params, n):
    k = params[0]
    polys = [oracle.rand_fe(100 + i, 1 << k) for i in range(n)]
    good = W.prove_batch(ctx, params, polys, claims=2)
    proofs = [p for p, _ in good]
    rng = np.random.default_rng(k)
    mixed = []
    for p in proofs:
        mixed.append(p)
        mixed.extend(corrupted(p, rng, 6))
    want = alone(params, [k], [[0]] * 2, mixed)
    got = W.verify_batch(ctx, params, [k], [[0]] * 2, mixed)
    assert got == want
    assert [g for g in got[::7]] == [(0, cp) for _, cp in good]
    assert {r for r, _ in want} >= {0, 1, 2}


def test_stacked_layout(ctx, oracle):
    params, ks, groups = (10, 3, 1, 1, 1, 32), [8, 6, 6, 8, 5], [[0, 3], [1, 2], [4], [3]]
    polys = [oracle.rand_fe(3 + i, 1 << k) for i, k in enumerate(ks)]
    proof, cp = oracle.prove(params, polys, ks, groups)
    rng = np.random.default_rng(2)
    mixed = [proof] + corrupted(proof, rng, 20)
    assert W.verify_batch(ctx, params, ks, groups, mixed) == alone(params, ks, groups, mixed)
    assert W.verify_batch(ctx, params, ks, groups, [proof]) == [(0, cp)]


def test_no_openings_and_empty_batch(ctx, oracle):
    params = (12, 4, 0, 1, 1, 100)  # rate 1: no STIR queries, nothing to hash
    poly = oracle.rand_fe(9, 1 << 12)
    proof, cp = oracle.prove(params, [poly], [12], [[0]])
    assert W.verify_batch(ctx, params, [12], [[0]], [proof, proof[:-4]]) == \
        alone(params, [12], [[0]], [proof, proof[:-4]])
    assert W.verify_batch(ctx, params, [12], [[0]], []) == []


def test_wide_batch(ctx, oracle):
    params = (16, 4, 2, 1, 1, 100)
    polys = [oracle.rand_fe(500 + i, 1 << 16) for i in range(256)]
    good = W.prove_batch(ctx, params, polys, claims=2)
    proofs = [p for p, _ in good]
    got = W.verify_batch(ctx, params, [16], [[0]] * 2, proofs)
    assert got == [(0, cp) for _, cp in good]
    # one bad opening in one proof of the 256 rejects that proof only
    bad = bytearray(proofs[77])
    bad[len(bad) // 2] ^= 2
    proofs[77] = bytes(bad)
    got = W.verify_batch(ctx, params, [16], [[0]] * 2, proofs)
    want77 = W.verify(params, [16], [[0]] * 2, proofs[77])
    assert got[77] == want77 and want77[0] != 0
    assert all(got[i] == (0, good[i][1]) for i in range(256) if i != 77)


def test_argument_errors(ctx):
    with pytest.raises(W.WhirError):
        W.verify_batch(ctx, (10, 4, 1, 1, 1, 100), [9], [[0]], [b"\0" * 64])  # layout != 2^k
    with pytest.raises(W.WhirError):
        W.verify_batch(ctx, (10, 4, 1, 1, 1, 100), [10], [[1]], [b"\0" * 64])  # unknown poly id


@pytest.mark.parametrize("seed", range(24))
def test_random_statements(ctx, oracle, seed):
    # shapes drawn as in the random proof sweep: folding 1-6, rates 0-3, the
    # three soundness modes, stacked polynomials and claim groups
    from test_gpu_random_shapes import draw_statement
    rng = np.random.default_rng(30000 + seed)
    params, ks, groups = draw_statement(rng)
    polys = [oracle.rand_fe(31000 + 16 * seed + i, 1 << kp) for i, kp in enumerate(ks)]
    try:
        proof, cp = oracle.prove(params, polys, ks, groups)
    except RuntimeError:
        return  # a statement the reference cannot run (refused by both sides)
    mixed = [proof] + corrupted(proof, np.random.default_rng(32000 + seed), 6)
    got = W.verify_batch(ctx, params, ks, groups, mixed)
    assert got == alone(params, ks, groups, mixed), (params, ks, groups)
    assert got[0] == (0, cp)
