"""whir_verify's two pass structures give the same answer.

By default whir_verify reads the whole proof first and hashes the Merkle
openings afterwards, as whir_verify_batch does (the openings are hints: no
challenge depends on them); with DEBUG_VERIFY_INLINE it hashes each opening
where it reads it, in Whir::verify's order (crates/whir/src/whir.rs:361-522).
A proof's result must be the same either way, also when several things are
wrong with it: the first failure in Whir::verify's order wins (an opening
that does not hash to its root, then a later truncation or a wrong final
polynomial, is a Merkle failure).  Proofs come from the oracle.
"""
import numpy as np
import pytest

import whir_gb300 as W


def both_orders(params, ks, groups, proof):
    try:
        W.debug_set(W.DEBUG_VERIFY_INLINE)
        inline = W.verify(params, ks, groups, proof)
    finally:
        W.debug_set(0)
    return inline, W.verify(params, ks, groups, proof)


@pytest.fixture(scope="module", params=[
    ((12, 4, 1, 1, 1, 100), [12], [[0]] * 2),      # two rounds of openings plus the final ones
    ((14, 2, 1, 1, 1, 64), [14], [[0]]),           # folding 2: base rows of 4 words, ext rows of 16
    ((10, 3, 1, 1, 1, 32), [8, 6, 6, 8, 5], [[0, 3], [1, 2], [4], [3]]),  # stacked layout
])
def case(request, oracle):
    params, ks, groups = request.param
    polys = [oracle.rand_fe(7 + i, 1 << k) for i, k in enumerate(ks)]
    proof, cp = oracle.prove(params, polys, ks, groups)
    return params, ks, groups, proof, cp


def test_valid_proof(case):
    params, ks, groups, proof, cp = case
    a, d = both_orders(params, ks, groups, proof)
    assert a == d == (0, cp)


def test_single_corruptions(case):
    params, ks, groups, proof, _ = case
    rng = np.random.default_rng(len(proof))
    codes = set()
    for _ in range(120):
        bad = bytearray(proof)
        bad[int(rng.integers(0, len(bad)))] ^= 1 << int(rng.integers(0, 7))
        a, d = both_orders(params, ks, groups, bytes(bad))
        assert a == d
        codes.add(a[0])
    assert 2 in codes  # some flips hit an opening


def test_merkle_failure_comes_before_later_failures(case):
    params, ks, groups, proof, _ = case
    rng = np.random.default_rng(3 * len(proof))
    seen = {}
    for _ in range(150):
        bad = bytearray(proof)
        p = int(rng.integers(0, len(bad)))
        bad[p] ^= 1 << int(rng.integers(0, 7))
        kind = int(rng.integers(0, 3))
        if kind == 0:    # and the proof ends early somewhere after it
            bad = bad[:int(rng.integers(p + 1, len(bad) + 1))]
        elif kind == 1:  # and the last words (the final openings) are garbled
            for q in range(max(p + 1, len(bad) - 64), len(bad)):
                bad[q] = int(rng.integers(0, 128))
        else:            # and a second flip anywhere
            bad[int(rng.integers(0, len(bad)))] ^= 1
        a, d = both_orders(params, ks, groups, bytes(bad))
        assert a == d, (p, kind)
        seen[a[0]] = seen.get(a[0], 0) + 1
    assert seen.get(2, 0) > 0 and seen.get(1, 0) > 0


def test_random_bytes_and_prefixes(case):
    params, ks, groups, proof, _ = case
    rng = np.random.default_rng(11)
    for trial in range(60):
        if trial % 2:
            b = proof[:int(rng.integers(0, len(proof)))]
        else:
            b = rng.integers(0, 256, int(rng.integers(0, len(proof) + 50)),
                             dtype=np.uint8).tobytes()
        a, d = both_orders(params, ks, groups, b)
        assert a == d
        assert a[0] != 0


def test_unknown_debug_flags_are_refused():
    with pytest.raises(W.WhirError):
        W.debug_set(8)
