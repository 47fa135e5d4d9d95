"""The library's host verifier (whir_verify, Whir::verify of
crates/whir/src/whir.rs:361-522) on the CPU, against proofs from the oracle
prover: it accepts them with the oracle's checkpoint, over the reference's
test_whir_poseidon parameter sweep (crates/whir/src/test.rs:256-282) and
stacked layouts, and rejects tampered, truncated or mismatched proofs.
"""
import numpy as np
import pytest

import whir_gb300 as W

SWEEP = [(s, k, f, ir, n)
         for s in (1, 2, 0) for k in (4, 6, 9, 12) for f in (1, 2, 3)
         for ir in range(1, f + 1) for n in (1, 3)
         if (k + f + ir + n + s) % 4 == 0 or k == 12 and ir == 1 and n == 1]


@pytest.mark.parametrize("s,k,f,ir,n", SWEEP)
def test_accepts_oracle_proofs(oracle, s, k, f, ir, n):
    poly = oracle.rand_fe(7 + k, 1 << k)
    params = (k, f, 1, ir, s, 32)
    proof, cp = oracle.prove(params, [poly], [k], [[0]] * n)
    res, vcp = W.verify(params, [k], [[0]] * n, proof)
    assert res == 0 and vcp == cp


@pytest.mark.parametrize("k,rate,n", [(10, 2, 2), (14, 1, 1), (12, 2, 4)])
def test_accepts_folding4_security100(oracle, k, rate, n):
    poly = oracle.rand_fe(3, 1 << k)
    params = (k, 4, rate, 1, 1, 100)
    proof, cp = oracle.prove(params, [poly], [k], [[0]] * n)
    assert W.verify(params, [k], [[0]] * n, proof) == (0, cp)


@pytest.mark.parametrize("params,n", [((14, 5, 1, 1, 1, 100), 2), ((13, 5, 1, 3, 0, 32), 1),
                                      ((12, 5, 1, 5, 2, 32), 4), ((15, 6, 1, 1, 1, 100), 3),
                                      # whir_bench's shape (crates/whir/src/test.rs:284-290) at k = 16
                                      ((16, 5, 1, 3, 1, 123), 1)])
def test_accepts_folding5_6(oracle, params, n):
    k = params[0]
    poly = oracle.rand_fe(4, 1 << k)
    proof, cp = oracle.prove(params, [poly], [k], [[0]] * n)
    assert W.verify(params, [k], [[0]] * n, proof) == (0, cp)


@pytest.mark.parametrize("params", [(6, 1, 0, 1, 1, 32), (8, 2, 0, 1, 0, 32), (9, 3, 0, 2, 2, 64),
                                    (12, 4, 0, 1, 1, 100)])
def test_rate_one_has_no_queries(oracle, params):
    # log_inv_rate 0: params.rs:118-122 casts a negative or -inf query count
    # with Rust's saturating `as usize`, so every round has 0 STIR queries
    k = params[0]
    poly = oracle.rand_fe(6, 1 << k)
    proof, cp = oracle.prove(params, [poly], [k], [[0]] * 2)
    assert W.verify(params, [k], [[0]] * 2, proof) == (0, cp)


def test_query_count_out_of_range_is_refused(oracle):
    params = (10, 2, 1, 1, 0, 100000)  # unique decoding, 100000-bit: ~10^5 queries
    with pytest.raises(W.WhirError):
        W.workspace_bytes(params)
    with pytest.raises(RuntimeError):
        oracle.prove(params, [oracle.rand_fe(1, 1 << 10)], [10], [[0]])


@pytest.mark.parametrize("params", [(10, 2, 1, 5, 1, 32), (8, 1, 1, 3, 0, 32), (7, 8, 1, 1, 1, 32),
                                    (22, 2, 6, 1, 1, 32), (10, 2, 1, 1, 1, -5)])
def test_parameters_the_reference_cannot_run_are_refused(oracle, params):
    # round shapes that go negative in the reference's usize arithmetic
    # (whir.rs:150-166, params.rs:186-202) panic there, and a codeword above
    # 2^24 rows has no two-adic subgroup: all are refused here
    k = params[0]
    with pytest.raises(W.WhirError):
        W.workspace_bytes(params)
    with pytest.raises(W.WhirError):
        W.verify(params, [k], [[0]], b"\0" * 64)
    if k <= 12:
        with pytest.raises(RuntimeError):
            oracle.prove(params, [oracle.rand_fe(1, 1 << k)], [k], [[0]])


def test_reduction_up_to_rate_plus_folding_is_accepted(oracle):
    # initial_reduction 4 > folding 3 at rate 1/2 keeps every shape >= 0
    params = (12, 3, 1, 4, 1, 32)
    poly = oracle.rand_fe(12, 1 << 12)
    proof, cp = oracle.prove(params, [poly], [12], [[0]] * 2)
    assert W.verify(params, [12], [[0]] * 2, proof) == (0, cp)


def test_accepts_stacked_layout(oracle):
    ks = [8, 6, 6, 8, 5]
    polys = [oracle.rand_fe(20 + i, 1 << k) for i, k in enumerate(ks)]
    k = int(np.ceil(np.log2(sum(1 << x for x in ks))))
    groups = [[0, 3], [1, 2], [4], [3]]
    params = (k, 3, 1, 1, 1, 32)
    proof, cp = oracle.prove(params, polys, ks, groups)
    assert W.verify(params, ks, groups, proof) == (0, cp)


@pytest.fixture(scope="module")
def one_proof(oracle):
    k, n = 12, 2
    params = (k, 4, 1, 1, 1, 100)
    poly = oracle.rand_fe(11, 1 << k)
    proof, cp = oracle.prove(params, [poly], [k], [[0]] * n)
    return params, k, n, proof, cp


def test_rejects_flipped_bytes(one_proof):
    params, k, n, proof, cp = one_proof
    rng = np.random.default_rng(5)
    # the root, a claim evaluation, the SVO rounds, then spread over the rest
    spots = [0, 31, 40, 100, 200] + sorted(int(x) for x in rng.integers(0, len(proof), 40))
    for pos in spots:
        bad = bytearray(proof)
        bad[pos] ^= 1 << int(rng.integers(0, 7))   # stays below 2^31 in the top byte
        res, _ = W.verify(params, [k], [[0]] * n, bytes(bad))
        assert res != 0, pos


def test_rejects_truncated_and_noncanonical(one_proof):
    params, k, n, proof, cp = one_proof
    assert W.verify(params, [k], [[0]] * n, proof[:-4])[0] == 1
    assert W.verify(params, [k], [[0]] * n, b"")[0] == 1
    bad = bytearray(proof)
    bad[0:4] = (0x7f000001).to_bytes(4, "little")    # p itself: not canonical
    assert W.verify(params, [k], [[0]] * n, bytes(bad))[0] == 1


def test_rejects_other_statement(one_proof):
    params, k, n, proof, cp = one_proof
    # a different number of claims changes every challenge after the root
    assert W.verify(params, [k], [[0]] * (n + 1), proof)[0] != 0
    # other security parameters change the query counts
    assert W.verify((k, 4, 1, 1, 1, 90), [k], [[0]] * n, proof)[0] != 0


def test_argument_errors():
    with pytest.raises(W.WhirError):
        W.verify((10, 4, 1, 1, 1, 100), [9], [[0]], b"\\0" * 64)   # layout size != 2^k
    with pytest.raises(W.WhirError):
        W.verify((10, 4, 1, 1, 1, 100), [10], [[1]], b"\\0" * 64)  # unknown poly id


@pytest.mark.parametrize("params,ks,groups", [
    ((10, 2, 1, 1, 1, 32), [10], [[0]] * 2),
    ((12, 4, 2, 1, 1, 100), [12], [[0]]),
    ((10, 3, 1, 1, 1, 32), [8, 6, 6, 8, 5], [[0, 3], [1, 2], [4], [3]]),
    ((6, 1, 0, 1, 1, 32), [6], [[0]])])
def test_rejects_random_and_corrupted_bytes(oracle, params, ks, groups):
    # random byte strings, proofs with random bytes overwritten, and random
    # prefixes: every one is rejected (never accepted, never a crash)
    polys = [oracle.rand_fe(3 + i, 1 << k) for i, k in enumerate(ks)]
    proof, _ = oracle.prove(params, polys, ks, groups)
    rng = np.random.default_rng(sum(ks))
    for trial in range(150):
        kind = trial % 3
        if kind == 0:
            b = rng.integers(0, 256, int(rng.integers(0, len(proof) + 100)), dtype=np.uint8).tobytes()
        elif kind == 1:
            m = bytearray(proof)
            for _ in range(int(rng.integers(1, 20))):
                m[int(rng.integers(0, len(m)))] = int(rng.integers(0, 256))
            if bytes(m) == proof:
                continue
            b = bytes(m)
        else:
            b = proof[:int(rng.integers(0, len(proof)))]
        assert W.verify(params, ks, groups, b)[0] != 0


@pytest.mark.parametrize("params,ks,groups", [
    ((5, 4, 0, 3, 1, 64), [2, 4], [[0], [1], [1]]),
    ((6, 5, 2, 1, 0, 32), [3, 5], [[1]]),
    ((6, 4, 2, 2, 1, 64), [3, 5, 4], []),        # no claim on the small one
])
def test_polynomials_smaller_than_the_folding_are_refused(oracle, params, ks, groups):
    # the reference's expression build fixes the low `folding` variables of
    # every stacked polynomial (compress_stacked asserts it,
    # crates/whir/src/sumcheck/prover.rs:216), so it cannot run such a
    # statement; the oracle and the library refuse it before any work
    polys = [oracle.rand_fe(1 + i, 1 << k) for i, k in enumerate(ks)]
    with pytest.raises(RuntimeError):
        oracle.prove(params, polys, ks, groups)
    assert oracle.verify(params, ks, groups, b"\0" * 64)[0] == -1
    with pytest.raises(W.WhirError):
        W.verify(params, ks, groups, b"\0" * 64)


def test_claim_group_of_mixed_sizes_is_refused(oracle):
    # one point per group, expanded to its first polynomial's size: every
    # member must have that size (library and oracle refuse alike)
    ks = [10, 9, 9]
    polys = [oracle.rand_fe(1 + i, 1 << k) for i, k in enumerate(ks)]
    params = (11, 3, 1, 1, 1, 32)
    with pytest.raises(RuntimeError):
        oracle.prove(params, polys, ks, [[0, 1]])
    with pytest.raises(W.WhirError):
        W.verify(params, ks, [[0, 1]], b"\0" * 64)
    proof, cp = oracle.prove(params, polys, ks, [[1, 2], [0]])
    assert W.verify(params, ks, [[1, 2], [0]], proof) == (0, cp)


def _random_statement(rng):
    # as tests/test_gpu_random_shapes.py draws them (folding 1-6, rates 0-3,
    # the three soundness modes, stacked layouts of mixed sizes)
    f = int(rng.integers(1, 7))
    k = int(rng.integers(f + 1, 13))
    rate = int(rng.integers(0, 4))
    params = (k, f, rate, int(rng.integers(1, rate + f + 1)), int(rng.integers(0, 3)),
              int(rng.choice([32, 64, 100])))
    ks, room = [], 1 << k
    for _ in range(int(rng.integers(1, 5))):
        kp = int(rng.integers(max(f, k - 3), k + 1))
        if (1 << kp) <= room:
            ks.append(kp)
            room -= 1 << kp
    groups = []
    for _ in range(int(rng.integers(0, 4))):
        kp = ks[int(rng.integers(0, len(ks)))]
        same = [i for i, x in enumerate(ks) if x == kp]
        groups.append(sorted(int(i) for i in rng.choice(same, size=int(rng.integers(1, len(same) + 1)),
                                                         replace=False)))
    return params, ks, groups


@pytest.mark.parametrize("seed", range(48))
def test_random_statements_both_verifiers_agree(oracle, seed):
    # the library's verifier accepts the oracle's proof of a random statement
    # with the oracle's checkpoint, and accepts or rejects corrupted copies
    # exactly when the oracle's own verifier does
    rng = np.random.default_rng(5000 + seed)
    params, ks, groups = _random_statement(rng)
    polys = [oracle.rand_fe(seed * 8 + i, 1 << kp) for i, kp in enumerate(ks)]
    try:
        proof, cp = oracle.prove(params, polys, ks, groups)
    except RuntimeError:
        with pytest.raises(W.WhirError):
            W.verify(params, ks, groups, b"\0" * 64)
        return
    assert W.verify(params, ks, groups, proof) == (0, cp)
    assert oracle.verify(params, ks, groups, proof) == (0, cp)
    for _ in range(12):
        bad = bytearray(proof)
        bad[int(rng.integers(0, len(bad)))] ^= 1 << int(rng.integers(0, 7))
        mine = W.verify(params, ks, groups, bytes(bad))[0]
        theirs = oracle.verify(params, ks, groups, bytes(bad))[0]
        assert (mine == 0) == (theirs == 0), (params, ks, groups)
