"""Debug mode of the prover (whir_debug_set) on the GPU.

With the reference's debug-build invariants switched on (after the
expression build and every sumcheck round <poly, weights> equals the claimed
sum, prover.rs:346,558 and expr.rs:68; every opened Merkle path hashes to its
root, poseidon_packed.rs:158-230; every opened row folded at the round point
equals the current polynomial at its domain point, whir.rs:263-264,287-288,
331-352; each virtual claim equals the claim made on the stacked polynomial,
sumcheck/prover.rs:257-266) and NVTX ranges on, proofs must still pass every
check and equal the oracle's byte for byte.
"""
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


@pytest.fixture
def debug_on():
    W.debug_set(W.DEBUG_CHECKS | W.DEBUG_NVTX)
    yield
    W.debug_set(0)


@pytest.mark.parametrize("params,groups", [
    ((12, 4, 1, 1, 1, 100), [[0], [0]]),
    ((14, 3, 2, 2, 1, 100), [[0]]),
    ((11, 2, 1, 1, 0, 90), [[0], [0], [0]]),
    ((16, 5, 1, 1, 2, 100), [[0]]),
    ((12, 4, 0, 1, 1, 100), [[0]]),       # rate 1: no STIR queries
    ((13, 4, 2, 3, 1, 100), [[0], [0]]),  # initial_reduction 3
    ((9, 4, 1, 1, 1, 100), [[0]]),        # no folding rounds: the final openings on the base tree
])
def test_debug_checks_pass_and_proofs_unchanged(ctx, oracle, debug_on, params, groups):
    k = params[0]
    poly = oracle.rand_fe(77 + k, 1 << k)
    proof, cp = W.prove_harness(ctx, params, [poly], [k], groups)
    assert (proof, cp) == oracle.prove(params, [poly], [k], groups)


def test_debug_checks_on_a_stacked_layout(ctx, oracle, debug_on):
    # five polynomials of three sizes stacked with selector bits: the virtual
    # claims also equal the claims made on the stacked polynomial directly
    params, ks, groups = (10, 3, 1, 1, 1, 32), [8, 6, 6, 8, 5], [[0, 3], [1, 2], [4], [3]]
    polys = [oracle.rand_fe(40 + i, 1 << k) for i, k in enumerate(ks)]
    got = W.prove_harness(ctx, params, polys, ks, groups)
    assert got == oracle.prove(params, polys, ks, groups)


def test_debug_flags_are_checked():  # no GPU work
    with pytest.raises(W.WhirError):
        W.debug_set(8)
    W.debug_set(0)
