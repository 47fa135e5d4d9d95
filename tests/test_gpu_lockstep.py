"""Lock-step batched proving (whir_prove_batch) on the GPU.

A batch runs many polynomials of one shape through every device pass in one
launch; each instance's proof must be byte-identical to the same polynomial
proved alone by the plain prover, and (for the small shapes) to the oracle's
proof, and the verifier must accept it.  The shapes cover the DFT's one-pass,
coset and two-pass forms, foldings 1-6, the three soundness modes, rate 1
(no STIR queries), zero claims, commitments alone, device-resident input and
batch sizes that are not powers of two.
"""
import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


def polys_for(oracle, params, n, seed):
    k = params[0]
    return [oracle.rand_fe(seed * 1000 + i, 1 << k) for i in range(n)]


def check_batch(ctx, oracle, params, n, claims, seed, commit_only=False, with_oracle=True,
                on_device=False):
    polys = polys_for(oracle, params, n, seed)
    k = params[0]
    if on_device:
        dev = [ctx.to_device(p) for p in polys]
        got = W.prove_batch(ctx, params, dev, claims=claims, commit_only=commit_only)
    else:
        got = W.prove_batch(ctx, params, polys, claims=claims, commit_only=commit_only)
    assert len(got) == n
    for i, (proof, cp) in enumerate(got):
        if commit_only:
            w = W.Whir(ctx, *params)
            t = W.PoseidonWriter()
            w.commit(t, [polys[i]], [k])
            want = (t.finalize(), t.draw_base())
            assert (proof, cp) == want, (params, i)
            continue
        want = W.prove_harness(ctx, params, [polys[i]], [k], [[0]] * claims)
        assert proof == want[0], (params, n, i)
        assert cp == want[1]
        assert W.verify(params, [k], [[0]] * claims, proof) == (0, cp)
        if with_oracle:
            assert oracle.prove(params, [polys[i]], [k], [[0]] * claims) == (proof, cp)


@pytest.mark.parametrize("params,n,claims", [
    ((12, 4, 1, 1, 1, 100), 3, 2),
    ((14, 4, 1, 1, 1, 100), 5, 1),
    ((16, 4, 2, 1, 1, 100), 8, 2),   # the small proofs of the mixed batch
    ((10, 2, 1, 1, 1, 100), 4, 1),
    ((11, 3, 2, 2, 0, 80), 6, 3),    # UniqueDecoding: no OOD samples
    ((12, 1, 1, 1, 2, 90), 2, 1),    # CapacityBound, folding 1
    ((12, 4, 1, 1, 1, 100), 1, 1),   # a batch of one
])
def test_lockstep_matches_plain_and_oracle(ctx, oracle, params, n, claims):
    check_batch(ctx, oracle, params, n, claims, seed=hash(params) % 97 + n)


def test_lockstep_zero_claims_and_rate_one(ctx, oracle):
    check_batch(ctx, oracle, (12, 4, 1, 1, 1, 100), 3, 0, seed=11)
    check_batch(ctx, oracle, (12, 4, 0, 1, 1, 100), 3, 1, seed=12)  # 0 STIR queries


def test_lockstep_foldings_5_and_6(ctx, oracle):
    check_batch(ctx, oracle, (15, 5, 1, 1, 1, 100), 3, 1, seed=13, with_oracle=False)
    check_batch(ctx, oracle, (18, 6, 1, 1, 1, 100), 2, 1, seed=14, with_oracle=False)


def test_lockstep_two_pass_dft_and_device_input(ctx, oracle):
    # 2^19-row base codewords take the two-pass DFT at a 3-instance width
    check_batch(ctx, oracle, (20, 4, 1, 1, 1, 100), 3, 2, seed=15, with_oracle=False,
                on_device=True)


def test_lockstep_commitments_alone(ctx, oracle):
    check_batch(ctx, oracle, (18, 4, 1, 1, 1, 100), 7, 0, seed=16, commit_only=True)


def test_lockstep_wide_batch(ctx, oracle):
    # 64 instances of a small shape: batched widths of 1024 and 4096 words
    check_batch(ctx, oracle, (12, 4, 2, 1, 1, 100), 64, 2, seed=17, with_oracle=False)


def test_lockstep_reuse_across_shapes(ctx, oracle):
    # one context's batch prover across growing and shrinking shapes
    for params, n in (((10, 4, 1, 1, 1, 100), 9), ((16, 4, 1, 1, 1, 100), 2),
                      ((12, 3, 2, 1, 1, 100), 5)):
        check_batch(ctx, oracle, params, n, 1, seed=18 + n, with_oracle=False)


def test_lockstep_refuses_oversized_batches(ctx, oracle):
    params = (22, 4, 2, 1, 1, 100)
    mx = W.batch_max(params)
    assert 1 <= mx < 1024
    polys = [np.zeros(1 << 10, np.uint32)] * 2
    with pytest.raises(W.WhirError):
        W.prove_batch(ctx, (10, 4, 1, 1, 1, 100), polys[:1] * (W.batch_max((10, 4, 1, 1, 1, 100)) + 1))
