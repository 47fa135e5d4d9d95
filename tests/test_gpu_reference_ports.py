"""Ports of two reference tests to the GPU path.

test_simple_whir_no_transpose (crates/whir/src/test.rs:95-172): the
Reed-Solomon encoding commutes with folding.  With a polynomial's words as
a row-major matrix of 2^f columns (column j holds P[2^f i + j], the layout
commit_base encodes, crates/whir/src/whir.rs:20-36), folding every codeword
row with eq(alpha) gives the encoding of the folded polynomial:

    compress_lo(dft(P), alpha) == dft(compress_lo(P, alpha)),

both sides computed on the GPU.  The reference's own sweep (k = 5, every
folding below k, rates 0..4) is also compared with the oracle; at the bench
workload's size (k = 24, folding 4, rate 1/4) and the whir_bench shape
(k = 25, folding 5, rate 1/2) the identity itself is the check.  The test's
first block is ported too: the evaluation at z equals the eq(z)-weighted
sum over the hypercube.

test_zkvm (crates/whir/src/sumcheck/test.rs:93-221): 20 polynomials of 20
variables and 125 of 8, claims at eight shared points over chosen subsets,
stacked into a 25-variable layout.  Here the whole WHIR proof of that
statement on the GPU equals the oracle's byte for byte, and verifies.
Exact field arithmetic throughout: zero tolerance.
"""
import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


def encode_fold(ctx, dev_poly, k, f, rate, alpha):
    """(rows of dft(P) folded with eq(alpha), dft of P folded with eq(alpha))"""
    kd = k + rate - f
    cw = W.dft_batch(ctx, dev_poly, 1 << (k - f), 1 << f, kd)
    lhs = W.compress_lo(ctx, cw, kd + f, alpha, f).download(4 << kd)
    cw.close()
    folded = W.compress_lo(ctx, dev_poly, k, alpha, f)
    rhs = W.dft_batch(ctx, folded, 1 << (k - f), 4, kd).download(4 << kd)
    return lhs, rhs


@pytest.mark.parametrize("f", range(5))
@pytest.mark.parametrize("rate", range(5))
def test_encode_commutes_with_folding_small(ctx, oracle, f, rate):
    k = 5
    poly = W.random_field(1, 1 << k)
    alpha = oracle.rand_fe(50 + 5 * f + rate, 4 * f)
    lhs, rhs = encode_fold(ctx, ctx.to_device(poly), k, f, rate, alpha)
    assert np.array_equal(lhs, rhs), (f, rate)
    kd = k + rate - f
    cw = oracle.dft_batch(poly, 1 << (k - f), 1 << f, kd)
    assert np.array_equal(lhs, oracle.compress_lo(cw, kd + f, alpha, f))
    folded = oracle.compress_lo(poly, k, alpha, f)
    assert np.array_equal(rhs, oracle.dft_batch(folded, 1 << (k - f), 4, kd))


@pytest.mark.parametrize("k,f,rate", [(24, 4, 2), (25, 5, 1), (20, 4, 1), (22, 6, 3)])
def test_encode_commutes_with_folding_full_size(ctx, oracle, k, f, rate):
    dev = ctx.to_device(W.random_field(k, 1 << k))
    alpha = oracle.rand_fe(60 + k, 4 * f)
    lhs, rhs = encode_fold(ctx, dev, k, f, rate, alpha)
    assert np.array_equal(lhs, rhs), (k, f, rate)
    dev.close()


def test_evaluation_is_the_eq_weighted_sum(ctx, oracle):
    k = 5
    f0 = W.random_field(1, 1 << k)
    z = oracle.rand_fe(70, 4 * k)
    eq = W.eq_table(ctx, z, k, oracle.ext_one()).download(4 << k).reshape(-1, 4)
    L, P = oracle.lib(), W.P
    acc = [0, 0, 0, 0]
    for i in range(1 << k):
        for c in range(4):
            acc[c] = (acc[c] + L.wo_fe_mul(int(f0[i]), int(eq[i, c]))) % P
    ext = np.zeros(4 << k, np.uint32)
    ext[0::4] = f0  # the base polynomial as extension elements
    got = W.eval_ext(ctx, ctx.to_device(ext), k, z)
    assert [int(x) for x in got] == acc


def test_zkvm_layout(ctx, oracle):
    ks = [20] * 20 + [8] * 29 + [8] * 96
    a, b, c = list(range(0, 20)), list(range(20, 49)), list(range(49, 145))
    groups = [
        [a[i] for i in [0] + list(range(2, 20))], [a[0], a[1]], a[:],              # table A
        [b[i] for i in range(6, 24)], [b[i] for i in list(range(0, 8)) + list(range(24, 29))],
        b[:],                                                                       # table B
        [c[i] for i in list(range(1, 20)) + list(range(88, 96))], c[:],            # table C
    ]
    polys = [oracle.rand_fe(40000 + i, 1 << kp) for i, kp in enumerate(ks)]
    params = (25, 5, 1, 1, 1, 100)
    got = W.prove_harness(ctx, params, polys, ks, groups)
    assert got == oracle.prove(params, polys, ks, groups)
    assert W.verify(params, ks, groups, got[0]) == (0, got[1])
