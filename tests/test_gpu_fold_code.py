"""fold_with_code's code pass on the GPU against the direct computation.

A port of the reference's test_fold_with_code
(crates/whir/src/sumcheck/prover.rs:598-768): a k = 25 polynomial, folding 5,
rate 1/2, its base codeword, 300 random indexes and alpha-power scales.  For
every round the device's row evaluations and per-query recursion
(whir_fold_code_rounds: row_evals_kernel, code_round_kernel) must give the
(c0, c2) that the sumcheck coefficients of the folded polynomial against the
combined power weights give directly (oracle compress_lo, combine_pows,
coeffs, fix_lo).  Exact field arithmetic: zero tolerance.
"""
import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


def ext_mul(oracle, a, b):
    out = np.zeros(4, np.uint32)
    oracle.lib().wo_ext_mul(oracle.ptr(np.ascontiguousarray(a, np.uint32)),
                            oracle.ptr(np.ascontiguousarray(b, np.uint32)), oracle.ptr(out))
    return out


def fe_pow(oracle, g, e):
    L = oracle.lib()
    r, b = int(oracle.to_mont(1)), int(g)
    while e:
        if e & 1:
            r = L.wo_fe_mul(r, b)
        b = L.wo_fe_mul(b, b)
        e >>= 1
    return r


def run_case(ctx, oracle, k, f, rate, n, seed):
    poly = W.random_field(seed, 1 << k)
    k_data = k + rate - f
    dev = ctx.to_device(poly)
    cw = W.dft_batch(ctx, dev, 1 << (k - f), 1 << f, k_data)
    rng = np.random.default_rng(seed)
    # Point::expand(folding, v): v, v^2, v^4, ...
    v = W.random_field(seed + 1, 4)
    rs = [v]
    for _ in range(f - 1):
        rs.append(ext_mul(oracle, rs[-1], rs[-1]))
    rs = np.concatenate(rs)
    idx = [int(x) for x in rng.integers(0, 1 << k_data, n)]
    alpha = W.random_field(seed + 2, 4)
    scales = [oracle.ext_one()]
    for _ in range(n - 1):
        scales.append(ext_mul(oracle, scales[-1], alpha))
    scales = np.concatenate(scales)
    r = W.random_field(seed + 3, 4 * f)
    got = W.fold_code_rounds(ctx, cw, k_data, f, idx, scales, rs, r)
    # the direct side: the folded polynomial and the combined power weights
    kk = k - f
    p = oracle.compress_lo(poly, k, rs, f)
    omega = oracle.lib().wo_two_adic_generator(k_data)
    vars_ = np.array([fe_pow(oracle, omega, i) for i in idx], np.uint32)
    pows = oracle.combine_pows(np.zeros(4 << kk, np.uint32), kk, vars_, n, alpha, 0)
    for j in range(f):
        c0, c2 = oracle.coeffs(p, pows, kk)
        assert np.array_equal(got[8 * j:8 * j + 4], c0), (k, f, j)
        assert np.array_equal(got[8 * j + 4:8 * j + 8], c2), (k, f, j)
        p = oracle.fix_lo(p, kk, r[4 * j:4 * j + 4])
        pows = oracle.fix_lo(pows, kk, r[4 * j:4 * j + 4])
        kk -= 1
    cw.close()
    dev.close()


def test_fold_with_code_reference_shape(ctx, oracle):
    run_case(ctx, oracle, 25, 5, 1, 300, seed=1)


@pytest.mark.parametrize("k,f,rate,n", [(16, 4, 2, 108), (14, 2, 1, 40), (18, 6, 1, 57),
                                        (12, 1, 3, 9)])
def test_fold_with_code_other_shapes(ctx, oracle, k, f, rate, n):
    run_case(ctx, oracle, k, f, rate, n, seed=k * 10 + f)
