"""Seeded random shapes for the piece-level entry points, each result equal
to the oracle's (exact field arithmetic: zero tolerance).

The kernel tests pick their shapes by hand; these draw them: the DFT over
heights 2^0..2^17, row widths 1..128 (odd, even, multiples of 4 and of 8:
the scalar, 4-column and 8-column tile paths) and ragged zero-padded
inputs; the Merkle commitment over heights 2^0..2^13 with any row length
1..80 or a folding's row length, every level and the openings of random
indexes; the claim compressions with 0..8 kept or fixed variables;
out-of-domain evaluations; sumcheck coefficients and folds; and the eq and
pow claim combinations with 1..120 claims.
"""
import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu

WIDTHS = [1, 2, 3, 4, 5, 6, 7, 8, 12, 16, 20, 24, 32, 40, 48, 64, 128]


@pytest.mark.parametrize("seed", range(40))
def test_random_dft(ctx, oracle, seed):
    rng = np.random.default_rng(7000 + seed)
    width = int(rng.choice(WIDTHS))
    log_h = int(rng.integers(0, 18))
    while (width << log_h) > (1 << 21):
        log_h -= 1
    h = 1 << log_h
    h_in = h if rng.random() < 0.3 else int(rng.integers(1, h + 1))
    x = oracle.rand_fe(8000 + seed, h_in * width)
    want = oracle.dft_batch(x, h_in, width, log_h)
    got = W.dft_batch(ctx, ctx.to_device(x), h_in, width, log_h).download(width << log_h)
    assert np.array_equal(got, want), (log_h, width, h_in)


@pytest.mark.parametrize("seed", range(30))
def test_random_merkle(ctx, oracle, seed):
    rng = np.random.default_rng(9000 + seed)
    log_h = int(rng.integers(0, 14))
    row_len = int(rng.choice([16, 32, 64, 128, 256])) if rng.random() < 0.4 \
        else int(rng.integers(1, 81))
    while (row_len << log_h) > (1 << 20):
        log_h -= 1
    rows = oracle.rand_fe(10000 + seed, row_len << log_h)
    want = oracle.merkle_tree(rows, log_h, row_len)
    t = W.MerkleTree(ctx, ctx.to_device(rows), log_h, row_len)
    try:
        assert np.array_equal(t.levels(), want), (log_h, row_len)
        assert np.array_equal(t.root, want[-8:])
        n = 1 << log_h
        idx = sorted(set(int(i) for i in rng.integers(0, n, min(n, 9))))
        op = t.open(idx)
        for q, i in enumerate(idx):
            assert np.array_equal(op[q, :row_len], rows[i * row_len:(i + 1) * row_len])
            a = i
            for lvl in range(log_h):
                mid = 1 << (log_h - lvl - 1)
                off = ((2 << log_h) - (2 << (log_h - lvl))) * 8
                sib = want[off + (a ^ mid) * 8: off + (a ^ mid) * 8 + 8]
                assert np.array_equal(op[q, row_len + 8 * lvl: row_len + 8 * lvl + 8], sib)
                a &= mid - 1
    finally:
        t.close()


@pytest.mark.parametrize("seed", range(24))
def test_random_claim_compressions(ctx, oracle, seed):
    rng = np.random.default_rng(11000 + seed)
    k = int(rng.integers(1, 17))
    poly = oracle.rand_fe(12000 + seed, 1 << k)
    dev = ctx.to_device(poly)
    # compress_hi keeps ks <= 8 variables (fixing the high kz = k - ks)
    ks = int(rng.integers(0, min(k, 8) + 1))
    pt = oracle.rand_fe(13000 + seed, 4 * (k - ks))
    got = W.compress_hi(ctx, dev, k, pt, k - ks)
    assert np.array_equal(got, oracle.compress_hi(poly, k, pt, k - ks)), (k, ks)
    # compress_lo fixes the low kz <= 8 variables
    kz = int(rng.integers(0, min(k, 8) + 1))
    pt = oracle.rand_fe(14000 + seed, 4 * kz)
    got = W.compress_lo(ctx, dev, k, pt, kz).download(4 << (k - kz))
    assert np.array_equal(got, oracle.compress_lo(poly, k, pt, kz)), (k, kz)


@pytest.mark.parametrize("seed", range(24))
def test_random_eq_eval_and_rounds(ctx, oracle, seed):
    rng = np.random.default_rng(15000 + seed)
    k = int(rng.integers(0, 15))
    pt = oracle.rand_fe(16000 + seed, 4 * k)
    scale = oracle.rand_fe(16500 + seed, 4)
    got = W.eq_table(ctx, pt, k, scale).download(4 << k)
    assert np.array_equal(got, oracle.eq_table(pt, k, scale)), k
    p = oracle.rand_fe(17000 + seed, 4 << k)
    dp = ctx.to_device(p)
    assert np.array_equal(W.eval_ext(ctx, dp, k, pt), oracle.eval_ext(p, k, pt)), k
    if k == 0:
        return
    w = oracle.rand_fe(18000 + seed, 4 << k)
    dw = ctx.to_device(w)
    c0, c2 = W.sumcheck_coeffs(ctx, dp, dw, k)
    e0, e2 = oracle.coeffs(p, w, k)
    assert np.array_equal(c0, e0) and np.array_equal(c2, e2), k
    r = oracle.rand_fe(19000 + seed, 4)
    po, wo = W.sumcheck_fold(ctx, dp, dw, k, r)
    assert np.array_equal(po.download(4 << (k - 1)), oracle.fix_lo(p, k, r)), k
    assert np.array_equal(wo.download(4 << (k - 1)), oracle.fix_lo(w, k, r)), k


@pytest.mark.parametrize("seed", range(24))
def test_random_combinations(ctx, oracle, seed):
    rng = np.random.default_rng(20000 + seed)
    k = int(rng.integers(2, 15))
    w = oracle.rand_fe(21000 + seed, 4 << k)
    alpha = oracle.rand_fe(21500 + seed, 4)
    n = int(rng.integers(1, 12))
    pts = oracle.rand_fe(22000 + seed, 4 * k * n)
    dw = ctx.to_device(w)
    W.combine_eqs(ctx, dw, k, pts, n, alpha)
    assert np.array_equal(dw.download(4 << k), oracle.combine_eqs(w, k, pts, n, alpha)), (k, n)
    n = int(rng.integers(1, 121))
    shift = int(rng.integers(0, 21))
    vars_ = oracle.rand_fe(23000 + seed, n)
    dw = ctx.to_device(w)
    W.combine_pows(ctx, dw, k, vars_, n, alpha, shift)
    assert np.array_equal(dw.download(4 << k),
                          oracle.combine_pows(w, k, vars_, n, alpha, shift)), (k, n, shift)
    scales = oracle.rand_fe(24000 + seed, 4 * n)
    dw = ctx.to_device(w)
    W.combine_pows_scaled(ctx, dw, k, vars_, n, scales)
    assert np.array_equal(dw.download(4 << k),
                          oracle.combine_pows_scaled(w, k, vars_, n, scales)), (k, n)
