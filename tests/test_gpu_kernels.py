"""GPU kernels through the C ABI against the oracle, bit for bit.

Each test mirrors one of the reference's equivalence tests for the same
routine (crates/poly/src/test.rs, crates/whir/src/sumcheck/combine.rs tests,
crates/merkle/src/lib.rs tests) and compares the CUDA result with the CPU
restatement on seeded inputs.  Field arithmetic is exact, so the tolerance is
zero.
"""
import ctypes

import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


def rand(oracle, seed, n):
    return oracle.rand_fe(seed, n)


@pytest.mark.parametrize("log_h,width,h_in", [
    (0, 16, 1), (1, 16, 1), (3, 2, 4), (5, 4, 8), (8, 16, 64), (11, 16, 1024), (11, 64, 512),
    (12, 16, 1024), (13, 8, 8192), (16, 64, 8192), (17, 16, 65536), (20, 16, 262144),
    (21, 64, 65536), (22, 16, 1 << 20), (4, 8, 16), (6, 4, 40), (9, 16, 300), (14, 8, 100),
    (15, 32, 1000),
    # two passes over a zero-padded input (pass 1 skips the zero stages):
    # ragged h_in, 4-column tiles, and a padding too deep for the short form
    (18, 8, 70000), (19, 4, 40000), (14, 16, 4097), (20, 8, 4000), (17, 8, 10000),
    # the row widths of foldings 5 and 6 (base 32 / 64, extension 128 / 256)
    (16, 32, 1 << 15), (13, 128, 1 << 10), (12, 256, 1 << 9),
    # 2^12-point coset transforms on 4-column tiles (the extension round two
    # of the k = 24 proof is (20, 64, 4096))
    (20, 64, 4096), (14, 16, 4096), (18, 8, 2049), (13, 4, 3000)])
def test_dft_batch(ctx, oracle, log_h, width, h_in):
    x = rand(oracle, 7 + log_h, h_in * width)
    want = oracle.dft_batch(x, h_in, width, log_h)
    got = W.dft_batch(ctx, ctx.to_device(x), h_in, width, log_h).download(width << log_h)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("log_h,row_len", [(0, 16), (1, 16), (2, 3), (3, 16), (5, 64), (7, 8),
                                           (10, 16), (12, 64), (16, 16), (17, 16), (18, 16),
                                           # foldings 5 and 6: base rows 32 / 64, extension rows 128 / 256
                                           (9, 32), (8, 128), (6, 256), (4, 48)])
def test_merkle_commit_and_open(ctx, oracle, log_h, row_len):
    rows = rand(oracle, 100 + log_h, row_len << log_h)
    want = oracle.merkle_tree(rows, log_h, row_len)
    t = W.MerkleTree(ctx, ctx.to_device(rows), log_h, row_len)
    got = t.levels()
    assert np.array_equal(got, want)
    assert np.array_equal(t.root, want[-8:])
    n = 1 << log_h
    idx = sorted(set([0, n - 1, n // 2, (7 * n) // 11 % n]))
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
    t.close()


@pytest.mark.parametrize("log_h,row_len", [(21, 32), (18, 128)])
def test_merkle_reference_bench_shapes(ctx, oracle, log_h, row_len):
    # bench_merkle_base_packed (2^21 rows of 32 base elements) and
    # bench_merkle_ext_packed (2^18 rows of 32 extension elements = 128 words),
    # crates/merkle/src/lib.rs:314-349 and :384-420: every level and one opening
    rows = oracle.rand_fe(0, row_len << log_h)
    want = oracle.merkle_tree(rows, log_h, row_len)
    t = W.MerkleTree(ctx, ctx.to_device(rows), log_h, row_len)
    assert np.array_equal(t.levels(), want)
    i = (5 << log_h) // 7
    op = t.open([i])
    assert np.array_equal(op[0, :row_len], rows[i * row_len:(i + 1) * row_len])
    t.close()


@pytest.mark.parametrize("k", [0, 1, 5, 12, 20])
def test_eq_table(ctx, oracle, k):
    pt = rand(oracle, 3, 4 * k)
    scale = rand(oracle, 4, 4)
    got = W.eq_table(ctx, pt, k, scale).download(4 << k)
    assert np.array_equal(got, oracle.eq_table(pt, k, scale))


@pytest.mark.parametrize("k,ks", [(4, 4), (5, 1), (8, 4), (14, 4), (20, 4), (24, 4), (16, 5)])
def test_compress_hi(ctx, oracle, k, ks):
    poly = rand(oracle, 11, 1 << k)
    kz = k - ks
    pt = rand(oracle, 12, 4 * kz)
    got = W.compress_hi(ctx, ctx.to_device(poly), k, pt, kz)
    assert np.array_equal(got, oracle.compress_hi(poly, k, pt, kz))


@pytest.mark.parametrize("k,kz", [(4, 4), (6, 1), (10, 4), (20, 4), (24, 4)])
def test_compress_lo(ctx, oracle, k, kz):
    poly = rand(oracle, 13, 1 << k)
    pt = rand(oracle, 14, 4 * kz)
    got = W.compress_lo(ctx, ctx.to_device(poly), k, pt, kz).download(4 << (k - kz))
    assert np.array_equal(got, oracle.compress_lo(poly, k, pt, kz))


@pytest.mark.parametrize("k", [0, 1, 4, 9, 16, 20])
def test_eval_ext(ctx, oracle, k):
    poly = rand(oracle, 15, 4 << k)
    pt = rand(oracle, 16, 4 * k)
    got = W.eval_ext(ctx, ctx.to_device(poly), k, pt)
    assert np.array_equal(got, oracle.eval_ext(poly, k, pt))


@pytest.mark.parametrize("k", [1, 2, 7, 16, 20])
def test_coeffs_and_fold(ctx, oracle, k):
    p = rand(oracle, 17, 4 << k)
    w = rand(oracle, 18, 4 << k)
    dp, dw = ctx.to_device(p), ctx.to_device(w)
    c0, c2 = W.sumcheck_coeffs(ctx, dp, dw, k)
    e0, e2 = oracle.coeffs(p, w, k)
    assert np.array_equal(c0, e0) and np.array_equal(c2, e2)
    r = rand(oracle, 19, 4)
    po, wo = W.sumcheck_fold(ctx, dp, dw, k, r)
    assert np.array_equal(po.download(4 << (k - 1)), oracle.fix_lo(p, k, r))
    assert np.array_equal(wo.download(4 << (k - 1)), oracle.fix_lo(w, k, r))


@pytest.mark.parametrize("k,n", [(2, 1), (5, 2), (9, 10), (9, 11), (16, 2)])
def test_combine_eqs(ctx, oracle, k, n):
    w = rand(oracle, 20, 4 << k)
    pts = rand(oracle, 21, 4 * k * n)
    alpha = rand(oracle, 22, 4)
    dw = ctx.to_device(w)
    W.combine_eqs(ctx, dw, k, pts, n, alpha)
    assert np.array_equal(dw.download(4 << k), oracle.combine_eqs(w, k, pts, n, alpha))


@pytest.mark.parametrize("k,n,shift", [(2, 1, 0), (5, 2, 11), (9, 10, 3), (9, 11, 11), (16, 52, 2),
                                         (17, 108, 0), (18, 1, 5), (18, 300, 1)])
def test_combine_pows(ctx, oracle, k, n, shift):
    w = rand(oracle, 23, 4 << k)
    vars_ = rand(oracle, 24, n)
    alpha = rand(oracle, 25, 4)
    dw = ctx.to_device(w)
    W.combine_pows(ctx, dw, k, vars_, n, alpha, shift)
    assert np.array_equal(dw.download(4 << k), oracle.combine_pows(w, k, vars_, n, alpha, shift))
    scales = rand(oracle, 26, 4 * n)
    dw2 = ctx.to_device(w)
    W.combine_pows_scaled(ctx, dw2, k, vars_, n, scales)
    assert np.array_equal(dw2.download(4 << k), oracle.combine_pows_scaled(w, k, vars_, n, scales))


class Shifted:
    """A device array starting one word past a 16-byte boundary: extension
    elements there are 4-byte aligned only, which the kernels must accept."""

    def __init__(self, ctx, arr):
        arr = np.ascontiguousarray(arr, np.uint32)
        self.ctx = ctx
        self.base = W.DeviceArray(ctx, arr.nbytes + 16)
        self.ptr = self.base.ptr + 4
        W._check(W.lib().whir_copy_to_device(ctx.h, self.ptr, arr.ctypes.data, arr.nbytes))

    def download(self, n_words):
        out = np.empty(n_words, np.uint32)
        W._check(W.lib().whir_copy_to_host(self.ctx.h, out.ctypes.data, self.ptr, out.nbytes))
        return out


@pytest.mark.parametrize("k", [9, 16])
def test_unaligned_extension_arrays(ctx, oracle, k):
    # the word-by-word variants of the kernels that otherwise move extension
    # elements as 16-byte vectors
    p = rand(oracle, 31, 4 << k)
    w = rand(oracle, 32, 4 << k)
    pt = rand(oracle, 33, 4 * k)
    assert np.array_equal(W.eval_ext(ctx, Shifted(ctx, p), k, pt), oracle.eval_ext(p, k, pt))
    c0, c2 = W.sumcheck_coeffs(ctx, Shifted(ctx, p), Shifted(ctx, w), k)
    e0, e2 = oracle.coeffs(p, w, k)
    assert np.array_equal(c0, e0) and np.array_equal(c2, e2)
    r = rand(oracle, 34, 4)
    po, wo = W.sumcheck_fold(ctx, Shifted(ctx, p), Shifted(ctx, w), k, r)
    assert np.array_equal(po.download(4 << (k - 1)), oracle.fix_lo(p, k, r))
    assert np.array_equal(wo.download(4 << (k - 1)), oracle.fix_lo(w, k, r))
    pts = rand(oracle, 35, 4 * k * 3)
    alpha = rand(oracle, 36, 4)
    dw = Shifted(ctx, w)
    W.combine_eqs(ctx, dw, k, pts, 3, alpha)
    assert np.array_equal(dw.download(4 << k), oracle.combine_eqs(w, k, pts, 3, alpha))
    vars_ = rand(oracle, 37, 5)
    dw = Shifted(ctx, w)
    W.combine_pows(ctx, dw, k, vars_, 5, alpha, 1)
    assert np.array_equal(dw.download(4 << k), oracle.combine_pows(w, k, vars_, 5, alpha, 1))
    base = rand(oracle, 38, 1 << k)
    rs = rand(oracle, 39, 4 * 4)
    got = W.compress_lo(ctx, Shifted(ctx, base), k, rs, 4).download(4 << (k - 4))
    assert np.array_equal(got, oracle.compress_lo(base, k, rs, 4))


def test_abi_errors_leave_the_context_usable(ctx, oracle):
    # bad shapes and parameters are refused with WHIR_ERR_ARG before any
    # launch, and the context keeps working afterwards
    L = W.lib()
    x = rand(oracle, 3, 64 * 16)
    dev = ctx.to_device(x)
    out = ctx.alloc(4 * (16 << 8))
    assert L.whir_dft_batch(ctx.h, dev.ptr, 64, 16, 25, out.ptr) == -1  # beyond two-adicity
    assert b"log_h" in L.whir_last_error()
    assert L.whir_dft_batch(ctx.h, dev.ptr, 64, 0, 8, out.ptr) == -1     # no columns
    assert L.whir_dft_batch(ctx.h, dev.ptr, 512, 16, 8, out.ptr) == -1   # input taller than the code
    h, root = W.vp(), np.zeros(8, np.uint32)
    assert L.whir_merkle_commit(ctx.h, dev.ptr, 6, 0, ctypes.byref(h),
                                root.ctypes.data_as(W.u32p)) == -1         # empty rows
    t = W.MerkleTree(ctx, dev, 6, 16)
    with pytest.raises(W.WhirError):
        t.open([64])                                                     # past the last leaf
    with pytest.raises(W.WhirError):
        W.Whir(ctx, 12, 9, 1, 1, 1, 100)                                 # folding above 8
    with pytest.raises(W.WhirError):
        W.Whir(ctx, 3, 4, 1, 1, 1, 100)                                  # k below the folding
    with pytest.raises(W.WhirError):
        W.Whir(ctx, 10, 2, 1, 5, 1, 32)                                  # a negative round rate
    got = W.dft_batch(ctx, dev, 64, 16, 8).download(16 << 8)
    assert np.array_equal(got, oracle.dft_batch(x, 64, 16, 8))
    assert np.array_equal(t.levels(), oracle.merkle_tree(x, 6, 16))
    t.close()
