"""The oracle prover and verifier, and the oracle's combination routines.

Ports of the reference's own tests: the prover/verifier round trip of
test_whir_poseidon (crates/whir/src/test.rs:256-282) on a subset of its sweep
(the full sweep runs in the GPU tests, where every GPU proof is checked
against the oracle), tamper rejection, and the naive-vs-split equivalence
tests of combine.rs (test_combine_eqs, test_combine_pows) and poly/src/test.rs.
"""
import numpy as np
import pytest

SWEEP = [(s, k, f, ir, n) for s in (1, 2, 0) for k in (4, 6, 9, 12) for f in (1, 2, 3)
         for ir in range(1, f + 1) for n in (1, 3) if (s + k + f + ir + n) % 2 == 0]


@pytest.mark.parametrize("s,k,f,ir,n", SWEEP)
def test_round_trip(oracle, s, k, f, ir, n):
    poly = oracle.rand_fe(1, 1 << k)
    params = (k, f, 1, ir, s, 32)
    proof, cp = oracle.prove(params, [poly], [k], [[0]] * n)
    rc, vcp = oracle.verify(params, [k], [[0]] * n, proof)
    assert rc == 0 and vcp == cp


def test_round_trip_bench_shape_small(oracle):
    k = 14
    poly = oracle.rand_fe(1, 1 << k)
    params = (k, 4, 2, 1, 1, 100)
    proof, cp = oracle.prove(params, [poly], [k], [[0]] * 4)
    rc, vcp = oracle.verify(params, [k], [[0]] * 4, proof)
    assert rc == 0 and vcp == cp


def test_stacked_round_trip(oracle):
    ks = [8, 6, 6, 8, 5]
    polys = [oracle.rand_fe(10 + i, 1 << x) for i, x in enumerate(ks)]
    groups = [[0, 3], [1, 2], [4], [3]]
    params = (10, 3, 1, 1, 1, 32)
    proof, cp = oracle.prove(params, polys, ks, groups)
    rc, vcp = oracle.verify(params, ks, groups, proof)
    assert rc == 0 and vcp == cp


def test_tampered_proofs_are_rejected(oracle):
    k = 9
    poly = oracle.rand_fe(2, 1 << k)
    params = (k, 2, 1, 1, 1, 32)
    proof, cp = oracle.prove(params, [poly], [k], [[0]])
    rng = np.random.default_rng(0)
    positions = sorted(set(int(x) for x in rng.integers(0, len(proof) // 4, 40)))
    rejected = 0
    for w in positions:
        b = bytearray(proof)
        v = int.from_bytes(b[4 * w:4 * w + 4], "little")
        b[4 * w:4 * w + 4] = ((v + 1) % oracle.P).to_bytes(4, "little")
        rc, vcp = oracle.verify(params, [k], [[0]], bytes(b))
        rejected += rc != 0 or vcp != cp
    assert rejected == len(positions)
    rc, _ = oracle.verify(params, [k], [[0]], proof[:-4])
    assert rc != 0


def test_wrong_claim_value_rejected(oracle):
    k = 8
    poly = oracle.rand_fe(3, 1 << k)
    params = (k, 2, 1, 1, 1, 32)
    proof, _ = oracle.prove(params, [poly], [k], [[0]])
    b = bytearray(proof)
    off = 32  # the claim's evaluation follows the 32-byte root
    v = int.from_bytes(b[off:off + 4], "little")
    b[off:off + 4] = ((v + 1) % oracle.P).to_bytes(4, "little")
    assert oracle.verify(params, [k], [[0]], bytes(b))[0] != 0


def _ext_mul(oracle, a, b):
    out = np.empty(4, np.uint32)
    oracle.lib().wo_ext_mul(oracle.ptr(np.ascontiguousarray(a, np.uint32)),
                            oracle.ptr(np.ascontiguousarray(b, np.uint32)), oracle.ptr(out))
    return out


def _ext_add(a, b, P):
    return ((a.astype(np.uint64) + b) % P).astype(np.uint32)


@pytest.mark.parametrize("k,n", [(1, 1), (3, 2), (5, 10), (6, 11)])
def test_combine_eqs_matches_naive(oracle, k, n):
    # combine_eq_ref of combine.rs: acc += sum_i alpha^i eq(z_i)
    alpha = oracle.rand_fe(5, 4)
    pts = oracle.rand_fe(6, 4 * k * n)
    want = np.zeros(4 << k, np.uint32)
    a = oracle.ext_one()
    for i in range(n):
        eq = oracle.eq_table(pts[4 * k * i:4 * k * (i + 1)], k, a)
        want = _ext_add(want, eq, oracle.P)
        a = _ext_mul(oracle, a, alpha)
    got = oracle.combine_eqs(np.zeros(4 << k, np.uint32), k, pts, n, alpha)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("k,n,shift", [(2, 1, 0), (4, 2, 11), (7, 11, 3)])
def test_combine_pows_matches_naive(oracle, k, n, shift):
    # combine_pow_ref of combine.rs: acc[j] += alpha^(shift+i) var_i^j
    L = oracle.lib()
    alpha = oracle.rand_fe(7, 4)
    vars_ = oracle.rand_fe(8, n)
    want = np.zeros((1 << k, 4), np.uint32)
    a = oracle.ext_one()
    for _ in range(shift):
        a = _ext_mul(oracle, a, alpha)
    for i in range(n):
        p = oracle.to_mont([1])[0]
        for j in range(1 << k):
            want[j] = _ext_add(want[j], np.array([L.wo_fe_mul(int(c), int(p)) for c in a],
                                                 np.uint32), oracle.P)
            p = L.wo_fe_mul(int(p), int(vars_[i]))
        a = _ext_mul(oracle, a, alpha)
    got = oracle.combine_pows(np.zeros(4 << k, np.uint32), k, vars_, n, alpha, shift)
    assert np.array_equal(got, want.ravel())


def test_compress_hi_lo_eval_consistency(oracle):
    # compress_hi then eval on the rest == eval (test_eq_compress_hi/lo of poly/src/test.rs)
    k, kz = 10, 6
    poly = oracle.rand_fe(9, 1 << k)
    z = oracle.rand_fe(10, 4 * k)
    full = oracle.eval_ext(_lift(oracle, poly), k, z)
    hi = oracle.compress_hi(poly, k, z[4 * (k - kz):], kz)
    assert np.array_equal(oracle.eval_ext(hi, k - kz, z[:4 * (k - kz)]), full)
    lo = oracle.compress_lo(poly, k, z[:4 * kz], kz)
    assert np.array_equal(oracle.eval_ext(lo, k - kz, z[4 * kz:]), full)


def _lift(oracle, poly):
    out = np.zeros((poly.size, 4), np.uint32)
    out[:, 0] = poly
    return out.ravel()


def _prod(oracle, p, w):
    acc = np.zeros(4, np.uint32)
    for i in range(p.size // 4):
        acc = _ext_add(acc, _ext_mul(oracle, p[4 * i:4 * i + 4], w[4 * i:4 * i + 4]), oracle.P)
    return acc


def test_round_polynomial_identity(oracle):
    # Expression::round (expr.rs:52-70): with h(0) = c0, h(1) = sum - c0,
    # h(2) = c2, the folded product equals h(r) (extrapolate_012, mod.rs:25-28)
    P = oracle.P
    k = 6
    p = oracle.rand_fe(11, 4 << k)
    w = oracle.rand_fe(12, 4 << k)
    total = _prod(oracle, p, w)
    c0, c2 = oracle.coeffs(p, w, k)
    r = oracle.rand_fe(13, 4)
    after = _prod(oracle, oracle.fix_lo(p, k, r), oracle.fix_lo(w, k, r))
    inv2 = oracle.to_mont([pow(2, -1, P)])[0]
    one = oracle.ext_one()
    two = _ext_add(one, one, P)
    neg = lambda a: ((P - a.astype(np.int64)) % P).astype(np.uint32)
    h1 = _ext_add(total, neg(c0), P)
    l0 = _ext_mul(oracle, _ext_mul(oracle, _ext_add(r, neg(one), P), _ext_add(r, neg(two), P)),
                  np.array([inv2, 0, 0, 0], np.uint32))
    l1 = _ext_mul(oracle, r, _ext_add(two, neg(r), P))
    l2 = _ext_mul(oracle, _ext_mul(oracle, r, _ext_add(r, neg(one), P)),
                  np.array([inv2, 0, 0, 0], np.uint32))
    h_r = _ext_add(_ext_add(_ext_mul(oracle, c0, l0), _ext_mul(oracle, h1, l1), P),
                   _ext_mul(oracle, c2, l2), P)
    assert np.array_equal(h_r, after)
