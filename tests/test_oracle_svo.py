"""The oracle's SVO claims and accumulators against brute force.

A port of the reference's test_accumulators (crates/whir/src/sumcheck/svo.rs:288-320):
for a random 12-variable polynomial P, a random point z and every number
l0 < 6 of SVO rounds, the claim value equals P(z), and the accumulator of
round r at a grid point u in {0, 1, 2}^(r+1) (u_0..u_{r-1} the base-3 digits
of the entry, u_r = 0 or 2) equals

    sum_x P(u, x) * eq(z)(u, x),

with P(u, .) and eq(z)(u, .) the multilinear extensions with their low
r + 1 variables fixed to u (compress_lo, checked on its own in the kernel
tests).  The products and the sum are computed here with numpy
arithmetic of this file's own: Montgomery products over KoalaBear
(p = 2^31 - 2^24 + 1) and the extension F[x]/(x^4 - 3).  The oracle's SVO
path feeds every proof's initial claims (svo.rs:64-91, 225-278).
"""
import numpy as np
import pytest

P = 0x7F000001
NEG_PINV = (-pow(P, -1, 1 << 32)) % (1 << 32)  # -p^-1 mod 2^32
R = (1 << 32) % P                               # Montgomery form of 1


def mont(x):
    return (x << 32) % P


def mmul(a, b):
    """Montgomery product of uint64 arrays of canonical words."""
    t = a * b
    m = ((t & 0xFFFFFFFF) * NEG_PINV) & 0xFFFFFFFF
    u = (t + m * P) >> 32
    return np.where(u >= P, u - P, u)


def madd(*xs):
    s = np.zeros_like(xs[0])
    for x in xs:
        s = (s + x) % P
    return s


W3 = np.uint64(mont(3))


def ext_mul(a, b):
    """(n, 4) x (n, 4) extension products mod x^4 - 3, Montgomery words."""
    a, b = a.astype(np.uint64), b.astype(np.uint64)
    m = lambda i, j: mmul(a[:, i], b[:, j])
    w = lambda x: mmul(x, np.full_like(x, W3))
    c0 = madd(m(0, 0), w(madd(m(1, 3), m(2, 2), m(3, 1))))
    c1 = madd(m(0, 1), m(1, 0), w(madd(m(2, 3), m(3, 2))))
    c2 = madd(m(0, 2), m(1, 1), m(2, 0), w(m(3, 3)))
    c3 = madd(m(0, 3), m(1, 2), m(2, 1), m(3, 0))
    return np.stack([c0, c1, c2, c3], axis=1)


def test_ext_mul_matches_the_oracle(oracle):
    a = oracle.rand_fe(1, 4 * 64).reshape(-1, 4)
    b = oracle.rand_fe(2, 4 * 64).reshape(-1, 4)
    got = ext_mul(a, b)
    for i in range(64):
        want = np.zeros(4, np.uint32)
        oracle.lib().wo_ext_mul(oracle.ptr(np.ascontiguousarray(a[i])),
                                oracle.ptr(np.ascontiguousarray(b[i])), oracle.ptr(want))
        assert [int(x) for x in got[i]] == [int(x) for x in want]


def fold_low(oracle, ext_words, k, u):
    """The multilinear extension of an extension-valued table with its low
    len(u) variables fixed to the base-field values u, coordinate by
    coordinate (the fixing is linear over the base field)."""
    l = len(u)
    point = np.zeros(4 * l, np.uint32)
    point[0::4] = [mont(x) for x in u]
    t = ext_words.reshape(-1, 4)
    out = np.zeros((1 << (k - l), 4), np.uint64)
    for c in range(4):
        col = np.ascontiguousarray(t[:, c])
        out[:, c] = oracle.compress_lo(col, k, point, l).reshape(-1, 4)[:, 0]
    return out


@pytest.mark.parametrize("l0", range(6))
def test_accumulators(oracle, l0):
    k = 12
    poly = oracle.rand_fe(1, 1 << k)
    z = oracle.rand_fe(2, 4 * k)
    value, acc = oracle.svo_accumulators(poly, k, z, l0)
    ext_poly = np.zeros(4 << k, np.uint32)
    ext_poly[0::4] = poly
    assert np.array_equal(value, oracle.eval_ext(ext_poly, k, z))
    eq = oracle.eq_table(z, k, oracle.ext_one())
    acc = acc.reshape(-1, 4)
    off = 0
    for r in range(l0):
        n = 3 ** r
        for which, last in ((0, 0), (1, 2)):
            for t in range(n):
                u, tt = [], t
                for _ in range(r):
                    u.append(tt % 3)
                    tt //= 3
                u.append(last)
                pu = fold_low(oracle, ext_poly, k, u)
                eu = fold_low(oracle, eq, k, u)
                want = ext_mul(pu, eu).sum(axis=0) % P
                assert [int(x) for x in acc[off + which * n + t]] == [int(x) for x in want], \
                    (l0, r, which, t)
        off += 2 * n
    assert off == len(acc)
