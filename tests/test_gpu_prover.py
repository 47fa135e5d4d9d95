"""Full GPU proofs through the C ABI, byte-identical to the oracle prover and
accepted by the oracle verifier.

The parameter sweep follows the reference's test_whir_poseidon
(crates/whir/src/test.rs:256-282: three soundness assumptions, k = 4..12,
folding 1..3, initial_reduction 1..folding, 1..4 claims, rate 1, 32-bit
security) on a subset that keeps the run short, plus the benchmark shapes
(k = 20 and k = 24, folding 4), foldings 5 and 6, the reference's whir_bench
shape (k = 25, folding 5) and stacked multi-polynomial layouts.
"""
import itertools

import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu

SWEEP = [(s, k, f, ir, n)
         for s in (1, 2, 0) for k in (4, 5, 7, 9, 12) for f in (1, 2, 3)
         for ir in range(1, f + 1) for n in (1, 4)
         if (k + f + ir + n + s) % 3 == 0 or k == 12]


def check(ctx, oracle, params, polys, poly_k, groups):
    proof, cp = W.prove_harness(ctx, params, polys, poly_k, groups)
    want, wcp = oracle.prove(params, polys, poly_k, groups)
    assert len(proof) == len(want)
    assert proof == want
    assert cp == wcp
    rc, vcp = oracle.verify(params, poly_k, groups, proof)
    assert rc == 0 and vcp == cp
    assert W.verify(params, poly_k, groups, proof) == (0, cp)  # the library's verifier


@pytest.mark.parametrize("s,k,f,ir,n", SWEEP)
def test_whir_sweep(ctx, oracle, s, k, f, ir, n):
    poly = oracle.rand_fe(1, 1 << k)
    check(ctx, oracle, (k, f, 1, ir, s, 32), [poly], [k], [[0]] * n)


@pytest.mark.parametrize("k,rate,n", [(10, 2, 2), (16, 1, 1), (20, 1, 1), (18, 2, 4)])
def test_whir_folding4_security100(ctx, oracle, k, rate, n):
    poly = oracle.rand_fe(1, 1 << k)
    check(ctx, oracle, (k, 4, rate, 1, 1, 100), [poly], [k], [[0]] * n)


# foldings 5 and 6: base rows of 32 / 64 words, extension rows of 128 / 256
# words, SVO grids of 3^5 / 3^6 points, fold_with_code over 32 / 64 rows
@pytest.mark.parametrize("params,n", [((14, 5, 1, 1, 1, 100), 2), ((16, 5, 2, 1, 1, 100), 2),
                                      ((13, 5, 1, 3, 0, 32), 1), ((12, 5, 1, 5, 2, 32), 4),
                                      ((15, 6, 1, 1, 1, 100), 3), ((18, 6, 2, 2, 1, 100), 1)])
def test_whir_folding5_6(ctx, oracle, params, n):
    k = params[0]
    poly = oracle.rand_fe(2, 1 << k)
    check(ctx, oracle, params, [poly], [k], [[0]] * n)


@pytest.mark.parametrize("params", [(6, 1, 0, 1, 1, 32), (9, 3, 0, 2, 2, 64),
                                    (12, 4, 0, 1, 1, 100), (14, 5, 0, 1, 0, 100)])
def test_rate_one(ctx, oracle, params):
    # log_inv_rate 0: no STIR queries in any round (Rust's saturating cast of
    # the query count, params.rs:118-122); nothing is opened or gathered
    k = params[0]
    poly = oracle.rand_fe(8, 1 << k)
    check(ctx, oracle, params, [poly], [k], [[0]] * 2)


# the largest foldings: 2^7 / 2^8-word base rows, 2^10-word extension rows
# (the generic leaf sponge), SVO claims over 2^8 columns
@pytest.mark.parametrize("params", [(12, 7, 1, 2, 0, 32), (16, 8, 1, 1, 1, 100),
                                    (14, 7, 2, 3, 2, 64), (10, 8, 1, 1, 1, 32)])
def test_whir_folding7_8(ctx, oracle, params):
    k = params[0]
    poly = oracle.rand_fe(9, 1 << k)
    check(ctx, oracle, params, [poly], [k], [[0]] * 2)


@pytest.mark.parametrize("params", [(12, 2, 1, 1, 0, 1000), (14, 4, 1, 1, 0, 1200)])
def test_many_queries(ctx, oracle, params):
    # unique decoding at 1000-1200 bits: 2410 and 2892 STIR queries, past the
    # 2048 indexes the opening gather takes by value (the uploaded-index
    # path) and near the 3072 the pow-claim combination holds
    k = params[0]
    poly = oracle.rand_fe(4, 1 << k)
    check(ctx, oracle, params, [poly], [k], [[0]] * 2)


def test_reference_bench_shape_k25(ctx, oracle):
    # the reference's own benchmark, whir_bench (crates/whir/src/test.rs:284-290):
    # k = 25, folding 5, rate 1/2, initial_reduction 3, JohnsonBound, 123-bit, 1 claim
    poly = oracle.rand_fe(1, 1 << 25)
    check(ctx, oracle, (25, 5, 1, 3, 1, 123), [poly], [25], [[0]])


@pytest.mark.parametrize("params,n", [((10, 2, 1, 1, 1, 32), 0), ((12, 4, 1, 1, 1, 100), 12),
                                      ((11, 3, 1, 1, 1, 32), 20)])
def test_claim_counts(ctx, oracle, params, n):
    # no claim at all (only the OOD claims), and more points than the split
    # eq tables take by value (8): the uploaded-point path
    k = params[0]
    poly = oracle.rand_fe(5, 1 << k)
    check(ctx, oracle, params, [poly], [k], [[0]] * n)


def test_stacked_layout(ctx, oracle):
    # several polynomials of different sizes in one layout (ProverStack::layout)
    ks = [8, 6, 6, 8, 5]
    polys = [oracle.rand_fe(10 + i, 1 << k) for i, k in enumerate(ks)]
    k = int(np.ceil(np.log2(sum(1 << x for x in ks))))
    groups = [[0, 3], [1, 2], [4], [3]]
    check(ctx, oracle, (k, 3, 1, 1, 1, 32), polys, ks, groups)


@pytest.mark.parametrize("f,ir,s,sec", [(5, 2, 1, 100), (6, 1, 0, 32)])
def test_stacked_layout_folding5_6(ctx, oracle, f, ir, s, sec):
    ks = [10, 8, 10, 7, 8]
    polys = [oracle.rand_fe(30 + i, 1 << k) for i, k in enumerate(ks)]
    k = int(np.ceil(np.log2(sum(1 << x for x in ks))))
    groups = [[0, 2], [1, 4], [3], [2]]
    check(ctx, oracle, (k, f, 1, ir, s, sec), polys, ks, groups)


def test_one_prover_across_layouts(ctx, oracle):
    # one Whir object proves different stacks in turn (polynomial counts,
    # sizes and claim groups change between proofs); each proof equals the
    # oracle's
    params = (10, 3, 1, 1, 1, 32)
    w = W.Whir(ctx, *params)
    for ks, groups in [([8, 6, 6, 8, 5], [[0, 3], [1, 2], [4], [3]]), ([10], [[0], [0]]),
                       ([9, 9], [[0, 1]]), ([8, 6, 6, 8, 5], [[4], [0]])]:
        polys = [oracle.rand_fe(40 + i, 1 << k) for i, k in enumerate(ks)]
        proof, cp = W.prove_harness(ctx, None, polys, ks, groups, whir=w)
        want, wcp = oracle.prove(params, polys, ks, groups)
        assert proof == want and cp == wcp
    w.close()


def _emul(a, b):
    # Ext4 product of Montgomery words (x^4 = 3), for expanding points in Python
    rinv = pow(2 ** 32, -1, W.P)
    c = [0] * 4
    for i in range(4):
        for j in range(4):
            t = a[i] * b[j] * rinv % W.P
            c[(i + j) % 4] += t if i + j < 4 else 3 * t
    return [x % W.P for x in c]


def test_fine_grained_calls_match_whir_prove(ctx, oracle):
    # whir_commit, then for each claim a transcript-drawn point expanded as
    # the harness does (Point::expand: z_i = x^(2^i), crates/whir/src/test.rs:225-228)
    # through whir_stack_eval, then whir_open: the bytes of whir_prove
    k = 12
    params = (k, 4, 1, 1, 1, 100)
    poly = oracle.rand_fe(77, 1 << k)
    want, wcp = W.prove_harness(ctx, params, [poly], [k], [[0], [0]])
    w = W.Whir(ctx, *params)
    t = W.PoseidonWriter()
    w.commit(t, [poly], [k])
    for _ in range(2):
        x = [int(v) for v in t.draw()]
        pt = []
        for _ in range(k):
            pt.append(x)
            x = _emul(x, x)
        w.stack_eval(t, 0, np.array(pt, np.uint32).ravel())
    w.open(t)
    cp = t.draw_base()
    assert t.finalize() == want and cp == wcp
    w.close()


def test_proof_is_deterministic_across_calls(ctx, oracle):
    poly = oracle.rand_fe(5, 1 << 12)
    w = W.Whir(ctx, 12, 4, 1, 1, 1, 100)
    a = W.prove_harness(ctx, None, [poly], [12], [[0]], whir=w)
    b = W.prove_harness(ctx, None, [poly], [12], [[0]], whir=w)
    assert a == b


def test_device_resident_input(ctx, oracle):
    k = 14
    poly = oracle.rand_fe(3, 1 << k)
    w = W.Whir(ctx, k, 4, 2, 1, 1, 100)
    t = W.PoseidonWriter()
    w.prove(t, ctx.to_device(poly), [k], [[0], [0]])
    cp = t.draw_base()
    want, wcp = oracle.prove((k, 4, 2, 1, 1, 100), [poly], [k], [[0], [0]])
    assert t.finalize() == want and cp == wcp


def test_bench_shape_k24(ctx, oracle):
    # the benchmark workload: k = 24, rate 1/4, folding 4, 4 claims, 100-bit JB
    k = 24
    poly = oracle.rand_fe(1, 1 << k)
    check(ctx, oracle, (k, 4, 2, 1, 1, 100), [poly], [k], [[0]] * 4)


@pytest.mark.parametrize("k,rate", [(26, 2), (24, 4)])
def test_max_sizes_verify(ctx, oracle, k, rate):
    # the largest codewords the 2^24 two-adic subgroup allows (2^24 rows of
    # 16 words): byte-identical to the oracle prover (about 20 s of host
    # work on 16 cores), accepted by both verifiers, deterministic
    poly = W.random_field(9 + k, 1 << k)
    params = (k, 4, rate, 1, 1, 100)
    proof, cp = W.prove_harness(ctx, params, [poly], [k], [[0]] * 2)
    want, wcp = oracle.prove(params, [poly], [k], [[0]] * 2)
    assert proof == want and cp == wcp
    assert W.verify(params, [k], [[0]] * 2, proof) == (0, cp)
    rc, vcp = oracle.verify(params, [k], [[0]] * 2, proof)
    assert rc == 0 and vcp == cp
    again, cp2 = W.prove_harness(ctx, params, [poly], [k], [[0]] * 2)
    assert again == proof and cp2 == cp


@pytest.mark.parametrize("k,f,rate", [(12, 4, 2), (18, 4, 2), (9, 1, 1)])
def test_pinned_host_input(ctx, oracle, k, f, rate):
    # the bench's end-to-end input: a polynomial in pinned host memory
    torch = pytest.importorskip("torch")
    poly = oracle.rand_fe(21 + k, 1 << k)
    pinned = torch.empty(1 << k, dtype=torch.int32, pin_memory=True)
    host = pinned.numpy().view(np.uint32)
    host[:] = poly
    params = (k, f, rate, 1, 1, 100 if f == 4 else 32)
    _, h2d0, _ = ctx.counters()
    proof, cp = W.prove_harness(ctx, params, host, [k], [[0], [0]])
    _, h2d1, _ = ctx.counters()
    assert h2d1 - h2d0 >= 4 << k  # the polynomial crossed the host link, counted
    want, wcp = oracle.prove(params, [poly], [k], [[0], [0]])
    assert proof == want and cp == wcp
    assert np.array_equal(host, poly)  # the input is only read
