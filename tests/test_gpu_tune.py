"""Launch-split choices (whir_tune_*, whir_autotune) change only the time:
trees, DFTs and whole proofs stay byte-identical to the oracle under every
choice."""
import numpy as np
import pytest

import whir_gb300 as W

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _reset():
    W.tune_reset()
    yield
    W.tune_reset()


@pytest.mark.parametrize("log_h", [11, 16, 18])
def test_tree_splits(ctx, oracle, log_h):
    rows = oracle.rand_fe(300 + log_h, 16 << log_h)
    want = oracle.merkle_tree(rows, log_h, 16)
    dev = ctx.to_device(rows)
    tried = 0
    for wl in range(12, 19):
        for sp in (-1, 0, 1):
            try:
                W.tune_tree(log_h, wl, sp)
            except W.WhirError:
                continue   # outside the valid range for this height
            t = W.MerkleTree(ctx, dev, log_h, 16)
            assert np.array_equal(t.levels(), want), (wl, sp)
            t.close()
            tried += 1
    assert tried >= 3


@pytest.mark.parametrize("log_h,width,h_in", [(16, 64, 2048), (20, 16, 1 << 18), (13, 8, 4096)])
def test_dft_splits(ctx, oracle, log_h, width, h_in):
    x = oracle.rand_fe(400 + log_h, h_in * width)
    want = oracle.dft_batch(x, h_in, width, log_h)
    dev = ctx.to_device(x)
    tried = 0
    for bias in (-2, -1, 0, 1, 2):
        try:
            W.tune_dft(log_h, width, bias)
        except W.WhirError:
            continue
        got = W.dft_batch(ctx, dev, h_in, width, log_h).download(width << log_h)
        assert np.array_equal(got, want), bias
        tried += 1
    assert tried >= 2


def test_autotune_then_prove(ctx, oracle):
    report = W.autotune(ctx, 8, 18)
    assert "tree log_h=18" in report and "dft log_h=" in report
    k = 16
    poly = oracle.rand_fe(77, 1 << k)
    params = (k, 4, 2, 1, 1, 100)
    proof, cp = W.prove_harness(ctx, params, [poly], [k], [[0]] * 2)
    want, wcp = oracle.prove(params, [poly], [k], [[0]] * 2)
    assert proof == want and cp == wcp


def test_tune_argument_checks():
    with pytest.raises(W.WhirError):
        W.tune_tree(16, 30, 0)
    with pytest.raises(W.WhirError):
        W.tune_dft(16, 16, 7)
