"""Host-side logic of the product library, run without a GPU.

libwhir_gb300.so loads on a machine without a GPU; its host-only entry points
(Poseidon2 permutation, seeded field sampling, the Fiat-Shamir transcript)
are checked here against the golden vectors and against the oracle, and its
argument checks against the C-ABI error contract.
"""
import ctypes
import json
import os

import numpy as np
import pytest

import whir_gb300 as W

HERE = os.path.dirname(os.path.abspath(__file__))
G = json.load(open(os.path.join(HERE, "golden", "golden.json")))


@pytest.mark.parametrize("width", [16, 24])
def test_poseidon2_host_matches_golden(width):
    for s, want in G[f"p2_{width}"]:
        assert list(W.poseidon2_permute(width, s)) == want


def test_random_field_matches_golden_and_oracle(oracle):
    assert list(W.random_field(1, 64)) == G["rand_fe_seed1_first64"]
    assert np.array_equal(W.random_field(9, 10000), oracle.rand_fe(9, 10000))


def test_transcript_challenger_sequence():
    # replay the golden challenger sequence through the transcript: observes
    # are base-field writes, samples are base-field draws
    t = W.PoseidonWriter()
    for op, v in G["challenger"]:
        if op == "observe":
            t.write_base(v)
        else:
            assert t.draw_base() == v
    written = [v for op, v in G["challenger"] if op == "observe"]
    raw = t.finalize()
    assert list(np.frombuffer(raw, np.uint32)) == written


def test_transcript_ext_draw_and_bits():
    # Challenge<F, Ext>::draw samples four base elements (coefficient 0 first);
    # ChallengeBits::draw masks the canonical value of one sample
    a, b = W.PoseidonWriter(), W.PoseidonWriter()
    for t in (a, b):
        t.write(np.array([1, 2, 3, 4], np.uint32))
    e = a.draw()
    s = [b.draw_base() for _ in range(4)]
    assert list(e) == s
    x = a.draw_base()
    y = b.draw_bits(20)
    assert y == (x * pow(2 ** 32, -1, W.P) % W.P) & ((1 << 20) - 1)


def test_abi_error_contract():
    L = W.lib()
    s = np.zeros(20, np.uint32)
    assert L.whir_poseidon2_permute(20, s.ctypes.data_as(W.u32p)) == -1
    assert b"width" in L.whir_last_error()
    s = np.full(16, W.P, np.uint32)
    assert L.whir_poseidon2_permute(16, s.ctypes.data_as(W.u32p)) == -1
    t = W.PoseidonWriter()
    out = ctypes.c_size_t()
    assert L.whir_transcript_draw_bits(t.h, 31, ctypes.byref(out)) == -1
    assert L.whir_transcript_write_base(t.h, W.P) == -1
    small = ctypes.create_string_buffer(1)
    t.write_base(5)
    assert L.whir_transcript_bytes(t.h, small, 1) == -4
