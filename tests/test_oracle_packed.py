"""The oracle's lane-packed Poseidon2 (the timed CPU baseline) gives the same
Merkle trees and proofs as its scalar permutation (the parity checker)."""
import numpy as np

from oracle import oracle as O


def test_packed_trees_equal_scalar():
    O.lib()
    for log_h, row_len, seed in ((0, 16, 1), (3, 16, 2), (9, 16, 3), (7, 64, 4), (5, 7, 5),
                                 (6, 33, 6), (4, 0, 7), (10, 32, 8)):
        rows = O.rand_fe(seed, max(1, (1 << log_h) * row_len))[: (1 << log_h) * row_len]
        O.set_packed(False)
        want = O.merkle_tree(rows, log_h, row_len)
        O.set_packed(True)
        try:
            got = O.merkle_tree(rows, log_h, row_len)
        finally:
            O.set_packed(False)
        assert np.array_equal(got, want), (log_h, row_len)


def test_packed_proof_equals_scalar():
    params = (14, 4, 2, 1, 1, 100)
    poly = O.rand_fe(9, 1 << 14)
    want = O.prove(params, [poly], [14], [[0], [0]])
    O.set_packed(True)
    try:
        got = O.prove(params, [poly], [14], [[0], [0]])
    finally:
        O.set_packed(False)
    assert got == want
