"""bench.py's work accounting, on the CPU.

The integer roofline of the leaf hash divides the width-24 permutations of
one proof by the leaf-hash time, so the permutation count must match the
commitments a proof makes.  These tests pin `leaf_permutations` against the
row counts of each commitment (one codeword row per leaf; a base row of
16 words is one permutation, an extension row of 64 words four) under the
reference's round rule (crates/whir/src/whir.rs:150-165: the domain of
round r's codeword is 2^(k + log_inv_rate - (initial_reduction + r)) points,
the base codeword's 2^(k + log_inv_rate), in rows of 2^4 points), with the
number of extension commitments taken from the oracle's restatement of the
parameters; and they pin the structural instruction count of the
permutation and the roofline arithmetic.
"""
import pytest

import bench

# (k, log_inv_rate, initial_reduction) -> rows of the base commitment, then of
# each extension commitment (folding 4)
SHAPES = {
    (24, 2, 1): [22, 21, 20, 19, 18],  # the bench workload
    (20, 1, 1): [17, 16, 15, 14],
    (16, 2, 1): [14, 13, 12],
    (22, 2, 1): [20, 19, 18, 17],
    (14, 1, 1): [11, 10],
    (24, 2, 2): [22, 20, 19, 18, 17],  # initial_reduction 2: round 0's domain a quarter of the base's
}


@pytest.mark.parametrize("shape", sorted(SHAPES))
def test_leaf_permutations_match_the_commitments(shape, oracle):
    k, rate, ir = shape
    rows = SHAPES[shape]
    want = (1 << rows[0]) + 4 * sum(1 << r for r in rows[1:])
    assert bench.leaf_permutations(k, 4, rate, ir) == want
    rounds, _final = oracle.number_of_rounds(4, k)
    assert len(rows) - 1 == rounds


def test_bench_workload_permutations():
    w = bench.WORKLOAD
    perms = bench.leaf_permutations(w["k"], w["folding"], w["rate"], w["initial_reduction"])
    assert perms == 19_922_944  # 2^22 + 4 (2^21 + 2^20 + 2^19 + 2^18)


def test_structural_instruction_count():
    # 8 external rounds of 24 S-boxes (11 each), 9 light MDS layers (330),
    # 23 internal layers of S-box + lane sum (28) + lane updates (145)
    assert bench.p2_structural_instructions(24) == 8 * 24 * 11 + 9 * 330 + 23 * (11 + 28 + 145)
    assert bench.p2_structural_instructions(24) == 9314
    assert len(bench.P2_STRUCTURE[24]["diag"]) == 24
    # the roofline divides by the tighter (smaller) of the two counts
    assert bench.LEAF_INSTR_PER_PERM24 < bench.p2_structural_instructions(24)


def test_integer_roofline_arithmetic():
    prof = {"leaf_hash": {"ms_per_step": 5.6}}
    r = bench.integer_roofline(24, prof, {"sm_mhz": 2000.0})
    achieved = 19_922_944 / 5.6e-3
    peak = 152 * 4 * 32 * 2000e6 / bench.LEAF_INSTR_PER_PERM24
    assert r["achieved"] == pytest.approx(achieved)
    assert r["peak"] == pytest.approx(peak)
    assert r["frac"] == pytest.approx(achieved / peak)
    assert bench.integer_roofline(24, {"leaf_hash": {"ms_per_step": 0}}, {}) is None
