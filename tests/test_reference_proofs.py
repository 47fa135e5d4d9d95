"""Proofs written by the Rust reference itself, checked byte for byte.

The reference cannot be built in this repository's environment, so parity
with it is pinned here only when proof files made by its own harness
(crates/whir/src/test.rs:174-254, run_whir_poseidon) are present under
tests/golden/reference_proofs/.  Each file is the harness's
`transcript.finalize()` bytes for one parameter set, named

    whir_k{k}_f{folding}_r{rate}_ir{initial_reduction}_{soundness}_s{security}_n{points}_cp{checkpoint}.bin

with soundness spelled as the reference's SecurityAssumption variant and the
checkpoint as the canonical u32 of the harness's last draw.  In the harness,
after `(proof, checkpoint_prover)` is computed, one std::fs::write of
`proof` to that name (checkpoint via as_canonical_u32, soundness via its
Debug form) produces them.  For every file the oracle prover, run on
the harness's inputs (the polynomial drawn by Poly::rand from the seed-1
StdRng, n_points claims on it), must produce the same bytes and checkpoint,
and the library's verifier must accept the reference's proof.  With no
files the tests are skipped.
"""
import os
import re

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
PROOF_DIR = os.path.join(HERE, "golden", "reference_proofs")
NAME = re.compile(r"whir_k(\d+)_f(\d+)_r(\d+)_ir(\d+)_(UniqueDecoding|JohnsonBound|CapacityBound)"
                  r"_s(\d+)_n(\d+)_cp(\d+)\.bin$")
SOUNDNESS = {"UniqueDecoding": 0, "JohnsonBound": 1, "CapacityBound": 2}


def parse(name):
    m = NAME.match(name)
    if not m:
        return None
    k, f, r, ir, snd, sec, n, cp = m.groups()
    return (int(k), int(f), int(r), int(ir), SOUNDNESS[snd], int(sec)), int(n), int(cp)


def reference_files():
    if not os.path.isdir(PROOF_DIR):
        return []
    return sorted(x for x in os.listdir(PROOF_DIR) if parse(x))


def test_name_format():
    params, n, cp = parse("whir_k12_f3_r1_ir2_JohnsonBound_s32_n4_cp123456.bin")
    assert params == (12, 3, 1, 2, 1, 32) and n == 4 and cp == 123456
    assert parse("whir_k12_f3_r1_ir2_Johnson_s32_n4_cp1.bin") is None


def check_file(oracle, path):
    name = os.path.basename(path)
    params, n, cp = parse(name)
    with open(path, "rb") as f:
        want = f.read()
    k = params[0]
    poly = oracle.rand_fe(1, 1 << k)  # Poly::rand(&mut rng(1), k)
    groups = [[0]] * n
    got, got_cp = oracle.prove(params, [poly], [k], groups)
    if got != want:
        diff = next((i for i, (a, b) in enumerate(zip(got, want)) if a != b),
                    min(len(got), len(want)))
        pytest.fail(f"{name}: oracle proof differs from the reference's at byte {diff}")
    assert got_cp == cp
    import whir_gb300 as W
    assert W.verify(params, [k], groups, want) == (0, cp)


@pytest.mark.parametrize("name", reference_files() or [None])
def test_reference_proof(oracle, name):
    if name is None:
        pytest.skip("no proofs from the Rust reference under tests/golden/reference_proofs "
                    "(they need a cargo-capable machine)")
    check_file(oracle, os.path.join(PROOF_DIR, name))


def test_checker_on_an_oracle_proof(oracle, tmp_path):
    # the checker itself: a file in the reference's naming holding the
    # oracle's proof passes, and one flipped byte fails
    params = (8, 2, 1, 1, 1, 32)
    proof, cp = oracle.prove(params, [oracle.rand_fe(1, 1 << 8)], [8], [[0]] * 2)
    path = tmp_path / f"whir_k8_f2_r1_ir1_JohnsonBound_s32_n2_cp{cp}.bin"
    path.write_bytes(proof)
    check_file(oracle, str(path))
    bad = bytearray(proof)
    bad[40] ^= 1
    path.write_bytes(bytes(bad))
    with pytest.raises(pytest.fail.Exception):
        check_file(oracle, str(path))
