// WHIR verifier on the host: Whir::verify (crates/whir/src/whir.rs:361-522)
// with SumcheckVerifier (crates/whir/src/sumcheck/verifier.rs), over the same
// transcript (PoseidonWriter reading side) and Merkle hashing as the prover.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "prover.h"

namespace whir {

// Why a proof was rejected (0: accepted).
enum VerifyResult {
  V_OK = 0,
  V_TRANSCRIPT = 1,  // proof bytes ran out or held a non-canonical word
  V_MERKLE = 2,      // an opening did not hash to its commitment
  V_STIR = 3,        // a final-round opening disagrees with the final polynomial
  V_SUMCHECK = 4,    // the sumcheck's final claim does not match
  V_SHAPE = 5,       // the proof's round structure does not match the parameters
};

// Checks a proof made by Prover::prove with the same parameters, polynomial
// sizes and claim groups.  On acceptance *checkpoint is the base element the
// harness draws after the proof (test.rs:236).  Argument errors throw.
VerifyResult verify(const Params &p, const std::vector<int> &poly_k,
                    const std::vector<std::vector<int>> &groups, const uint8_t *proof, size_t len,
                    uint32_t *checkpoint);

// The path check of MerkleTree::verify (crates/merkle/src/poseidon_packed.rs:235-257,
// poseidon.rs:22-41) over words already read: the opened row (row_len words)
// hashed as a leaf, then log_h sibling digests bottom-up, must give root.
bool merkle_path_ok(const uint32_t root[8], size_t index, const uint32_t *row, size_t row_len,
                    const uint32_t *siblings, int log_h);

}  // namespace whir
