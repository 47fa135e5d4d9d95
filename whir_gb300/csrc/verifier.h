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

// The Merkle openings of one proof, read but not hashed.  The openings are
// hints (never observed by the challenger), so nothing the transcript draws
// depends on whether they hash to their roots: a verifier can read a whole
// proof, do every other check, and hash the paths afterwards in one batch.
// An opening's words are contiguous in the proof: the row (row_len words,
// hashed as a leaf), then log_h sibling digests bottom-up; `word` is the
// index of its first word in the proof (byte offset / 4).
struct PathCheck {
  size_t word;
  uint64_t index;
  int log_h;
  int row_len;
  uint32_t root[8];
};
struct DeferredPaths {
  std::vector<PathCheck> checks;  // in the order the verifier meets them
};
// the checks' outcomes on the host (1: the path climbs to its root)
std::vector<uint8_t> deferred_paths_ok(const uint8_t *proof, size_t len, const DeferredPaths &d);

// Checks a proof made by Prover::prove with the same parameters, polynomial
// sizes and claim groups.  On acceptance *checkpoint is the base element the
// harness draws after the proof (test.rs:236).  Argument errors throw.
// With defer != nullptr the Merkle paths are recorded instead of hashed
// (they are taken as good); the result is then the first failure of the
// other checks, and every path recorded precedes it.  The sequential result
// is verify_resolve of that and the paths' outcomes.
VerifyResult verify(const Params &p, const std::vector<int> &poly_k,
                    const std::vector<std::vector<int>> &groups, const uint8_t *proof, size_t len,
                    uint32_t *checkpoint, DeferredPaths *defer = nullptr);
// The result verify() gives without deferral: a failed path comes before
// any failure found with the paths deferred (path_ok: one flag per check).
VerifyResult verify_resolve(VerifyResult deferred, const DeferredPaths &d, const uint8_t *path_ok);

// The path check of MerkleTree::verify (crates/merkle/src/poseidon_packed.rs:235-257,
// poseidon.rs:22-41) over words already read: the opened row (row_len words)
// hashed as a leaf, then log_h sibling digests bottom-up, must give root.
bool merkle_path_ok(const uint32_t root[8], size_t index, const uint32_t *row, size_t row_len,
                    const uint32_t *siblings, int log_h);

}  // namespace whir
