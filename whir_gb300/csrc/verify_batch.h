// Many proofs of one shape verified together (no counterpart in the
// reference, whose Whir::verify checks one proof, crates/whir/src/whir.rs:
// 361-522).  Each proof's transcript pass runs on a pool of host threads with
// its Merkle paths deferred (verifier.h: the openings are hints, so no draw
// depends on them); then the proofs are copied to the device once and every
// path of every proof is hashed in one launch (kernels.h, verify_paths).  A
// proof's result is the first failure in the order verify() meets them, so
// results and checkpoints equal verify()'s on each proof alone.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "batch_prover.h"
#include "verifier.h"

namespace whir {

class BatchVerifier {
 public:
  BatchVerifier(Context *ctx, int host_threads);
  // results[b] (VerifyResult) and checkpoints[b] (0 unless accepted) for
  // proofs[b] of lens[b] bytes, b < n.  Argument errors throw.
  void verify(const Params &p, const std::vector<int> &poly_k,
              const std::vector<std::vector<int>> &groups, int n, const uint8_t *const *proofs,
              const size_t *lens, int32_t *results, uint32_t *checkpoints);
  // paths hashed by the last call
  size_t last_paths() const { return last_paths_; }

 private:
  Context *ctx_;
  HostPool pool_;
  DeviceBuffer dev_;
  PinnedBuffer stage_;
  size_t last_paths_ = 0;
};

}  // namespace whir
