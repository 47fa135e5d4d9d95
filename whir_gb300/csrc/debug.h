// Debug mode of the provers, off by default (whir_debug_set): the
// reference's debug-build invariants checked on the device's results, NVTX
// ranges named like the reference's tracing spans so that a profiler
// timeline lines up with them, and the verifier's inline path order.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace whir {

enum DebugFlags : unsigned {
  // after every sumcheck round and expression build: <poly, weights> equals
  // the running claimed sum (crates/whir/src/sumcheck/prover.rs:346,558,
  // expr.rs:68); every opened Merkle path hashes to its root
  // (crates/merkle/src/poseidon_packed.rs:158-230); every opened row folded at
  // the round point equals the polynomial at its domain point
  // (crates/whir/src/whir.rs:263-264, 287-288, 331-352); each out-of-domain
  // claim equals the claim made on the stacked polynomial
  // (crates/whir/src/sumcheck/prover.rs:257-266)
  DEBUG_CHECKS = 1u,
  // NVTX ranges around the prover's phases (crates/whir/src/whir.rs:19-314,
  // crates/whir/src/sumcheck/prover.rs:184-497)
  DEBUG_NVTX = 2u,
  // whir_verify hashes each Merkle opening where it reads it (the order of
  // Whir::verify, crates/whir/src/whir.rs:361-522) instead of after the
  // transcript pass (the order whir_verify_batch uses); the same results
  DEBUG_VERIFY_INLINE = 4u,
};
void set_debug(unsigned flags);
unsigned debug_flags();
inline bool debug_checks() { return (debug_flags() & DEBUG_CHECKS) != 0; }

// an NVTX range for the lifetime of the object while DEBUG_NVTX is set
class Span {
 public:
  explicit Span(const char *name) : on_((debug_flags() & DEBUG_NVTX) != 0) {
    if (on_) nvtxRangePushA(name);
  }
  ~Span() {
    if (on_) nvtxRangePop();
  }
  Span(const Span &) = delete;
  Span &operator=(const Span &) = delete;

 private:
  bool on_;
};

}  // namespace whir
