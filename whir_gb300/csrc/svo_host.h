// Host side of the small-value-optimised (SVO) claims and rounds, shared by
// the single-instance and the batched prover (crates/whir/src/sumcheck/svo.rs,
// crates/whir/src/sumcheck/prover.rs:64-90,232-354).  The heavy part of a
// claim, compress_hi over the whole polynomial, runs on the device; what
// follows here is 3^r-sized.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "kb.cuh"
#include "transcript.h"

namespace whir {

struct SvoClaim {
  int poly = 0;
  int k = 0;
  std::vector<kb::E4> point;
  std::vector<kb::E4> compressed;  // 2^ks
  std::vector<kb::E4> partial;     // l = 1..ks, 2^l each, concatenated
  kb::E4 eval;
};
inline size_t partial_off(int l) { return ((size_t)1 << l) - 2; }

struct VirtClaim {
  std::vector<kb::E4> point;
  kb::E4 eval;
  std::vector<kb::E4> acc;
};

size_t ipow3(int r);
// a field element from 4 unreduced 64-bit sums of canonical words
kb::E4 reduce_acc(const unsigned long long *a);
// SVO accumulators over ks rounds: sum_r 2 3^r
size_t svo_acc_size(int ks);

// SvoPoint::new + eval (svo.rs:64-91) after the device pass: c.point (c.k
// coordinates) is set and sums holds compress_hi's 4 * 2^ks unreduced sums;
// fills c.compressed, c.eval and the partial evals (svo_partial_evals,
// svo.rs:18-38).
void svo_finish(SvoClaim &c, int ks, const unsigned long long *sums);

// Svo::calculate_accumulators (svo.rs:225-278) with the base-field eq tables
// of the {0,1,2} grid built once (Svo::new, svo.rs:158-222).
class SvoTables {
 public:
  // tables for rounds 0..ks-1 (kept; a larger ks only adds rounds)
  void build(int ks);
  // accv += the accumulators of claim c weighted by w
  void accumulate(std::vector<kb::E4> &accv, const SvoClaim &c, const kb::E4 &w, int ks);

 private:
  std::vector<std::vector<uint32_t>> eq_;
};

// The SVO rounds of ProverLayout::new_prover (prover.rs:309-343): per round
// (c0, c2) from the accumulators and the Lagrange weights of the challenges
// so far, written to the transcript; draws r, extrapolates sum, appends r.
void svo_rounds(Transcript &ts, const std::vector<kb::E4> &accv, int ks, kb::E4 &sum,
                std::vector<kb::E4> &rs);

}  // namespace whir
