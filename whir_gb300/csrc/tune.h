// Per-size scheduling choices of the Merkle tree build and the two-pass DFT,
// picked by timing the candidates on the device (gpu::TreeTune, gpu::DftTune
// in kernels.h).  Outputs never depend on the choice, only the time does.
#pragma once
#include <string>

#include "prover.h"

namespace whir {

// Times every valid candidate for tree heights and DFT sizes in
// [log_h_lo, log_h_hi] on ctx's stream, installs the fastest for each size
// (process-wide) and returns a text report, one line per size.
std::string autotune(Context &ctx, int log_h_lo, int log_h_hi);
void tune_reset();

}  // namespace whir
