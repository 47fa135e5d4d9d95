// DuplexChallenger and transcript (see transcript.h).
#include "transcript.h"

#include <string.h>

#include "poseidon2_host.h"

namespace whir {

Challenger::Challenger() {
  memset(state_, 0, sizeof state_);
  memset(out_, 0, sizeof out_);
  memset(in_, 0, sizeof in_);
}

// overwrite the first n_in rate lanes with the pending inputs, permute, and
// expose the 8 rate lanes as outputs (sampled from the back)
void Challenger::duplexing() {
  for (int i = 0; i < n_in_; i++) state_[i] = in_[i];
  n_in_ = 0;
  poseidon2_permute_host(poseidon2_constants(16), state_);
  for (int i = 0; i < 8; i++) out_[i] = state_[i];
  n_out_ = 8;
}

void Challenger::observe(uint32_t v) {
  n_out_ = 0;  // buffered outputs no longer reflect the transcript
  in_[n_in_++] = v;
  if (n_in_ == 8) duplexing();
}

uint32_t Challenger::sample() {
  if (n_in_ > 0 || n_out_ == 0) duplexing();
  return out_[--n_out_];
}

size_t Challenger::sample_bits(int bits) {
  uint32_t v = kb::to_canonical(sample());
  return (size_t)v & (((size_t)1 << bits) - 1);
}

void Transcript::hint_words(const uint32_t *v, size_t n) { hint_fill(hint_reserve(n), v, n); }

void Transcript::hint_fill(size_t off, const uint32_t *v, size_t n) {
  uint8_t *d = bytes_.data() + off;
  for (size_t i = 0; i < n; i++) {
    d[4 * i] = (uint8_t)v[i];
    d[4 * i + 1] = (uint8_t)(v[i] >> 8);
    d[4 * i + 2] = (uint8_t)(v[i] >> 16);
    d[4 * i + 3] = (uint8_t)(v[i] >> 24);
  }
}

}  // namespace whir
