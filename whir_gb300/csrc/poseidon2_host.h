// Poseidon2 over KoalaBear on the host: constant generation for both widths
// and the width-16 permutation the Fiat-Shamir challenger runs.
//
// Restates Poseidon2KoalaBear<16|24>::new_from_rng_128(&mut rng(1000)) as used
// by the reference harness (crates/whir/src/test.rs:195-196): StdRng seeded by
// SeedableRng::seed_from_u64 (PCG32 expansion into a ChaCha12 key), KoalaBear
// drawn as next_u32() >> 1 with rejection at p, external constants for the 4
// initial then 4 terminal rounds, then one constant per partial round.
#pragma once
#include <stdint.h>

namespace whir {

struct Poseidon2Constants {
  int width;
  int rounds_p;
  uint32_t ext_rc[8][24];  // [round][lane], rounds 0..3 initial, 4..7 terminal
  uint32_t int_rc[24];
  uint32_t diag[24];       // internal matrix 1 1^T + diag(diag), Montgomery form
};

// Constants for width 16 or 24 (computed once, thread-safe).
const Poseidon2Constants &poseidon2_constants(int width);

// In-place permutation on the host (Montgomery-form words).
void poseidon2_permute_host(const Poseidon2Constants &c, uint32_t *state);

// rand_core seed_from_u64 + ChaCha12: the field elements Poly::rand draws.
void std_rng_fill_field(uint64_t seed, uint32_t *out, uint64_t n);

}  // namespace whir
