// Poseidon2 permutation on the device: one permutation per thread, the state
// in registers, round constants and internal diagonals in constant memory
// (every thread of a warp reads the same constant, which the constant cache
// broadcasts), Montgomery products on the 32-bit IMAD pipe.
//
// Permutation shape (p3-poseidon2, as used by the reference's
// PaddingFreeSponge<Poseidon2KoalaBear<24>> leaf hash and
// TruncatedPermutation<Poseidon2KoalaBear<16>> node compression,
// crates/whir/src/test.rs:188-189): light MDS, 4 external rounds, rounds_p
// internal rounds (S-box on lane 0, then 1 1^T + diag), 4 external rounds.
#pragma once
#include "kb.cuh"

namespace whir {
namespace gpu {

// [0 .. 8*W) external constants (round-major), then rounds_p internal, then W
// diag.  Defined here (one translation unit includes this header: merkle.cu,
// which also uploads them).
__constant__ uint32_t c_p2_16[8 * 16 + 20 + 16];
__constant__ uint32_t c_p2_24[8 * 24 + 23 + 24];

template <int W>
struct P2Shape;
template <>
struct P2Shape<16> {
  static constexpr int RP = 20;
};
template <>
struct P2Shape<24> {
  static constexpr int RP = 23;
};

template <int W>
__device__ __forceinline__ const uint32_t *p2_consts() {
  if constexpr (W == 16) return c_p2_16;
  else return c_p2_24;
}

__device__ __forceinline__ void p2_mat4(uint32_t &x0, uint32_t &x1, uint32_t &x2, uint32_t &x3) {
  using namespace kb;
  uint32_t t01 = add(x0, x1), t23 = add(x2, x3);
  uint32_t t0123 = add(t01, t23);
  uint32_t t01123 = add(t0123, x1), t01233 = add(t0123, x3);
  uint32_t y3 = add(t01233, dbl(x0));
  uint32_t y1 = add(t01123, dbl(x2));
  uint32_t y0 = add(t01123, t01);
  uint32_t y2 = add(t01233, t23);
  x0 = y0; x1 = y1; x2 = y2; x3 = y3;
}

template <int W>
__device__ __forceinline__ void p2_mds_light(uint32_t (&s)[W]) {
#pragma unroll
  for (int i = 0; i < W; i += 4) p2_mat4(s[i], s[i + 1], s[i + 2], s[i + 3]);
  uint32_t sum[4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    uint32_t a = s[c];
#pragma unroll
    for (int i = c + 4; i < W; i += 4) a = kb::add(a, s[i]);
    sum[c] = a;
  }
#pragma unroll
  for (int i = 0; i < W; i++) s[i] = kb::add(s[i], sum[i & 3]);
}

template <int W>
__device__ __forceinline__ void p2_permute(uint32_t (&s)[W]) {
  using namespace kb;
  const uint32_t *C = p2_consts<W>();
  constexpr int RP = P2Shape<W>::RP;
  const uint32_t *I = C + 8 * W;
  const uint32_t *D = C + 8 * W + RP;
  p2_mds_light<W>(s);
#pragma unroll
  for (int r = 0; r < 4; r++) {
#pragma unroll
    for (int i = 0; i < W; i++) s[i] = cube(add(s[i], C[r * W + i]));
    p2_mds_light<W>(s);
  }
#pragma unroll
  for (int r = 0; r < RP; r++) {
    s[0] = cube(add(s[0], I[r]));
    uint32_t sum = s[0];
#pragma unroll
    for (int i = 1; i < W; i++) sum = add(sum, s[i]);
#pragma unroll
    for (int i = 0; i < W; i++) s[i] = add(sum, mul(D[i], s[i]));
  }
#pragma unroll
  for (int r = 4; r < 8; r++) {
#pragma unroll
    for (int i = 0; i < W; i++) s[i] = cube(add(s[i], C[r * W + i]));
    p2_mds_light<W>(s);
  }
}

}  // namespace gpu
}  // namespace whir
