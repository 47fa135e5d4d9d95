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
#include <utility>

#include "kb.cuh"

namespace whir {
namespace gpu {

// [0 .. 8*W) external constants (round-major), then rounds_p internal, then W
// diag.  The round constants are stored minus p (mod 2^32): state + (c - p)
// is then the signed value state + c - p in [-p, p), which the signed S-box
// takes without a reduction.  Defined here (one translation unit includes this header: merkle.cu,
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

// Internal diagonals of p3-koala-bear's Poseidon2 as sign * num / 2^log_den
// (the same values poseidon2_host.cpp uploads for the generic path).  Every
// entry is 1, 2, 3, 4 or 2^-e up to sign, so the product needs no multiplier.
struct DiagEntry {
  int sign, num, log_den;
};
__host__ __device__ constexpr DiagEntry diag_entry16(int i) {
  constexpr DiagEntry v[16] = {{-1, 2, 0}, {1, 1, 0},  {1, 2, 0},  {1, 1, 1},
                               {1, 3, 0},  {1, 4, 0},  {-1, 1, 1}, {-1, 3, 0},
                               {-1, 4, 0}, {1, 1, 8},  {1, 1, 3},  {1, 1, 24},
                               {-1, 1, 8}, {-1, 1, 3}, {-1, 1, 4}, {-1, 1, 24}};
  return v[i];
}
__host__ __device__ constexpr DiagEntry diag_entry24(int i) {
  constexpr DiagEntry v[24] = {{-1, 2, 0}, {1, 1, 0},  {1, 2, 0},  {1, 1, 1},  {1, 3, 0},
                               {1, 4, 0},  {-1, 1, 1}, {-1, 3, 0}, {-1, 4, 0}, {1, 1, 8},
                               {1, 1, 2},  {1, 1, 3},  {1, 1, 4},  {1, 1, 5},  {1, 1, 6},
                               {1, 1, 24}, {-1, 1, 8}, {-1, 1, 3}, {-1, 1, 4}, {-1, 1, 5},
                               {-1, 1, 6}, {-1, 1, 7}, {-1, 1, 9}, {-1, 1, 24}};
  return v[i];
}

// x * num mod p for num in 1..4 on a canonical word (Montgomery form is
// linear, so scaling the word scales the element)
template <int NUM>
__device__ __forceinline__ uint32_t mul_small(uint32_t x) {
  using namespace kb;
  if constexpr (NUM == 1) {
    return x;
  } else if constexpr (NUM == 2) {
    return dbl(x);
  } else if constexpr (NUM == 3) {
    return add(dbl(x), x);
  } else {
    static_assert(NUM == 4, "diag entry");
    return dbl(dbl(x));
  }
}

// Lanes with a diagonal entry +-2^-e.
//  e < 7: x 2^-e = (x + m p) / 2^e with m = -x mod 2^e (x + m p is divisible
//         by 2^e because p = 127 * 2^24 + 1), = (x + m) / 2^e + m K with
//         K = 127 * 2^(24-e); below p for a canonical x.  Then one modular
//         add or subtract.
//  e >= 7: write x = q 2^e + lo (lo < 2^e); since 2^-e = -K (mod p),
//         x 2^-e = q - lo K with q < 2^(31-e) <= 2^24 and lo K < p, for any
//         lane word x < 2^31.
//    +2^-e: (sum + p) + q - lo K lies in [1, 2^32 - 2^24]; one conditional
//         subtraction leaves it in [0, 2^31), congruent but not always
//         canonical ("loose"; the lane sum and this same update accept such a
//         word, and the permutation reduces it after the internal rounds).
//    -2^-e: reduce(sum + lo K) - q lies in (-2^24, p); one conditional
//         addition makes it canonical.
// (On GB300 the e >= 7 forms are 2% faster over a leaf-hash launch; the same
// forms for e < 7 were slower than the ones above.)
// Entries 1, 2, 3, 4 (up to sign) are sums of canonical words.
template <int W, int I>
__device__ __forceinline__ constexpr bool p2_loose_lane() {
  constexpr DiagEntry d = W == 16 ? diag_entry16(I) : diag_entry24(I);
  return d.log_den >= 7 && d.sign > 0;
}
template <int W, int I>
__device__ __forceinline__ void p2_internal_lane(uint32_t (&s)[W], uint32_t sum, uint32_t sum_p) {
  using namespace kb;
  constexpr DiagEntry d = W == 16 ? diag_entry16(I) : diag_entry24(I);
  constexpr int E = d.log_den;
  const uint32_t x = s[I];
  if constexpr (E >= 7) {
    constexpr uint32_t MASK = (1u << E) - 1u, K = 127u << (24 - E);
    if constexpr (d.sign > 0) {
      uint32_t r = sum_p + (x >> E) - (x & MASK) * K;
      s[I] = kb::umin(r, r - P);
    } else {
      uint32_t t = sum + (x & MASK) * K;
      t = kb::umin(t, t - P);
      uint32_t r = t - (x >> E);
      s[I] = kb::umin(r, r + P);
    }
  } else if constexpr (E > 0) {
    constexpr uint32_t MASK = (1u << E) - 1u, K = 127u << (24 - E);
    uint32_t m = (0u - x) & MASK;
    uint32_t y = ((x + m) >> E) + m * K;
    s[I] = d.sign > 0 ? add(sum, y) : sub(sum, y);
  } else {
    uint32_t y = mul_small<d.num>(x);
    s[I] = d.sign > 0 ? add(sum, y) : sub(sum, y);
  }
}
template <int W, int... I>
__device__ __forceinline__ void p2_internal_all(uint32_t (&s)[W], uint32_t sum,
                                                std::integer_sequence<int, I...>) {
  const uint32_t sum_p = sum + kb::P;
  (p2_internal_lane<W, I>(s, sum, sum_p), ...);
}
// canonical form of the loose lanes, after the last internal round
template <int W, int... I>
__device__ __forceinline__ void p2_reduce_loose(uint32_t (&s)[W], std::integer_sequence<int, I...>) {
  ((p2_loose_lane<W, I>() ? (void)(s[I] = kb::umin(s[I], s[I] - kb::P)) : (void)0), ...);
}

// Signed Montgomery product of int32 words with |a * b| < p * 2^31: with t
// = a*b*p^-1 mod 2^32 read as signed, (a*b - t*p) / 2^32 lies in (-p, p).
__device__ __forceinline__ int32_t smul(int32_t a, int32_t b) {
  int64_t prod = (int64_t)a * (int64_t)b;
  int32_t t = (int32_t)kb::times_mu((uint32_t)prod);
  return (int32_t)(prod >> 32) - __mulhi(t, (int32_t)kb::P);
}
// x^3 for x in [-p, p) (a state word plus a stored constant), canonical out
__device__ __forceinline__ uint32_t sbox(int32_t x) {
  uint32_t r = (uint32_t)smul(smul(x, x), x);
  return kb::umin(r, r + kb::P);
}

template <int W>
__device__ __forceinline__ void p2_external_round(uint32_t (&s)[W], const uint32_t *rc) {
#pragma unroll
  for (int i = 0; i < W; i++) s[i] = sbox((int32_t)(s[i] + rc[i]));
  p2_mds_light<W>(s);
}

template <int W>
__device__ __forceinline__ void p2_internal_round(uint32_t (&s)[W], uint32_t rc) {
  using namespace kb;
  s[0] = sbox((int32_t)(s[0] + rc));
  // sum of the W lanes in 64 bits: every lane is below 2^31 (canonical or
  // loose), so pairs add without overflow in 32 bits; then one reduction: 2^31 = 2^24 - 1 (mod p) folds the high
  // part, leaving < 2p
  uint64_t wide = 0;
  if constexpr (W == 24) {
    // a pair and a lane per step, lanes 1..23 first and the S-box lane last:
    // the same instruction count as pairs, and on GB300 1.5% more width-24
    // permutations/s on 16-word leaf rows, 0.4% on 64-word rows (at width 16
    // the pairs below are fastest)
    int i = 1;
#pragma unroll
    for (; i + 2 < W; i += 3) wide = wide + (uint64_t)(uint32_t)(s[i] + s[i + 1]) + (uint64_t)s[i + 2];
#pragma unroll
    for (; i < W; i++) wide += s[i];  // lanes 22 and 23
    wide += s[0];
  } else {
#pragma unroll
    for (int i = 0; i < W; i += 2) wide += (uint32_t)(s[i] + s[i + 1]);
  }
  uint32_t folded = (uint32_t)(wide & 0x7fffffffu) + (uint32_t)(wide >> 31) * 0x00ffffffu;
  uint32_t sum = kb::umin(folded, folded - P);
  p2_internal_all<W>(s, sum, std::make_integer_sequence<int, W>{});
}

// The round loops stay rolled on purpose: fully unrolled, one permutation is
// several thousand instructions, more than the SM's instruction cache holds,
// and the kernels then stall on instruction fetch (measured on GB300: rolled
// loops permute 24-wide states 1.28x and 16-wide 1.24x faster).
template <int W>
__device__ __forceinline__ void p2_permute(uint32_t (&s)[W]) {
  const uint32_t *C = p2_consts<W>();
  constexpr int RP = P2Shape<W>::RP;
  const uint32_t *I = C + 8 * W;
  p2_mds_light<W>(s);
#pragma unroll 1
  for (int r = 0; r < 8; r++) {
    if (r == 4) {
      // two internal rounds per loop trip (measured: 1.7% more width-24
      // permutations/s than one; the loop stays small enough for the
      // instruction cache)
      int q = 0;
#pragma unroll 1
      for (; q + 1 < RP; q += 2) {
        p2_internal_round<W>(s, I[q]);
        p2_internal_round<W>(s, I[q + 1]);
      }
      if constexpr (RP % 2 == 1) p2_internal_round<W>(s, I[q]);
      p2_reduce_loose<W>(s, std::make_integer_sequence<int, W>{});
    }
    p2_external_round<W>(s, C + r * W);
  }
}

}  // namespace gpu
}  // namespace whir
