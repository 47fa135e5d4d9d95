// KoalaBear field (p = 2^31 - 2^24 + 1) in Montgomery form and its quartic
// extension F[x]/(x^4 - 3), usable from host and device code.
//
// Representation matches Plonky3's MontyField31 (the field behind
// crates/common/src/field.rs): a u32 holding x * 2^32 mod p, always canonical
// (< p) at every kernel boundary.  An extension element is 4 such words, the
// coefficients of 1, x, x^2, x^3.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define KB_HD __host__ __device__ __forceinline__
#else
#define KB_HD inline
#endif

namespace kb {

constexpr uint32_t P = 0x7f000001u;
constexpr uint32_t MU = 0x81000001u;   // p^-1 mod 2^32
constexpr uint32_t R2 = 0x17f7efe4u;   // 2^64 mod p
constexpr uint32_t ONE = 0x01fffffeu;  // 2^32 mod p
constexpr uint32_t THREE = 0x05fffffau;  // Montgomery form of 3 (the extension's W)

KB_HD uint32_t mulhi(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}
KB_HD uint32_t umin(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return ::min(a, b);
#else
  return a < b ? a : b;
#endif
}

// t = lo * p^-1 mod 2^32 as one low multiply.  MU = 2^31 + 2^24 + 1 also
// allows two shifted adds, but on GB300 the multiply is faster in the
// Poseidon2 S-box (3.44 -> 3.62 G width-24 permutations/s) and in chains of
// Montgomery products (+5.6%); a 64-bit wide multiply costs more than a low
// and a high one, and splitting a*b into those two costs more than the wide
// one (all measured).
KB_HD uint32_t times_mu(uint32_t lo) { return lo * MU; }

// Montgomery product: (a*b - t*p) / 2^32 with t = a*b*p^-1 mod 2^32.
// Valid for a < 2^32 and b < p (the product is below p * 2^32).
KB_HD uint32_t mul(uint32_t a, uint32_t b) {
  uint64_t prod = (uint64_t)a * b;
  uint32_t lo = (uint32_t)prod, hi = (uint32_t)(prod >> 32);
  uint32_t th = mulhi(times_mu(lo), P);
  uint32_t r = hi - th;  // in (-p, p); as u32, r + p is the smaller one iff r < 0
  return umin(r, r + P);
}
// reduction of a 64-bit sum x < 2p * 2^32 (e.g. four products of canonical words)
KB_HD uint32_t reduce_wide(uint64_t x) {
  uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
  uint32_t th = mulhi(times_mu(lo), P);
  uint32_t r = hi - th;  // in (-p, 2p)
  if (hi < th) return r + P;
  return umin(r, r - P);
}
// a + b and a - b of canonical words: one add and an unsigned min (measured
// on GB300 to be the fastest reduction of the alternatives tried).
KB_HD uint32_t add(uint32_t a, uint32_t b) {
  uint32_t r = a + b;
  return umin(r, r - P);
}
KB_HD uint32_t sub(uint32_t a, uint32_t b) {
  uint32_t r = a - b;
  return umin(r, r + P);
}
KB_HD uint32_t neg(uint32_t a) { return a ? P - a : 0; }
KB_HD uint32_t dbl(uint32_t a) { return add(a, a); }
KB_HD uint32_t from_canonical(uint32_t x) { return mul(x % P, R2); }
KB_HD uint32_t to_canonical(uint32_t a) { return mul(a, 1u); }
KB_HD uint32_t cube(uint32_t x) { return mul(mul(x, x), x); }
KB_HD uint32_t pow(uint32_t a, uint64_t e) {
  uint32_t r = ONE;
  while (e) {
    if (e & 1) r = mul(r, a);
    a = mul(a, a);
    e >>= 1;
  }
  return r;
}
KB_HD uint32_t inv(uint32_t a) { return pow(a, P - 2); }

struct E4 {
  uint32_t c[4];
};

KB_HD E4 e_zero() { return E4{{0, 0, 0, 0}}; }
KB_HD E4 e_one() { return E4{{ONE, 0, 0, 0}}; }
KB_HD E4 e_from(uint32_t a) { return E4{{a, 0, 0, 0}}; }
KB_HD E4 e_add(const E4 &a, const E4 &b) {
  return E4{{add(a.c[0], b.c[0]), add(a.c[1], b.c[1]), add(a.c[2], b.c[2]), add(a.c[3], b.c[3])}};
}
KB_HD E4 e_sub(const E4 &a, const E4 &b) {
  return E4{{sub(a.c[0], b.c[0]), sub(a.c[1], b.c[1]), sub(a.c[2], b.c[2]), sub(a.c[3], b.c[3])}};
}
KB_HD E4 e_neg(const E4 &a) { return E4{{neg(a.c[0]), neg(a.c[1]), neg(a.c[2]), neg(a.c[3])}}; }
KB_HD E4 e_dbl(const E4 &a) { return e_add(a, a); }
KB_HD E4 e_scale(const E4 &a, uint32_t s) {
  return E4{{mul(a.c[0], s), mul(a.c[1], s), mul(a.c[2], s), mul(a.c[3], s)}};
}
KB_HD uint32_t triple(uint32_t a) { return add(dbl(a), a); }
// (a0 + a1 x + a2 x^2 + a3 x^3)(b0 + ...) mod x^4 - 3, each output coefficient
// one 64-bit sum of four products and a single wide reduction.
KB_HD E4 e_mul(const E4 &a, const E4 &b) {
  uint32_t b1 = triple(b.c[1]), b2 = triple(b.c[2]), b3 = triple(b.c[3]);
  uint64_t s0 = (uint64_t)a.c[0] * b.c[0] + (uint64_t)a.c[1] * b3 + (uint64_t)a.c[2] * b2 +
                (uint64_t)a.c[3] * b1;
  uint64_t s1 = (uint64_t)a.c[0] * b.c[1] + (uint64_t)a.c[1] * b.c[0] + (uint64_t)a.c[2] * b3 +
                (uint64_t)a.c[3] * b2;
  uint64_t s2 = (uint64_t)a.c[0] * b.c[2] + (uint64_t)a.c[1] * b.c[1] + (uint64_t)a.c[2] * b.c[0] +
                (uint64_t)a.c[3] * b3;
  uint64_t s3 = (uint64_t)a.c[0] * b.c[3] + (uint64_t)a.c[1] * b.c[2] + (uint64_t)a.c[2] * b.c[1] +
                (uint64_t)a.c[3] * b.c[0];
  return E4{{reduce_wide(s0), reduce_wide(s1), reduce_wide(s2), reduce_wide(s3)}};
}
KB_HD E4 e_sq(const E4 &a) { return e_mul(a, a); }
KB_HD bool e_eq(const E4 &a, const E4 &b) {
  return a.c[0] == b.c[0] && a.c[1] == b.c[1] && a.c[2] == b.c[2] && a.c[3] == b.c[3];
}
KB_HD E4 e_pow(E4 a, uint64_t e) {
  E4 r = e_one();
  while (e) {
    if (e & 1) r = e_mul(r, a);
    a = e_mul(a, a);
    e >>= 1;
  }
  return r;
}

}  // namespace kb
