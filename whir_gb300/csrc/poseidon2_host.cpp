// Host Poseidon2 constants and permutation (see poseidon2_host.h).
#include "poseidon2_host.h"

#include <mutex>
#include <utility>

#include "kb.cuh"

namespace whir {
namespace {

// ChaCha with the original 64-bit block counter (words 12-13) and a zero
// stream id (words 14-15): the block function behind rand's StdRng.
struct ChaCha12 {
  uint32_t key[8];
  uint64_t counter = 0;
  uint32_t buf[16];
  int idx = 16;

  static uint32_t rotl(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }
  static void quarter(uint32_t &a, uint32_t &b, uint32_t &c, uint32_t &d) {
    a += b; d ^= a; d = rotl(d, 16);
    c += d; b ^= c; b = rotl(b, 12);
    a += b; d ^= a; d = rotl(d, 8);
    c += d; b ^= c; b = rotl(b, 7);
  }
  void refill() {
    uint32_t s[16] = {0x61707865, 0x3320646e, 0x79622d32, 0x6b206574};
    for (int i = 0; i < 8; i++) s[4 + i] = key[i];
    s[12] = (uint32_t)counter;
    s[13] = (uint32_t)(counter >> 32);
    s[14] = 0;
    s[15] = 0;
    uint32_t x[16];
    for (int i = 0; i < 16; i++) x[i] = s[i];
    for (int r = 0; r < 12; r += 2) {
      quarter(x[0], x[4], x[8], x[12]);
      quarter(x[1], x[5], x[9], x[13]);
      quarter(x[2], x[6], x[10], x[14]);
      quarter(x[3], x[7], x[11], x[15]);
      quarter(x[0], x[5], x[10], x[15]);
      quarter(x[1], x[6], x[11], x[12]);
      quarter(x[2], x[7], x[8], x[13]);
      quarter(x[3], x[4], x[9], x[14]);
    }
    for (int i = 0; i < 16; i++) buf[i] = x[i] + s[i];
    counter++;
    idx = 0;
  }
  explicit ChaCha12(uint64_t seed) {
    // rand_core: PCG32 output words fill the 32-byte seed little-endian.
    const uint64_t mul = 6364136223846793005ull, inc = 11634580027462260723ull;
    for (int i = 0; i < 8; i++) {
      seed = seed * mul + inc;
      uint32_t xs = (uint32_t)(((seed >> 18) ^ seed) >> 27);
      uint32_t rot = (uint32_t)(seed >> 59);
      key[i] = (xs >> rot) | (xs << ((32 - rot) & 31));
    }
  }
  uint32_t next_u32() {
    if (idx == 16) refill();
    return buf[idx++];
  }
  // StandardUniform<MontyField31>: 31 random bits, rejected at p, kept as the
  // Montgomery word.
  uint32_t next_field() {
    for (;;) {
      uint32_t v = next_u32() >> 1;
      if (v < kb::P) return v;
    }
  }
};

// Internal diagonals of p3-koala-bear's Poseidon2 (V in M_I = 1 1^T + diag(V)),
// entry i = sign * num / 2^log_den.
constexpr int v16[16][3] = {{-1, 2, 0}, {1, 1, 0},  {1, 2, 0},  {1, 1, 1},
                            {1, 3, 0},  {1, 4, 0},  {-1, 1, 1}, {-1, 3, 0},
                            {-1, 4, 0}, {1, 1, 8},  {1, 1, 3},  {1, 1, 24},
                            {-1, 1, 8}, {-1, 1, 3}, {-1, 1, 4}, {-1, 1, 24}};
constexpr int v24[24][3] = {{-1, 2, 0}, {1, 1, 0},  {1, 2, 0},  {1, 1, 1},  {1, 3, 0},
                            {1, 4, 0},  {-1, 1, 1}, {-1, 3, 0}, {-1, 4, 0}, {1, 1, 8},
                            {1, 1, 2},  {1, 1, 3},  {1, 1, 4},  {1, 1, 5},  {1, 1, 6},
                            {1, 1, 24}, {-1, 1, 8}, {-1, 1, 3}, {-1, 1, 4}, {-1, 1, 5},
                            {-1, 1, 6}, {-1, 1, 7}, {-1, 1, 9}, {-1, 1, 24}};

// diag entry sign * num / 2^log_den
uint32_t diag_value(int sign, uint32_t num, int log_den) {
  uint32_t v = kb::mul(kb::from_canonical(num), kb::inv(kb::pow(kb::from_canonical(2), log_den)));
  return sign < 0 ? kb::neg(v) : v;
}

void build(Poseidon2Constants &c, int width) {
  c.width = width;
  c.rounds_p = width == 16 ? 20 : 23;  // poseidon2_round_numbers_128 for 31-bit p, D = 3
  for (int i = 0; i < width; i++) {
    const int *v = width == 16 ? v16[i] : v24[i];
    c.diag[i] = diag_value(v[0], (uint32_t)v[1], v[2]);
  }
  ChaCha12 rng(1000);
  for (int r = 0; r < 8; r++)
    for (int i = 0; i < width; i++) c.ext_rc[r][i] = rng.next_field();
  for (int r = 0; r < c.rounds_p; r++) c.int_rc[r] = rng.next_field();
}

// x mod p for x < 2^38: 2^31 = 2^24 - 1 (mod p) folds the bits above 31,
// leaving a value below 2^32 < 3p, then two conditional subtractions.
inline uint32_t reduce38(uint64_t x) {
  uint64_t y = (x & 0x7fffffffu) + (x >> 31) * 0x00ffffffull;
  y = y >= 2ull * kb::P ? y - 2ull * kb::P : y;
  return (uint32_t)(y >= kb::P ? y - kb::P : y);
}

// The linear layers in 64-bit lanes with one reduction per output word.
inline void mat4_wide(uint64_t *x) {
  uint64_t t01 = x[0] + x[1], t23 = x[2] + x[3];
  uint64_t t0123 = t01 + t23;
  uint64_t t01123 = t0123 + x[1], t01233 = t0123 + x[3];
  uint64_t y3 = t01233 + 2 * x[0];
  uint64_t y1 = t01123 + 2 * x[2];
  uint64_t y0 = t01123 + t01;
  uint64_t y2 = t01233 + t23;
  x[0] = y0; x[1] = y1; x[2] = y2; x[3] = y3;
}
// light MDS of canonical words: every output below 49 p < 2^38 before its
// reduction
template <int W>
inline void mds_light(uint32_t *s) {
  uint64_t x[W];
  for (int i = 0; i < W; i++) x[i] = s[i];
  for (int i = 0; i < W; i += 4) mat4_wide(x + i);
  uint64_t sums[4] = {0, 0, 0, 0};
  for (int i = 0; i < W; i++) sums[i & 3] += x[i];
  for (int i = 0; i < W; i++) s[i] = reduce38(x[i] + sums[i & 3]);
}
// s_i <- sum + d_i s_i with the diagonal's small entries (Montgomery form is
// linear, so scaling the word scales the element): num in 1..4 as a multiple
// of x or of p - x; 2^-e as (x + m p) / 2^e with m = -x mod 2^e (exact, since
// p = 1 mod 2^24), below 2p; every lane below 2^38 before one reduction.
// Each lane's form is fixed at compile time.
template <int W, int I>
inline void internal_lane(uint32_t *s, uint64_t sum) {
  constexpr int sign = W == 16 ? v16[I][0] : v24[I][0];
  constexpr int num = W == 16 ? v16[I][1] : v24[I][1];
  constexpr int e = W == 16 ? v16[I][2] : v24[I][2];
  const uint64_t x = s[I];
  uint64_t t;
  if constexpr (e == 0) {
    t = sign > 0 ? (uint64_t)num * x : (uint64_t)num * (kb::P - x);
  } else {
    const uint64_t m = (0 - x) & ((1ull << e) - 1);
    const uint64_t y = (x + m * kb::P) >> e;  // < 2p
    t = sign > 0 ? y : 2ull * kb::P - y;
  }
  s[I] = reduce38(sum + t);
}
template <int W, int... I>
inline void internal_lanes(uint32_t *s, uint64_t sum, std::integer_sequence<int, I...>) {
  (internal_lane<W, I>(s, sum), ...);
}
template <int W>
inline void internal_layer(uint32_t *s) {
  uint64_t total = 0;
  for (int i = 0; i < W; i++) total += s[i];
  internal_lanes<W>(s, reduce38(total), std::make_integer_sequence<int, W>{});
}

template <int W>
void permute_w(const Poseidon2Constants &c, uint32_t *s) {
  using namespace kb;
  mds_light<W>(s);
  for (int r = 0; r < 4; r++) {
    for (int i = 0; i < W; i++) s[i] = cube(add(s[i], c.ext_rc[r][i]));
    mds_light<W>(s);
  }
  for (int r = 0; r < c.rounds_p; r++) {
    s[0] = cube(add(s[0], c.int_rc[r]));
    internal_layer<W>(s);
  }
  for (int r = 4; r < 8; r++) {
    for (int i = 0; i < W; i++) s[i] = cube(add(s[i], c.ext_rc[r][i]));
    mds_light<W>(s);
  }
}

}  // namespace

const Poseidon2Constants &poseidon2_constants(int width) {
  static Poseidon2Constants c16, c24;
  static std::once_flag once;
  std::call_once(once, [] {
    build(c16, 16);
    build(c24, 24);
  });
  return width == 16 ? c16 : c24;
}

void poseidon2_permute_host(const Poseidon2Constants &c, uint32_t *s) {
  if (c.width == 16) permute_w<16>(c, s);
  else permute_w<24>(c, s);
}

void std_rng_fill_field(uint64_t seed, uint32_t *out, uint64_t n) {
  ChaCha12 rng(seed);
  for (uint64_t i = 0; i < n; i++) out[i] = rng.next_field();
}

}  // namespace whir
