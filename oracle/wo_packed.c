/* Lane-packed Poseidon2 for the timed CPU baseline -- test infrastructure.
 *
 * The reference hashes its Merkle leaves and nodes with Plonky3's packed
 * Poseidon2 (crates/merkle/src/poseidon_packed.rs:98-143, 269-304: one SIMD
 * lane per state, all lanes through the same rounds).  This restates that
 * shape in plain C: WO_LANES states in structure-of-arrays form
 * (s[word][lane]), every operation a loop over the lanes that the compiler
 * turns into vector instructions (NEON on Grace, SSE/AVX on x86).  The
 * arithmetic is the scalar permutation's (wo_field.c), lane by lane, so the
 * results are identical; tests/test_oracle_packed.py checks that.  Only the
 * timed baseline switches it on (wo_set_packed); the scalar code stays the
 * parity checker.
 */
#include <stdlib.h>
#include <string.h>

#include "wo_internal.h"
#include "whir_oracle.h"

#define L WO_LANES

static int g_packed;
void wo_set_packed(int on) { g_packed = on != 0; }
int wo_packed(void) { return g_packed; }

typedef fe lanes[L];

static inline void v_add(lanes r, const lanes a, const lanes b) {
  for (int j = 0; j < L; j++) {
    uint32_t t = a[j] + b[j];
    r[j] = t >= WO_P ? t - WO_P : t;
  }
}
static inline void v_add_c(lanes r, const lanes a, fe c) {
  for (int j = 0; j < L; j++) {
    uint32_t t = a[j] + c;
    r[j] = t >= WO_P ? t - WO_P : t;
  }
}
/* Montgomery product, lane by lane (fe_reduce of wo_internal.h) */
static inline void v_mul(lanes r, const lanes a, const lanes b) {
  for (int j = 0; j < L; j++) {
    uint64_t x = (uint64_t)a[j] * b[j];
    uint32_t t = (uint32_t)x * WO_MU;
    uint32_t th = (uint32_t)(((uint64_t)t * WO_P) >> 32), xh = (uint32_t)(x >> 32);
    uint32_t d = xh - th;
    r[j] = xh < th ? d + WO_P : d;
  }
}
static inline void v_cube_rc(lanes x, fe rc) {
  lanes t, sq;
  v_add_c(t, x, rc);
  v_mul(sq, t, t);
  v_mul(x, sq, t);
}

static void v_mat4(lanes *x) {
  lanes t01, t23, t0123, t01123, t01233, d0, d2;
  v_add(t01, x[0], x[1]);
  v_add(t23, x[2], x[3]);
  v_add(t0123, t01, t23);
  v_add(t01123, t0123, x[1]);
  v_add(t01233, t0123, x[3]);
  v_add(d0, x[0], x[0]);
  v_add(d2, x[2], x[2]);
  v_add(x[3], t01233, d0);
  v_add(x[1], t01123, d2);
  v_add(x[0], t01123, t01);
  v_add(x[2], t01233, t23);
}
static void v_mds_light(lanes *s, int w) {
  for (int i = 0; i < w; i += 4) v_mat4(s + i);
  lanes sums[4];
  memset(sums, 0, sizeof sums);
  for (int i = 0; i < w; i++) v_add(sums[i & 3], sums[i & 3], s[i]);
  for (int i = 0; i < w; i++) v_add(s[i], s[i], sums[i & 3]);
}

/* diag * x for the internal layer's entries (1 1^T + diag(V)): every V is
 * +-1, +-2, +-3, +-4 or +-2^-e, so, as Plonky3's packed permutation does,
 * multiply by shifts: x 2^-e = (x + m p) / 2^e = ((x + m) >> e) + m K with
 * m = -x mod 2^e, K = (p - 1) / 2^e = 127 2^(24-e) (p = 127 2^24 + 1). */
static inline void v_neg(lanes x) {
  for (int j = 0; j < L; j++) x[j] = x[j] ? WO_P - x[j] : 0;
}
static inline __attribute__((always_inline)) void v_mul_diag(lanes r, const lanes x, int sign,
                                                             int num, int e) {
  if (e > 0) {
    const uint32_t mask = (1u << e) - 1u, K = 127u << (24 - e);
    for (int j = 0; j < L; j++) {
      uint32_t m = (0u - x[j]) & mask;
      r[j] = ((x[j] + m) >> e) + m * K;
    }
  } else if (num == 1) {
    memcpy(r, x, sizeof(lanes));
  } else if (num == 2) {
    v_add(r, x, x);
  } else if (num == 3) {
    lanes d;
    v_add(d, x, x);
    v_add(r, d, x);
  } else {
    lanes d;
    v_add(d, x, x);
    v_add(r, d, d);
  }
  if (sign < 0) v_neg(r);
}
static const signed char DIAG24[24][3] = {
    {-1, 2, 0}, {1, 1, 0},  {1, 2, 0},  {1, 1, 1},  {1, 3, 0},  {1, 4, 0},
    {-1, 1, 1}, {-1, 3, 0}, {-1, 4, 0}, {1, 1, 8},  {1, 1, 2},  {1, 1, 3},
    {1, 1, 4},  {1, 1, 5},  {1, 1, 6},  {1, 1, 24}, {-1, 1, 8}, {-1, 1, 3},
    {-1, 1, 4}, {-1, 1, 5}, {-1, 1, 6}, {-1, 1, 7}, {-1, 1, 9}, {-1, 1, 24}};
static const signed char DIAG16[16][3] = {
    {-1, 2, 0}, {1, 1, 0},  {1, 2, 0},  {1, 1, 1}, {1, 3, 0},  {1, 4, 0},  {-1, 1, 1}, {-1, 3, 0},
    {-1, 4, 0}, {1, 1, 8}, {1, 1, 3}, {1, 1, 24}, {-1, 1, 8}, {-1, 1, 3}, {-1, 1, 4}, {-1, 1, 24}};

/* p2_permute (wo_field.c) on L states at once; w is a constant in each
 * caller, so the diagonal's per-lane forms are specialised */
static inline __attribute__((always_inline)) void v_permute_w(const wo_p2 *p, lanes *s,
                                                              const int w) {
  v_mds_light(s, w);
  for (int rd = 0; rd < 4; rd++) {
    for (int i = 0; i < w; i++) v_cube_rc(s[i], p->ext_rc[rd][i]);
    v_mds_light(s, w);
  }
  for (int rd = 0; rd < p->rounds_p; rd++) {
    v_cube_rc(s[0], p->int_rc[rd]);
    lanes sum;
    memset(sum, 0, sizeof sum);
    for (int i = 0; i < w; i++) v_add(sum, sum, s[i]);
#pragma GCC unroll 24
    for (int i = 0; i < w; i++) {
      lanes d;
      const signed char *v = w == 16 ? DIAG16[i] : DIAG24[i];
      v_mul_diag(d, s[i], v[0], v[1], v[2]);
      v_add(s[i], sum, d);
    }
  }
  for (int rd = 4; rd < 8; rd++) {
    for (int i = 0; i < w; i++) v_cube_rc(s[i], p->ext_rc[rd][i]);
    v_mds_light(s, w);
  }
}

static void v_permute24(const wo_p2 *p, lanes *s) { v_permute_w(p, s, 24); }
static void v_permute16(const wo_p2 *p, lanes *s) { v_permute_w(p, s, 16); }

/* hash_leaf (PaddingFreeSponge<P24, 24, 16, 8>) of rows r0 .. r0 + n - 1
 * (n <= L), each row_len words, digests to out (8 words per row) */
void hash_leaves_packed(const fe *rows, size_t row_len, size_t r0, int n, fe *out) {
  const wo_p2 *p = p2_get(24);
  lanes s[24];
  memset(s, 0, sizeof s);
  size_t pos = 0;
  for (;;) {
    size_t take = row_len - pos < 16 ? row_len - pos : 16;
    for (size_t i = 0; i < take; i++)
      for (int j = 0; j < L; j++) s[i][j] = j < n ? rows[(r0 + j) * row_len + pos + i] : 0;
    pos += take;
    if (take == 0) break;  /* an empty trailing chunk is not permuted */
    v_permute24(p, s);
    if (pos == row_len || take < 16) break;
  }
  for (int j = 0; j < n; j++)
    for (int i = 0; i < 8; i++) out[(size_t)j * 8 + i] = s[i][j];
}

/* compress2 (TruncatedPermutation<P16, 2, 8, 16>) of node pairs
 * (i, i + half) for i = i0 .. i0 + n - 1 (n <= L) */
void compress_nodes_packed(const fe *src, size_t half, size_t i0, int n, fe *dst) {
  const wo_p2 *p = p2_get(16);
  lanes s[16];
  for (int w = 0; w < 8; w++)
    for (int j = 0; j < L; j++) {
      size_t i = i0 + (size_t)(j < n ? j : 0);
      s[w][j] = src[i * 8 + w];
      s[8 + w][j] = src[(i + half) * 8 + w];
    }
  v_permute16(p, s);
  for (int j = 0; j < n; j++)
    for (int w = 0; w < 8; w++) dst[(i0 + (size_t)j) * 8 + w] = s[w][j];
}
