/*
 * Internal definitions shared by the oracle's translation units.
 * Test infrastructure: see whir_oracle.h.
 */
#ifndef WO_INTERNAL_H
#define WO_INTERNAL_H

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "whir_oracle.h"

#ifdef _OPENMP
#include <omp.h>
#endif

typedef uint32_t fe;
typedef struct { fe c[4]; } ext;

/* KoalaBear p = 2^31 - 2^24 + 1, Montgomery radix 2^32 (p3-koala-bear). */
#define WO_P 0x7f000001u
#define WO_MU 0x81000001u     /* p^-1 mod 2^32 */
#define WO_R2 0x17f7efe4u     /* 2^64 mod p */
#define WO_ONE 0x01fffffeu    /* 2^32 mod p: Montgomery form of 1 */

static inline fe fe_reduce(uint64_t x) { /* Montgomery reduction, x < p*2^32 */
  uint32_t t = (uint32_t)x * WO_MU;
  uint64_t tp = (uint64_t)t * WO_P;
  uint32_t xh = (uint32_t)(x >> 32), th = (uint32_t)(tp >> 32);
  uint32_t r = xh - th;
  return xh < th ? r + WO_P : r;
}
static inline fe fe_mul(fe a, fe b) { return fe_reduce((uint64_t)a * b); }
static inline fe fe_add(fe a, fe b) { uint32_t r = a + b; return r >= WO_P ? r - WO_P : r; }
static inline fe fe_sub(fe a, fe b) { return a >= b ? a - b : a + WO_P - b; }
static inline fe fe_neg(fe a) { return a ? WO_P - a : 0; }
static inline fe fe_dbl(fe a) { return fe_add(a, a); }
static inline fe fe_from(uint32_t x) { return fe_mul(x % WO_P, WO_R2); }
static inline fe fe_canon(fe a) { return fe_reduce(a); }
fe fe_pow(fe a, uint64_t e);
fe fe_inv(fe a);
fe fe_two_adic(int bits);

static inline ext ext_zero(void) { ext r = {{0, 0, 0, 0}}; return r; }
static inline ext ext_one(void) { ext r = {{WO_ONE, 0, 0, 0}}; return r; }
static inline ext ext_from_fe(fe a) { ext r = {{a, 0, 0, 0}}; return r; }
static inline ext ext_add(ext a, ext b) {
  ext r; for (int i = 0; i < 4; i++) r.c[i] = fe_add(a.c[i], b.c[i]); return r;
}
static inline ext ext_sub(ext a, ext b) {
  ext r; for (int i = 0; i < 4; i++) r.c[i] = fe_sub(a.c[i], b.c[i]); return r;
}
static inline ext ext_neg(ext a) {
  ext r; for (int i = 0; i < 4; i++) r.c[i] = fe_neg(a.c[i]); return r;
}
static inline ext ext_scale(ext a, fe s) {
  ext r; for (int i = 0; i < 4; i++) r.c[i] = fe_mul(a.c[i], s); return r;
}
static inline ext ext_dbl(ext a) { return ext_add(a, a); }
ext ext_mul(ext a, ext b);
static inline ext ext_sq(ext a) { return ext_mul(a, a); }
static inline int ext_eq(ext a, ext b) { return memcmp(&a, &b, sizeof(ext)) == 0; }
static inline int ext_is_zero(ext a) { return !(a.c[0] | a.c[1] | a.c[2] | a.c[3]); }
ext ext_pow(ext a, uint64_t e);

/* ---- rng (rand 0.10 StdRng = ChaCha12, seeded by PCG32 expansion) ---- */
typedef struct {
  uint32_t key[8];
  uint64_t counter;
  uint32_t buf[16];
  int idx;
} wo_rng;
void rng_seed(wo_rng *r, uint64_t seed);
uint32_t rng_u32(wo_rng *r);
fe rng_fe(wo_rng *r);

/* ---- Poseidon2 ---- */
typedef struct {
  int width, rounds_f, rounds_p;
  fe ext_rc[8][24];
  fe int_rc[32];
  fe diag[24];
} wo_p2;
const wo_p2 *p2_get(int width);
void p2_permute(const wo_p2 *p, fe *state);
void hash_leaf(const fe *in, size_t n, fe out[8]);
void compress2(const fe l[8], const fe r[8], fe out[8]);
/* lane-packed hashing for the timed baseline (wo_packed.c): WO_LANES states
 * per call, the same results as hash_leaf / compress2 */
#define WO_LANES 8
int wo_packed(void);
void hash_leaves_packed(const fe *rows, size_t row_len, size_t r0, int n, fe *out);
void compress_nodes_packed(const fe *src, size_t half, size_t i0, int n, fe *dst);

/* ---- challenger + transcript (crates/transcript/src/poseidon.rs) ---- */
typedef struct {
  fe state[16];
  fe in[8];
  int n_in;
  fe out[8];
  int n_out;
} wo_chal;
void chal_init(wo_chal *c);
void chal_observe(wo_chal *c, fe v);
fe chal_sample(wo_chal *c);
size_t chal_sample_bits(wo_chal *c, int bits);

typedef struct {
  wo_chal ch;
  uint8_t *buf;
  size_t len, cap;
  int reading; /* 0 writer, 1 reader */
  int err;
} wo_ts;
void ts_writer(wo_ts *t, uint8_t *buf, size_t cap);
void ts_reader(wo_ts *t, const uint8_t *buf, size_t len);
void ts_write_fe(wo_ts *t, fe v, int observe);
void ts_write_ext(wo_ts *t, ext v, int observe);
void ts_write_digest(wo_ts *t, const fe d[8], int observe);
fe ts_read_fe(wo_ts *t, int observe);
ext ts_read_ext(wo_ts *t, int observe);
void ts_read_digest(wo_ts *t, fe d[8], int observe);
ext ts_draw_ext(wo_ts *t);
fe ts_draw_fe(wo_ts *t);
size_t ts_draw_bits(wo_ts *t, int bits);

/* ---- poly helpers ---- */
void eq_table(const ext *z, int k, ext scale, ext *out);
ext eval_eq_xy(const ext *x, const ext *y, int n);
ext eval_pow_xy_f(const fe *x, const ext *y, int n);
ext eval_base(const fe *poly, int k, const ext *z);
ext eval_extp(const ext *poly, int k, const ext *z);
ext horner(const ext *c, size_t n, ext x);
ext eval_univariate(const ext *poly, size_t n, ext x);
void compress_hi_base(const fe *poly, int k, const ext *z, int kz, ext *out);
void compress_lo_base(const fe *poly, int k, const ext *z, int kz, ext *out);
void fix_lo(ext *a, size_t n, ext r);
void coeffs(const ext *poly, const ext *w, size_t n, ext *c0, ext *c2);
void combine_eqs(ext *w, int k, const ext *points, int n, ext alpha);
void combine_pows(ext *w, int k, const fe *vars, int n, ext alpha, int shift);
void combine_pows_scaled(ext *w, int k, const fe *vars, int n, const ext *scales);
void dft_batch(const fe *in, size_t h_in, size_t width, int log_h, fe *out);

/* ---- merkle tree with all levels (halves pairing) ---- */
typedef struct {
  int log_h;
  size_t row_len;  /* field elements per leaf row */
  const fe *rows;  /* borrowed codeword */
  fe *nodes;       /* level 0 .. log_h, level l at offset (2^(h+1) - 2^(h-l+1))*8 */
} wo_tree;
void tree_build(wo_tree *t, const fe *rows, int log_h, size_t row_len);
void tree_free(wo_tree *t);
const fe *tree_node(const wo_tree *t, int level, size_t i);
void tree_query(const wo_tree *t, wo_ts *ts, size_t index);
int tree_verify(wo_ts *ts, const fe root[8], size_t index, size_t row_len, int log_h,
                fe *row_out);

#endif
