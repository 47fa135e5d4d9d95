/*
 * Field, extension, randomness, Poseidon2, challenger and transcript.
 * Test infrastructure (the oracle): see whir_oracle.h.
 *
 * Third-party algorithms restated here (absent from the reference tree):
 *  - p3-koala-bear / p3-monty-31 @ e52636ec: KoalaBear in Montgomery form,
 *    two-adic generators, BinomialExtensionField<_, 4> with W = 3.
 *  - p3-poseidon2 @ e52636ec: external MDSMat4 light layer, internal layer
 *    1 + diag(V), S-box x^3, rounds (8, 20) for width 16 and (8, 23) for 24,
 *    constants drawn by Poseidon2::new_from_rng_128 from StdRng(1000).
 *  - rand 0.10 / rand_core 0.10 / chacha20 0.10: StdRng = ChaCha12 with key
 *    from SeedableRng::seed_from_u64 (PCG32 expansion).
 *  - p3-challenger DuplexChallenger<F, P16, 16, 8>.
 *  - bincode 1.3 + p3 serde: an element is 4 bytes LE of its Montgomery word.
 * Reference call sites: crates/whir/src/test.rs:183-200,
 * crates/transcript/src/poseidon.rs:13-164, crates/transcript/src/field.rs:1-25.
 */
#include "wo_internal.h"

fe fe_pow(fe a, uint64_t e) {
  fe r = WO_ONE;
  while (e) {
    if (e & 1) r = fe_mul(r, a);
    a = fe_mul(a, a);
    e >>= 1;
  }
  return r;
}
fe fe_inv(fe a) { return fe_pow(a, WO_P - 2); }

/* p3-koala-bear TWO_ADIC_GENERATORS (canonical).  Entry b generates the
 * subgroup of order 2^b; entry 24 equals 3^127 and each entry squares to the
 * previous one (checked in tests/test_oracle_field.py). */
static const uint32_t TWO_ADIC[25] = {
    0x1,        0x7f000000, 0x7e010002, 0x6832fe4a, 0x08dbd69c, 0x0a28f031, 0x5c4a5b99,
    0x29b75a80, 0x17668b8a, 0x27ad539b, 0x334d48c7, 0x7744959c, 0x768fc6fa, 0x303964b2,
    0x3e687d4d, 0x45a60e61, 0x6e2f4d7a, 0x163bd499, 0x6c4a8a45, 0x143ef899, 0x514ddcad,
    0x484ef19b, 0x205d63c3, 0x68e7dd49, 0x6ac49f88};
fe fe_two_adic(int bits) { return fe_from(TWO_ADIC[bits]); }

/* F[x]/(x^4 - W), W = 3 (p3-koala-bear BinomiallyExtendable<4>). */
ext ext_mul(ext a, ext b) {
  const fe W = 0x05fffffau; /* Montgomery form of 3 = 3 * 2^32 mod p */
  fe t[7] = {0};
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) t[i + j] = fe_add(t[i + j], fe_mul(a.c[i], b.c[j]));
  ext r;
  r.c[0] = fe_add(t[0], fe_mul(W, t[4]));
  r.c[1] = fe_add(t[1], fe_mul(W, t[5]));
  r.c[2] = fe_add(t[2], fe_mul(W, t[6]));
  r.c[3] = t[3];
  return r;
}
ext ext_pow(ext a, uint64_t e) {
  ext r = ext_one();
  while (e) {
    if (e & 1) r = ext_mul(r, a);
    a = ext_mul(a, a);
    e >>= 1;
  }
  return r;
}

/* ---------------- ChaCha12 StdRng ---------------- */
static inline uint32_t rotl(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }
#define QR(a, b, c, d)                      \
  a += b; d ^= a; d = rotl(d, 16);          \
  c += d; b ^= c; b = rotl(b, 12);          \
  a += b; d ^= a; d = rotl(d, 8);           \
  c += d; b ^= c; b = rotl(b, 7);

void wo_chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream, int rounds,
                     uint32_t out[16]) {
  uint32_t s[16] = {0x61707865, 0x3320646e, 0x79622d32, 0x6b206574};
  for (int i = 0; i < 8; i++) s[4 + i] = key[i];
  s[12] = (uint32_t)counter;
  s[13] = (uint32_t)(counter >> 32);
  s[14] = (uint32_t)stream;
  s[15] = (uint32_t)(stream >> 32);
  uint32_t x[16];
  memcpy(x, s, sizeof x);
  for (int i = 0; i < rounds; i += 2) {
    QR(x[0], x[4], x[8], x[12]) QR(x[1], x[5], x[9], x[13])
    QR(x[2], x[6], x[10], x[14]) QR(x[3], x[7], x[11], x[15])
    QR(x[0], x[5], x[10], x[15]) QR(x[1], x[6], x[11], x[12])
    QR(x[2], x[7], x[8], x[13]) QR(x[3], x[4], x[9], x[14])
  }
  for (int i = 0; i < 16; i++) out[i] = x[i] + s[i];
}

/* rand_core SeedableRng::seed_from_u64: PCG32 stream fills the 32-byte seed. */
void rng_seed(wo_rng *r, uint64_t state) {
  const uint64_t MUL = 6364136223846793005ull, INC = 11634580027462260723ull;
  for (int i = 0; i < 8; i++) {
    state = state * MUL + INC;
    uint32_t xs = (uint32_t)(((state >> 18) ^ state) >> 27);
    uint32_t rot = (uint32_t)(state >> 59);
    r->key[i] = (xs >> rot) | (xs << ((32 - rot) & 31));
  }
  r->counter = 0;
  r->idx = 16;
}
uint32_t rng_u32(wo_rng *r) {
  if (r->idx == 16) {
    wo_chacha_block(r->key, r->counter++, 0, 12, r->buf);
    r->idx = 0;
  }
  return r->buf[r->idx++];
}
/* StandardUniform for MontyField31: next_u32 >> 1, rejected unless < p,
 * taken as the Montgomery word. */
fe rng_fe(wo_rng *r) {
  for (;;) {
    uint32_t v = rng_u32(r) >> 1;
    if (v < WO_P) return v;
  }
}
void wo_rand_fe(uint64_t seed, uint32_t *out, size_t n) {
  wo_rng r;
  rng_seed(&r, seed);
  for (size_t i = 0; i < n; i++) out[i] = rng_fe(&r);
}

/* ---------------- Poseidon2 ---------------- */
static wo_p2 P2_16, P2_24;
static int p2_ready;

static fe frac(int sign, uint32_t num, int log_den) {
  fe v = fe_mul(fe_from(num), fe_inv(fe_pow(fe_from(2), (uint64_t)log_den)));
  return sign < 0 ? fe_neg(v) : v;
}

static void p2_make(wo_p2 *p, int width) {
  /* internal diagonal V: M_I = 1 1^T + diag(V) (p3-koala-bear poseidon2.rs) */
  static const int V16[16][3] = {{-1, 2, 0}, {1, 1, 0},  {1, 2, 0},   {1, 1, 1},
                                 {1, 3, 0},  {1, 4, 0},  {-1, 1, 1},  {-1, 3, 0},
                                 {-1, 4, 0}, {1, 1, 8},  {1, 1, 3},   {1, 1, 24},
                                 {-1, 1, 8}, {-1, 1, 3}, {-1, 1, 4},  {-1, 1, 24}};
  static const int V24[24][3] = {
      {-1, 2, 0}, {1, 1, 0},  {1, 2, 0},  {1, 1, 1},  {1, 3, 0},  {1, 4, 0},
      {-1, 1, 1}, {-1, 3, 0}, {-1, 4, 0}, {1, 1, 8},  {1, 1, 2},  {1, 1, 3},
      {1, 1, 4},  {1, 1, 5},  {1, 1, 6},  {1, 1, 24}, {-1, 1, 8}, {-1, 1, 3},
      {-1, 1, 4}, {-1, 1, 5}, {-1, 1, 6}, {-1, 1, 7}, {-1, 1, 9}, {-1, 1, 24}};
  p->width = width;
  p->rounds_f = 8;
  p->rounds_p = width == 16 ? 20 : 23;
  for (int i = 0; i < width; i++) {
    const int *v = width == 16 ? V16[i] : V24[i];
    p->diag[i] = frac(v[0], (uint32_t)v[1], v[2]);
  }
  /* new_from_rng_128: initial external [F; W] x4, terminal x4, internal x rounds_p */
  wo_rng r;
  rng_seed(&r, 1000);
  for (int rd = 0; rd < 8; rd++)
    for (int i = 0; i < width; i++) p->ext_rc[rd][i] = rng_fe(&r);
  for (int rd = 0; rd < p->rounds_p; rd++) p->int_rc[rd] = rng_fe(&r);
}

/* built once at load time, before any parallel region can race on it */
__attribute__((constructor)) static void p2_init(void) {
  p2_make(&P2_16, 16);
  p2_make(&P2_24, 24);
  p2_ready = 1;
}
const wo_p2 *p2_get(int width) {
  if (!p2_ready) p2_init();
  return width == 16 ? &P2_16 : &P2_24;
}

static void mat4(fe *x) {
  fe t01 = fe_add(x[0], x[1]), t23 = fe_add(x[2], x[3]);
  fe t0123 = fe_add(t01, t23);
  fe t01123 = fe_add(t0123, x[1]), t01233 = fe_add(t0123, x[3]);
  fe y3 = fe_add(t01233, fe_dbl(x[0]));
  fe y1 = fe_add(t01123, fe_dbl(x[2]));
  fe y0 = fe_add(t01123, t01);
  fe y2 = fe_add(t01233, t23);
  x[0] = y0; x[1] = y1; x[2] = y2; x[3] = y3;
}
static void mds_light(fe *s, int w) {
  for (int i = 0; i < w; i += 4) mat4(s + i);
  fe sums[4] = {0, 0, 0, 0};
  for (int i = 0; i < w; i++) sums[i & 3] = fe_add(sums[i & 3], s[i]);
  for (int i = 0; i < w; i++) s[i] = fe_add(s[i], sums[i & 3]);
}
static inline fe cube(fe x) { return fe_mul(fe_mul(x, x), x); }

void p2_permute(const wo_p2 *p, fe *s) {
  int w = p->width;
  mds_light(s, w);
  for (int rd = 0; rd < 4; rd++) {
    for (int i = 0; i < w; i++) s[i] = cube(fe_add(s[i], p->ext_rc[rd][i]));
    mds_light(s, w);
  }
  for (int rd = 0; rd < p->rounds_p; rd++) {
    s[0] = cube(fe_add(s[0], p->int_rc[rd]));
    fe sum = 0;
    for (int i = 0; i < w; i++) sum = fe_add(sum, s[i]);
    for (int i = 0; i < w; i++) s[i] = fe_add(sum, fe_mul(p->diag[i], s[i]));
  }
  for (int rd = 4; rd < 8; rd++) {
    for (int i = 0; i < w; i++) s[i] = cube(fe_add(s[i], p->ext_rc[rd][i]));
    mds_light(s, w);
  }
}

int wo_p2_permute(int width, uint32_t *state) {
  if (width != 16 && width != 24) return -1;
  p2_permute(p2_get(width), state);
  return 0;
}
int wo_p2_constants(int width, uint32_t *ext_rc, uint32_t *int_rc, uint32_t *diag,
                    int *rounds_p) {
  if (width != 16 && width != 24) return -1;
  const wo_p2 *p = p2_get(width);
  for (int rd = 0; rd < 8; rd++) memcpy(ext_rc + rd * width, p->ext_rc[rd], 4 * width);
  memcpy(int_rc, p->int_rc, 4 * p->rounds_p);
  memcpy(diag, p->diag, 4 * width);
  *rounds_p = p->rounds_p;
  return 0;
}

/* PaddingFreeSponge<P24, 24, 16, 8>: overwrite-mode absorption, no padding;
 * a trailing partial chunk is permuted, an empty trailing chunk is not. */
void hash_leaf(const fe *in, size_t n, fe out[8]) {
  const wo_p2 *p = p2_get(24);
  fe s[24] = {0};
  size_t pos = 0;
  for (;;) {
    size_t i = 0;
    for (; i < 16 && pos < n; i++) s[i] = in[pos++];
    if (i == 16) {
      p2_permute(p, s);
      if (pos == n) break;
      continue;
    }
    if (i != 0) p2_permute(p, s);
    break;
  }
  memcpy(out, s, 32);
}
void wo_hash_leaf(const uint32_t *in, size_t n, uint32_t out[8]) { hash_leaf(in, n, out); }

/* TruncatedPermutation<P16, 2, 8, 16> */
void compress2(const fe l[8], const fe r[8], fe out[8]) {
  fe s[16];
  memcpy(s, l, 32);
  memcpy(s + 8, r, 32);
  p2_permute(p2_get(16), s);
  memcpy(out, s, 32);
}
void wo_compress(const uint32_t left[8], const uint32_t right[8], uint32_t out[8]) {
  compress2(left, right, out);
}

/* ---------------- DuplexChallenger<F, P16, 16, 8> ---------------- */
void chal_init(wo_chal *c) { memset(c, 0, sizeof *c); }
static void duplexing(wo_chal *c) {
  for (int i = 0; i < c->n_in; i++) c->state[i] = c->in[i];
  c->n_in = 0;
  p2_permute(p2_get(16), c->state);
  memcpy(c->out, c->state, 32);
  c->n_out = 8;
}
void chal_observe(wo_chal *c, fe v) {
  c->n_out = 0;
  c->in[c->n_in++] = v;
  if (c->n_in == 8) duplexing(c);
}
fe chal_sample(wo_chal *c) {
  if (c->n_in || !c->n_out) duplexing(c);
  return c->out[--c->n_out];
}
size_t chal_sample_bits(wo_chal *c, int bits) {
  fe v = chal_sample(c);
  return (size_t)fe_canon(v) & ((1ull << bits) - 1);
}

/* ---------------- transcript ---------------- */
void ts_writer(wo_ts *t, uint8_t *buf, size_t cap) {
  memset(t, 0, sizeof *t);
  chal_init(&t->ch);
  t->buf = buf;
  t->cap = cap;
}
void ts_reader(wo_ts *t, const uint8_t *buf, size_t len) {
  memset(t, 0, sizeof *t);
  chal_init(&t->ch);
  t->buf = (uint8_t *)buf;
  t->cap = len;
  t->reading = 1;
}
static void put_u32(wo_ts *t, uint32_t v) {
  if (t->len + 4 > t->cap) { t->err = 1; return; }
  for (int i = 0; i < 4; i++) t->buf[t->len++] = (uint8_t)(v >> (8 * i));
}
static uint32_t get_u32(wo_ts *t) {
  if (t->len + 4 > t->cap) { t->err = 1; return 0; }
  uint32_t v = 0;
  for (int i = 0; i < 4; i++) v |= (uint32_t)t->buf[t->len++] << (8 * i);
  if (v >= WO_P) { t->err = 1; return 0; }
  return v;
}
void ts_write_fe(wo_ts *t, fe v, int observe) {
  put_u32(t, v);
  if (observe) chal_observe(&t->ch, v);
}
void ts_write_ext(wo_ts *t, ext v, int observe) {
  for (int i = 0; i < 4; i++) put_u32(t, v.c[i]);
  if (observe) for (int i = 0; i < 4; i++) chal_observe(&t->ch, v.c[i]);
}
void ts_write_digest(wo_ts *t, const fe d[8], int observe) {
  for (int i = 0; i < 8; i++) put_u32(t, d[i]);
  if (observe) for (int i = 0; i < 8; i++) chal_observe(&t->ch, d[i]);
}
fe ts_read_fe(wo_ts *t, int observe) {
  fe v = get_u32(t);
  if (observe) chal_observe(&t->ch, v);
  return v;
}
ext ts_read_ext(wo_ts *t, int observe) {
  ext v;
  for (int i = 0; i < 4; i++) v.c[i] = get_u32(t);
  if (observe) for (int i = 0; i < 4; i++) chal_observe(&t->ch, v.c[i]);
  return v;
}
void ts_read_digest(wo_ts *t, fe d[8], int observe) {
  for (int i = 0; i < 8; i++) d[i] = get_u32(t);
  if (observe) for (int i = 0; i < 8; i++) chal_observe(&t->ch, d[i]);
}
ext ts_draw_ext(wo_ts *t) {
  ext v;
  for (int i = 0; i < 4; i++) v.c[i] = chal_sample(&t->ch);
  return v;
}
fe ts_draw_fe(wo_ts *t) { return chal_sample(&t->ch); }
size_t ts_draw_bits(wo_ts *t, int bits) { return chal_sample_bits(&t->ch, bits); }

/* ---------------- exported scalar helpers ---------------- */
uint32_t wo_fe_from_u32(uint32_t c) { return fe_from(c); }
uint32_t wo_fe_to_u32(uint32_t m) { return fe_canon(m); }
uint32_t wo_fe_mul(uint32_t a, uint32_t b) { return fe_mul(a, b); }
uint32_t wo_fe_add(uint32_t a, uint32_t b) { return fe_add(a, b); }
uint32_t wo_fe_inv(uint32_t a) { return fe_inv(a); }
void wo_ext_mul(const uint32_t *a, const uint32_t *b, uint32_t *out) {
  ext x, y;
  memcpy(&x, a, 16);
  memcpy(&y, b, 16);
  ext r = ext_mul(x, y);
  memcpy(out, &r, 16);
}
uint32_t wo_two_adic_generator(int bits) { return fe_two_adic(bits); }

int wo_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void wo_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
