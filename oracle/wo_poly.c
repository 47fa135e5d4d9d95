/*
 * Multilinear-polynomial kernels, constraint combination, DFT and Merkle
 * tree of the oracle.  Test infrastructure: see whir_oracle.h.
 *
 * Each function is the plain (unpacked, unsplit) form of the reference's
 * routine; the reference's split/packed variants compute the same exact
 * field values, so one restatement covers both.
 */
#include "wo_internal.h"

/* Point::eq (crates/poly/src/point.rs:110-126): LSB-first doubling, bit i of
 * the index selects z_i. */
void eq_table(const ext *z, int k, ext scale, ext *out) {
  out[0] = scale;
  for (int i = 0; i < k; i++) {
    size_t h = (size_t)1 << i;
    for (size_t j = 0; j < h; j++) {
      ext hi = ext_mul(out[j], z[i]);
      out[j + h] = hi;
      out[j] = ext_sub(out[j], hi);
    }
  }
}

/* eval_eq_xy (crates/poly/src/lib.rs:17-23): prod (2 x y - x - y + 1) */
ext eval_eq_xy(const ext *x, const ext *y, int n) {
  ext acc = ext_one();
  for (int i = 0; i < n; i++) {
    ext t = ext_sub(ext_sub(ext_dbl(ext_mul(y[i], x[i])), x[i]), y[i]);
    acc = ext_mul(acc, ext_add(t, ext_one()));
  }
  return acc;
}
/* eval_pow_xy (crates/poly/src/lib.rs:25-31): prod (x y - y + 1) */
ext eval_pow_xy_f(const fe *x, const ext *y, int n) {
  ext acc = ext_one();
  for (int i = 0; i < n; i++) {
    ext t = ext_add(ext_sub(ext_scale(y[i], x[i]), y[i]), ext_one());
    acc = ext_mul(acc, t);
  }
  return acc;
}

/* Poly::eval_base / eval_ext via SplitEq (crates/poly/src/eq.rs:107-250) */
ext eval_base(const fe *poly, int k, const ext *z) {
  size_t n = (size_t)1 << k;
  if (n == 1) return ext_from_fe(poly[0]);
  ext *eq = malloc(n * sizeof(ext));
  eq_table(z, k, ext_one(), eq);
  ext acc = ext_zero();
  for (size_t i = 0; i < n; i++) acc = ext_add(acc, ext_scale(eq[i], poly[i]));
  free(eq);
  return acc;
}
ext eval_extp(const ext *poly, int k, const ext *z) {
  size_t n = (size_t)1 << k;
  if (n == 1) return poly[0];
  int k0 = k / 2, k1 = k - k0;
  size_t n0 = (size_t)1 << k0, n1 = (size_t)1 << k1;
  ext *e0 = malloc(n0 * sizeof(ext)), *e1 = malloc(n1 * sizeof(ext));
  eq_table(z, k0, ext_one(), e0);
  eq_table(z + k0, k1, ext_one(), e1);
  ext acc = ext_zero();
  for (size_t h = 0; h < n1; h++) {
    ext part = ext_zero();
    for (size_t l = 0; l < n0; l++) part = ext_add(part, ext_mul(e0[l], poly[h * n0 + l]));
    acc = ext_add(acc, ext_mul(part, e1[h]));
  }
  free(e0);
  free(e1);
  return acc;
}

/* VecOps::horner (crates/common/src/utils.rs:124-127): rfold acc*x + c */
ext horner(const ext *c, size_t n, ext x) {
  ext acc = ext_zero();
  for (size_t i = n; i-- > 0;) acc = ext_add(ext_mul(acc, x), c[i]);
  return acc;
}
/* Poly::eval_univariate -> par_horner (crates/common/src/utils.rs:95-117) */
ext eval_univariate(const ext *poly, size_t n, ext x) { return horner(poly, n, x); }

/* SplitEq::compress_hi (crates/poly/src/eq.rs:290-398): fix the high kz
 * variables to z: out[j] = sum_h eq(z)[h] * P[h * 2^(k-kz) + j] */
void compress_hi_base(const fe *poly, int k, const ext *z, int kz, ext *out) {
  size_t nz = (size_t)1 << kz, inner = (size_t)1 << (k - kz);
  ext *eq = malloc(nz * sizeof(ext));
  eq_table(z, kz, ext_one(), eq);
  for (size_t j = 0; j < inner; j++) out[j] = ext_zero();
#pragma omp parallel
  {
    ext *acc = calloc(inner, sizeof(ext));
#pragma omp for schedule(static)
    for (long long h = 0; h < (long long)nz; h++)
      for (size_t j = 0; j < inner; j++)
        acc[j] = ext_add(acc[j], ext_scale(eq[h], poly[(size_t)h * inner + j]));
#pragma omp critical
    for (size_t j = 0; j < inner; j++) out[j] = ext_add(out[j], acc[j]);
    free(acc);
  }
  free(eq);
}

/* SplitEq::compress_lo / compress_lo_into (crates/poly/src/eq.rs:400-539):
 * fix the low kz variables: out[i] = sum_j eq(z)[j] * P[i * 2^kz + j] */
void compress_lo_base(const fe *poly, int k, const ext *z, int kz, ext *out) {
  size_t nz = (size_t)1 << kz, nout = (size_t)1 << (k - kz);
  ext *eq = malloc(nz * sizeof(ext));
  eq_table(z, kz, ext_one(), eq);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)nout; i++) {
    ext acc = ext_zero();
    for (size_t j = 0; j < nz; j++) acc = ext_add(acc, ext_scale(eq[j], poly[(size_t)i * nz + j]));
    out[i] = acc;
  }
  free(eq);
}

/* Poly::fix_lo_var_mut (crates/poly/src/poly.rs:131-142) */
void fix_lo(ext *a, size_t n, ext r) {
  for (size_t i = 0; i < n / 2; i++)
    a[i] = ext_add(ext_mul(ext_sub(a[2 * i + 1], a[2 * i]), r), a[2 * i]);
}

/* coeffs (crates/whir/src/sumcheck/expr.rs:14-27) */
void coeffs(const ext *poly, const ext *w, size_t n, ext *c0, ext *c2) {
  ext a0 = ext_zero(), a2 = ext_zero();
  for (size_t i = 0; i < n; i += 2) {
    a0 = ext_add(a0, ext_mul(w[i], poly[i]));
    ext dw = ext_sub(ext_dbl(w[i + 1]), w[i]);
    ext df = ext_sub(ext_dbl(poly[i + 1]), poly[i]);
    a2 = ext_add(a2, ext_mul(dw, df));
  }
  *c0 = a0;
  *c2 = a2;
}

/* eq::combine_eqs (crates/whir/src/sumcheck/combine.rs:179-203):
 * w[i] += sum_n alpha^n eq(z_n)[i] */
void combine_eqs(ext *w, int k, const ext *points, int n, ext alpha) {
  size_t N = (size_t)1 << k;
  ext *eq = malloc(N * sizeof(ext));
  ext a = ext_one();
  for (int t = 0; t < n; t++) {
    eq_table(points + (size_t)t * k, k, a, eq);
    for (size_t i = 0; i < N; i++) w[i] = ext_add(w[i], eq[i]);
    a = ext_mul(a, alpha);
  }
  free(eq);
}

/* pow::combine_pows (combine.rs:408-438): w[i] += sum_n alpha^(shift+n) var_n^i */
void combine_pows(ext *w, int k, const fe *vars, int n, ext alpha, int shift) {
  size_t N = (size_t)1 << k;
  ext a = ext_pow(alpha, (uint64_t)shift);
  for (int t = 0; t < n; t++) {
    fe p = WO_ONE;
    for (size_t i = 0; i < N; i++) {
      w[i] = ext_add(w[i], ext_scale(a, p));
      p = fe_mul(p, vars[t]);
    }
    a = ext_mul(a, alpha);
  }
}
/* pow::combine_pows_scaled (combine.rs:441-468): w[i] += sum_n s_n var_n^i */
void combine_pows_scaled(ext *w, int k, const fe *vars, int n, const ext *scales) {
  size_t N = (size_t)1 << k;
  for (int t = 0; t < n; t++) {
    fe p = WO_ONE;
    for (size_t i = 0; i < N; i++) {
      w[i] = ext_add(w[i], ext_scale(scales[t], p));
      p = fe_mul(p, vars[t]);
    }
  }
}

/* TwoAdicSubgroupDft::dft_batch (p3-dft, called at crates/whir/src/whir.rs:34):
 * out[i][c] = sum_r in[r][c] * w^(r i), w = two_adic_generator(log_h),
 * natural order; rows >= h_in are zero.  Iterative radix-2 per column. */
void dft_batch(const fe *in, size_t h_in, size_t width, int log_h, fe *out) {
  size_t h = (size_t)1 << log_h;
  fe *tw = malloc((h / 2 + 1) * sizeof(fe));
  fe g = fe_two_adic(log_h);
  tw[0] = WO_ONE;
  for (size_t i = 1; i < h / 2; i++) tw[i] = fe_mul(tw[i - 1], g);
  /* bit-reversed positions, shared by every column */
  uint32_t *rev = malloc(h * sizeof(uint32_t));
  rev[0] = 0;
  for (size_t i = 1; i < h; i++) rev[i] = (rev[i >> 1] >> 1) | ((uint32_t)(i & 1) << (log_h - 1));
#pragma omp parallel
  {
    fe *a = malloc(h * sizeof(fe));
#pragma omp for schedule(dynamic)
    for (long long c = 0; c < (long long)width; c++) {
      memset(a, 0, h * sizeof(fe));
      for (size_t i = 0; i < h_in; i++) a[rev[i]] = in[i * width + c];
      for (int s = 1; s <= log_h; s++) {
        size_t m = (size_t)1 << s, half = m / 2, step = h / m;
        for (size_t blk = 0; blk < h; blk += m)
          for (size_t j = 0; j < half; j++) {
            fe u = a[blk + j], v = fe_mul(a[blk + j + half], tw[j * step]);
            a[blk + j] = fe_add(u, v);
            a[blk + j + half] = fe_sub(u, v);
          }
      }
      for (size_t i = 0; i < h; i++) out[i * width + c] = a[i];
    }
    free(a);
  }
  free(rev);
  free(tw);
}
void wo_dft_batch(const uint32_t *in, size_t h_in, size_t width, int log_h_out,
                  uint32_t *out) {
  dft_batch(in, h_in, width, log_h_out, out);
}

/* Merkle tree with every level kept (crates/merkle/src/poseidon.rs:61-105,
 * poseidon_packed.rs:98-143): node_{l+1}[i] = C(node_l[i], node_l[i + n/2]). */
static size_t level_off(int log_h, int level) {
  return (((size_t)2 << log_h) - ((size_t)2 << (log_h - level))) * 8;
}
const fe *tree_node(const wo_tree *t, int level, size_t i) {
  return t->nodes + level_off(t->log_h, level) + i * 8;
}
void tree_build(wo_tree *t, const fe *rows, int log_h, size_t row_len) {
  size_t h = (size_t)1 << log_h;
  t->log_h = log_h;
  t->row_len = row_len;
  t->rows = rows;
  t->nodes = malloc((2 * h - 1) * 8 * sizeof(fe));
  if (wo_packed()) {  /* the timed baseline: WO_LANES leaves / nodes per call */
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)h; i += WO_LANES)
      hash_leaves_packed(rows, row_len, (size_t)i,
                         (int)((long long)h - i < WO_LANES ? (long long)h - i : WO_LANES),
                         t->nodes + (size_t)i * 8);
    for (int l = 0; l < log_h; l++) {
      size_t n = h >> l, half = n / 2;
      fe *src = t->nodes + level_off(log_h, l), *dst = t->nodes + level_off(log_h, l + 1);
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)half; i += WO_LANES)
        compress_nodes_packed(src, half, (size_t)i,
                              (int)((long long)half - i < WO_LANES ? (long long)half - i : WO_LANES),
                              dst);
    }
    return;
  }
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)h; i++)
    hash_leaf(rows + (size_t)i * row_len, row_len, t->nodes + (size_t)i * 8);
  for (int l = 0; l < log_h; l++) {
    size_t n = h >> l, half = n / 2;
    fe *src = t->nodes + level_off(log_h, l), *dst = t->nodes + level_off(log_h, l + 1);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)half; i++)
      compress2(src + (size_t)i * 8, src + ((size_t)i + half) * 8, dst + (size_t)i * 8);
  }
}
void tree_free(wo_tree *t) { free(t->nodes); t->nodes = NULL; }
void wo_merkle_tree(const uint32_t *rows, int log_h, size_t row_len, uint32_t *levels) {
  wo_tree t;
  tree_build(&t, rows, log_h, row_len);
  memcpy(levels, t.nodes, (((size_t)2 << log_h) - 1) * 32);
  tree_free(&t);
}

/* query (poseidon_packed.rs:145-233): leaf row as F hints, then the k sibling
 * digests bottom-up as hints; nothing observed. */
void tree_query(const wo_tree *t, wo_ts *ts, size_t index) {
  const fe *row = t->rows + index * t->row_len;
  for (size_t i = 0; i < t->row_len; i++) ts_write_fe(ts, row[i], 0);
  size_t idx = index;
  for (int l = 0; l < t->log_h; l++) {
    size_t mid = (size_t)1 << (t->log_h - l - 1);
    ts_write_digest(ts, tree_node(t, l, idx ^ mid), 0);
    idx &= mid - 1;
  }
}
/* verify (poseidon_packed.rs:235-257) + verify_merkle_proof (poseidon.rs:11-30) */
int tree_verify(wo_ts *ts, const fe root[8], size_t index, size_t row_len, int log_h,
                fe *row_out) {
  for (size_t i = 0; i < row_len; i++) row_out[i] = ts_read_fe(ts, 0);
  fe acc[8];
  hash_leaf(row_out, row_len, acc);
  if (index >= ((size_t)1 << log_h)) return -1;
  size_t idx = index;
  for (int l = 0; l < log_h; l++) {
    fe w[8], nxt[8];
    ts_read_digest(ts, w, 0);
    size_t mid = (size_t)1 << (log_h - l - 1);
    if (idx >= mid) compress2(w, acc, nxt);
    else compress2(acc, w, nxt);
    memcpy(acc, nxt, 32);
    idx &= mid - 1;
  }
  if (ts->err) return -2;
  return memcmp(acc, root, 32) == 0 ? 0 : -3;
}

/* ---------------- exported wrappers (raw uint32 buffers) ---------------- */
void wo_eq_table(const uint32_t *point, int k, const uint32_t *scale, uint32_t *out) {
  ext s;
  memcpy(&s, scale, 16);
  eq_table((const ext *)point, k, s, (ext *)out);
}
void wo_compress_hi(const uint32_t *poly, int k, const uint32_t *point, int kz,
                    uint32_t *out) {
  compress_hi_base(poly, k, (const ext *)point, kz, (ext *)out);
}
void wo_compress_lo(const uint32_t *poly, int k, const uint32_t *point, int kz,
                    uint32_t *out) {
  compress_lo_base(poly, k, (const ext *)point, kz, (ext *)out);
}
void wo_eval_ext(const uint32_t *poly, int k, const uint32_t *point, uint32_t *out) {
  ext r = eval_extp((const ext *)poly, k, (const ext *)point);
  memcpy(out, &r, 16);
}
void wo_coeffs(const uint32_t *poly, const uint32_t *weights, int k, uint32_t *c0,
               uint32_t *c2) {
  ext a, b;
  coeffs((const ext *)poly, (const ext *)weights, (size_t)1 << k, &a, &b);
  memcpy(c0, &a, 16);
  memcpy(c2, &b, 16);
}
void wo_fix_lo(uint32_t *poly, int k, const uint32_t *r) {
  ext rr;
  memcpy(&rr, r, 16);
  fix_lo((ext *)poly, (size_t)1 << k, rr);
}
void wo_combine_eqs(uint32_t *weights, int k, const uint32_t *points, int n,
                    const uint32_t *alpha) {
  ext a;
  memcpy(&a, alpha, 16);
  combine_eqs((ext *)weights, k, (const ext *)points, n, a);
}
void wo_combine_pows(uint32_t *weights, int k, const uint32_t *vars, int n,
                     const uint32_t *alpha, int shift) {
  ext a;
  memcpy(&a, alpha, 16);
  combine_pows((ext *)weights, k, vars, n, a, shift);
}
void wo_combine_pows_scaled(uint32_t *weights, int k, const uint32_t *vars, int n,
                            const uint32_t *scales) {
  combine_pows_scaled((ext *)weights, k, vars, n, (const ext *)scales);
}
