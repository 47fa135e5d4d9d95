/*
 * WHIR parameters, stacked sumcheck prover (SVO rounds, expression,
 * fold, fold_with_code), WHIR commit/open, and the verifier.
 * Test infrastructure (the oracle): see whir_oracle.h.
 *
 * Follows crates/whir/src/{params.rs, whir.rs, sumcheck/{mod,prover,svo,
 * expr,combine,verifier}.rs} and the harness crates/whir/src/test.rs:174-254.
 */
#include <math.h>
#include <stdio.h>

#include "wo_internal.h"

/* ---------------- params.rs ---------------- */
static const double LOG2_10 = 3.321928094887362347870319429489390175864831393;

static double log_eta(int s, int lir) {
  if (s == 0) return 0.;
  if (s == 1) return -(0.5 * lir + LOG2_10 + 1.);
  return -(lir + LOG2_10 + 1.);
}
static double list_size_bits(int s, int log_degree, int lir) {
  double le = log_eta(s, lir);
  if (s == 0) return 0.;
  if (s == 1) return lir / 2. - (1. + le);
  return (double)(log_degree + lir) - le;
}
static double log_1_delta(int s, int lir) {
  double eta = pow(2., log_eta(s, lir));
  double rate = 1. / (double)(1u << lir);
  double delta;
  if (s == 0) delta = 0.5 * (1. - rate);
  else if (s == 1) delta = 1. - sqrt(rate) - eta;
  else delta = 1. - rate - eta;
  return log2(1. - delta);
}
/* params.rs:118-122 converts with Rust's `as usize`, which saturates: NaN
 * and negative values (rate 1, log_inv_rate 0, where log(1 - delta) is 0 or
 * positive) give 0 queries.  Counts past MAX_STIR (the library's limit,
 * within the 4096-entry index arrays here) are reported as -1. */
#define MAX_STIR 3072 /* the library's limit */
int wo_n_stir_queries(int s, int security, int lir) {
  double q = ceil(-(double)security / log_1_delta(s, lir));
  if (!(q > 0.)) return 0;
  if (q > (double)MAX_STIR) return -1;
  return (int)q;
}
static double ood_error(int s, int log_degree, int lir, int field_bits, int samples) {
  if (s == 0) return 0.;
  double lsb = list_size_bits(s, log_degree, lir);
  double error = 2. * lsb + (double)(log_degree * samples);
  return (double)(samples * field_bits) + 1. - error;
}
int wo_n_ood_queries(int s, int security, int log_degree, int lir, int field_bits) {
  if (s == 0) return 0;
  for (int n = 1; n < 64; n++)
    if (ood_error(s, log_degree, lir, field_bits, n) >= (double)security) return n;
  return -1; /* the reference panics here */
}
void wo_number_of_rounds(int folding, int k, int *n_rounds, int *final_rounds) {
  if (k <= 6) { *n_rounds = 0; *final_rounds = k - folding; return; }
  int nr = (k - 6 + folding - 1) / folding;
  *final_rounds = k - nr * folding;
  *n_rounds = nr - 1;
}
#define EXT_BITS 124 /* bits of |BinomialExtensionField<KoalaBear, 4>| */

/* ---------------- small helpers ---------------- */
static ext *ext_alloc(size_t n) { return calloc(n ? n : 1, sizeof(ext)); }
static void expand(ext *out, int k, ext v) { /* Point::expand (point.rs:115-124) */
  for (int i = 0; i < k; i++) { out[i] = v; v = ext_sq(v); }
}
static ext inv_two_ext(void) { return ext_from_fe(fe_inv(fe_from(2))); }
/* lagrange_weights_012 / extrapolate_012 (sumcheck/mod.rs:17-28) */
static void lagrange012(ext r, ext w[3]) {
  ext it = inv_two_ext(), one = ext_one(), two = ext_dbl(ext_one());
  w[0] = ext_mul(ext_mul(ext_sub(r, one), ext_sub(r, two)), it);
  w[1] = ext_mul(r, ext_sub(two, r));
  w[2] = ext_mul(ext_mul(r, ext_sub(r, one)), it);
}
static ext extrapolate012(ext e0, ext e1, ext e2, ext r) {
  ext w[3];
  lagrange012(r, w);
  return ext_add(ext_add(ext_mul(e0, w[0]), ext_mul(e1, w[1])), ext_mul(e2, w[2]));
}
static size_t ipow3(int r) { size_t v = 1; while (r--) v *= 3; return v; }

/* ---------------- SVO (sumcheck/svo.rs) ---------------- */
typedef struct {
  int k, k_svo;
  ext *point;       /* [k] */
  ext *compressed;  /* [2^k_svo] */
  ext *partial;     /* concatenated partial evals, l = 1..k_svo, 2^l each */
  ext eval;
} svo_claim;

static size_t partial_off(int l) { return ((size_t)1 << l) - 2; } /* sum_{j<l} 2^j for j>=1 */

/* SvoPoint::new + SvoPoint::eval (svo.rs:64-91) */
static void svo_claim_make(svo_claim *c, int k_svo, const ext *point, int k, const fe *poly) {
  c->k = k;
  c->k_svo = k_svo;
  c->point = ext_alloc(k);
  memcpy(c->point, point, k * sizeof(ext));
  size_t ns = (size_t)1 << k_svo;
  c->compressed = ext_alloc(ns);
  compress_hi_base(poly, k, point + k_svo, k - k_svo, c->compressed);
  ext *eq = ext_alloc(ns);
  eq_table(point, k_svo, ext_one(), eq);
  c->eval = ext_zero();
  for (size_t j = 0; j < ns; j++) c->eval = ext_add(c->eval, ext_mul(eq[j], c->compressed[j]));
  free(eq);
  c->partial = ext_alloc(partial_off(k_svo + 1));
  for (int l = 1; l <= k_svo; l++) { /* svo_partial_evals (svo.rs:18-38) */
    size_t na = (size_t)1 << l, nr = (size_t)1 << (k_svo - l);
    ext *er = ext_alloc(nr);
    eq_table(point + l, k_svo - l, ext_one(), er);
    ext *out = c->partial + partial_off(l);
    for (size_t a = 0; a < na; a++) {
      ext acc = ext_zero();
      for (size_t r = 0; r < nr; r++) acc = ext_add(acc, ext_mul(c->compressed[a + na * r], er[r]));
      out[a] = acc;
    }
    free(er);
  }
}
static void svo_claim_free(svo_claim *c) {
  free(c->point); free(c->compressed); free(c->partial);
}

/* Svo::calculate_accumulators for one claim weighted by alpha (svo.rs:225-278).
 * The reference groups claims sharing a point; accumulators are linear in the
 * weighted partial evals, so per-claim accumulation gives the same sums.
 * acc layout: per round r, [acc0 (3^r) | acc2 (3^r)]. */
static size_t acc_size(int k_svo) { size_t s = 0; for (int r = 0; r < k_svo; r++) s += 2 * ipow3(r); return s; }
static void accumulate(ext *acc, const svo_claim *c, ext alpha) {
  int k = c->k_svo;
  size_t off = 0;
  for (int r = 0; r < k; r++) {
    int l = r + 1;
    size_t n = ipow3(r), na = (size_t)1 << l;
    const ext *pe = c->partial + partial_off(l);
    ext *eq = ext_alloc(na), *u = ext_alloc(l);
    for (int which = 0; which < 2; which++) {
      for (size_t t = 0; t < n; t++) {
        size_t tt = t;
        for (int i = 0; i < r; i++) { u[i] = ext_from_fe(fe_from((uint32_t)(tt % 3))); tt /= 3; }
        u[r] = which ? ext_dbl(ext_one()) : ext_zero();
        eq_table(u, l, ext_one(), eq);
        ext dot = ext_zero();
        for (size_t a = 0; a < na; a++) dot = ext_add(dot, ext_mul(ext_mul(alpha, pe[a]), eq[a]));
        ext v = ext_mul(eval_eq_xy(u, c->point, l), dot);
        acc[off + which * n + t] = ext_add(acc[off + which * n + t], v);
      }
    }
    free(eq); free(u);
    off += 2 * n;
  }
}

/* SvoPoint::new + SvoPoint::eval and Svo::calculate_accumulators for one
 * claim of weight 1 (svo.rs:64-91, 225-278), exported for the port of
 * svo.rs's test_accumulators.  out: the claim value (4 words), then the
 * accumulators in accumulate()'s layout (acc_size(l0) extension elements). */
void wo_svo_accumulators(const uint32_t *poly, int k, const uint32_t *point, int l0,
                         uint32_t *out) {
  svo_claim c;
  svo_claim_make(&c, l0, (const ext *)point, k, (const fe *)poly);
  size_t n = acc_size(l0);
  ext *acc = ext_alloc(n ? n : 1);
  for (size_t i = 0; i < n; i++) acc[i] = ext_zero();
  accumulate(acc, &c, ext_one());
  memcpy(out, &c.eval, sizeof(ext));
  memcpy(out + 4, acc, n * sizeof(ext));
  free(acc);
  svo_claim_free(&c);
}

/* ---------------- stacked layout (prover.rs:32-354) ---------------- */
typedef struct { int nbits; unsigned char bits[32]; int poly; } lay_entry;

static int sel_cmp(const void *pa, const void *pb) { /* Ord for Selector(Vec<bool>) */
  const lay_entry *a = pa, *b = pb;
  int n = a->nbits < b->nbits ? a->nbits : b->nbits;
  for (int i = 0; i < n; i++)
    if (a->bits[i] != b->bits[i]) return a->bits[i] < b->bits[i] ? -1 : 1;
  return (a->nbits > b->nbits) - (a->nbits < b->nbits);
}
static size_t sel_index(const lay_entry *e) {
  size_t v = 0;
  for (int i = 0; i < e->nbits; i++) v |= (size_t)e->bits[i] << i;
  return v;
}
/* ProverStack::layout / VerifierLayout::new: stable sort by k, place the
 * largest first, then order by selector. Returns total k. */
static int make_layout(int n, const int *pk, lay_entry *out) {
  int *order = malloc(n * sizeof(int));
  for (int i = 0; i < n; i++) order[i] = i;
  for (int i = 1; i < n; i++) { /* stable insertion sort by k */
    int v = order[i], j = i;
    while (j > 0 && pk[order[j - 1]] > pk[v]) { order[j] = order[j - 1]; j--; }
    order[j] = v;
  }
  size_t total = 0;
  for (int i = 0; i < n; i++) total += (size_t)1 << pk[i];
  int k = 0;
  while (((size_t)1 << k) < total) k++;
  size_t off = 0;
  for (int t = 0; t < n; t++) {
    int id = order[n - 1 - t];
    lay_entry *e = &out[t];
    e->poly = id;
    e->nbits = k - pk[id];
    size_t idx = off >> pk[id];
    for (int b = 0; b < e->nbits; b++) e->bits[b] = (idx >> b) & 1;
    off += (size_t)1 << pk[id];
  }
  qsort(out, n, sizeof(lay_entry), sel_cmp);
  free(order);
  return k;
}

typedef struct {
  ext *point; /* [k] */
  ext eval;
  ext *acc;   /* accumulators, acc_size(k_svo) */
} virt_claim;

typedef struct {
  const wo_params *prm;
  int n_polys;
  const int *pk;
  const fe **polys;
  int k, k_svo;
  lay_entry *lay;
  int n_claims;
  svo_claim *claims; /* creation order */
  int *claim_poly;
  int n_virt;
  virt_claim virt[64];
  fe *stacked;       /* layout.poly */
} prover_layout;

/* claims in layout order: for each selector, that poly's claims in creation order */
static int claims_layout_order(const prover_layout *L, int *out_idx, int *out_ent) {
  int m = 0;
  for (int e = 0; e < L->n_polys; e++)
    for (int c = 0; c < L->n_claims; c++)
      if (L->claim_poly[c] == L->lay[e].poly) { out_idx[m] = c; out_ent[m] = e; m++; }
  return m;
}

/* ProverLayout::write_virtual_eval (prover.rs:232-277) */
static void write_virtual_eval(prover_layout *L, wo_ts *ts) {
  virt_claim *v = &L->virt[L->n_virt++];
  v->point = ext_alloc(L->k);
  expand(v->point, L->k, ts_draw_ext(ts));
  v->eval = ext_zero();
  v->acc = ext_alloc(acc_size(L->k_svo));
  for (int e = 0; e < L->n_polys; e++) {
    int id = L->lay[e].poly, kp = L->pk[id];
    ext sel[32];
    for (int b = 0; b < L->lay[e].nbits; b++)
      sel[b] = L->lay[e].bits[b] ? ext_one() : ext_zero();
    ext weight = eval_eq_xy(sel, v->point + kp, L->lay[e].nbits);
    svo_claim c;
    svo_claim_make(&c, L->k_svo, v->point, kp, L->polys[id]);
    v->eval = ext_add(v->eval, ext_mul(weight, c.eval));
    accumulate(v->acc, &c, weight);
    svo_claim_free(&c);
  }
  ts_write_ext(ts, v->eval, 1);
}

typedef struct {
  ext sum, alpha;
  ext *rs; int n_rs;
  ext *poly, *w; /* expression */
  int k;         /* variables of the expression */
} sumcheck;

/* ProverLayout::new_prover (prover.rs:280-354) incl. expression (225-229) */
static void new_prover(prover_layout *L, wo_ts *ts, sumcheck *sc) {
  ext alpha = ts_draw_ext(ts);
  int n = L->n_claims;
  int *ord = malloc((n + 1) * sizeof(int)), *ent = malloc((n + 1) * sizeof(int));
  int m = claims_layout_order(L, ord, ent);
  ext *alphas = ext_alloc(n);
  ext *evals = ext_alloc(n + L->n_virt);
  ext a = ext_one();
  for (int i = 0; i < m; i++) { alphas[ord[i]] = a; evals[i] = L->claims[ord[i]].eval; a = ext_mul(a, alpha); }
  for (int v = 0; v < L->n_virt; v++) evals[m + v] = L->virt[v].eval;
  ext sum = horner(evals, m + L->n_virt, alpha);

  size_t as = acc_size(L->k_svo);
  ext *acc = ext_alloc(as);
  for (int c = 0; c < n; c++) accumulate(acc, &L->claims[c], alphas[c]);
  ext av = ext_pow(alpha, (uint64_t)n);
  for (int v = 0; v < L->n_virt; v++) {
    for (size_t i = 0; i < as; i++) acc[i] = ext_add(acc[i], ext_mul(av, L->virt[v].acc[i]));
    av = ext_mul(av, alpha);
  }
  sc->rs = ext_alloc(64);
  sc->n_rs = 0;
  size_t off = 0;
  for (int r = 0; r < L->k_svo; r++) {
    size_t nw = ipow3(r);
    ext *wts = ext_alloc(nw);
    wts[0] = ext_one();
    size_t len = 1;
    for (int i = 0; i < r; i++) { /* lagrange_weights_012_multi (svo.rs:7-16) */
      ext l3[3];
      lagrange012(sc->rs[i], l3);
      ext *nx = ext_alloc(len * 3);
      for (int d = 0; d < 3; d++)
        for (size_t t = 0; t < len; t++) nx[d * len + t] = ext_mul(wts[t], l3[d]);
      free(wts); wts = nx; len *= 3;
    }
    ext c0 = ext_zero(), c2 = ext_zero();
    for (size_t t = 0; t < nw; t++) {
      c0 = ext_add(c0, ext_mul(acc[off + t], wts[t]));
      c2 = ext_add(c2, ext_mul(acc[off + nw + t], wts[t]));
    }
    free(wts);
    off += 2 * nw;
    ts_write_ext(ts, c0, 1);
    ts_write_ext(ts, c2, 1);
    ext rr = ts_draw_ext(ts);
    sum = extrapolate012(c0, ext_sub(sum, c0), c2, rr);
    sc->rs[sc->n_rs++] = rr;
  }
  free(acc);

  /* expression: compress_stacked + combine_eqs (prover.rs:185-222) */
  int ks = L->k_svo;
  sc->k = L->k - ks;
  size_t N = (size_t)1 << sc->k;
  sc->poly = ext_alloc(N);
  sc->w = ext_alloc(N);
  for (int e = 0; e < L->n_polys; e++) {
    int id = L->lay[e].poly, kp = L->pk[id];
    size_t o = sel_index(&L->lay[e]) << (kp - ks);
    compress_lo_base(L->polys[id], kp, sc->rs, ks, sc->poly + o);
  }
  a = ext_one();
  for (int i = 0; i < m; i++) {
    const svo_claim *c = &L->claims[ord[i]];
    int ksplit = c->k - c->k_svo;
    size_t size = (size_t)1 << ksplit, o = sel_index(&L->lay[ent[i]]) * size;
    ext scale = ext_mul(a, eval_eq_xy(c->point, sc->rs, ks));
    ext *eq = ext_alloc(size);
    eq_table(c->point + ks, ksplit, scale, eq);
    for (size_t j = 0; j < size; j++) sc->w[o + j] = ext_add(sc->w[o + j], eq[j]);
    free(eq);
    a = ext_mul(a, alpha);
  }
  for (int v = 0; v < L->n_virt; v++) {
    ext scale = ext_mul(a, eval_eq_xy(L->virt[v].point, sc->rs, ks));
    ext *eq = ext_alloc(N);
    eq_table(L->virt[v].point + ks, sc->k, scale, eq);
    for (size_t j = 0; j < N; j++) sc->w[j] = ext_add(sc->w[j], eq[j]);
    free(eq);
    a = ext_mul(a, alpha);
  }
  sc->sum = sum;
  sc->alpha = alpha;
  free(ord); free(ent); free(alphas); free(evals);
}

/* Expression::round (expr.rs:52-70) */
static ext sc_round(sumcheck *sc, wo_ts *ts) {
  size_t N = (size_t)1 << sc->k;
  ext c0, c2;
  coeffs(sc->poly, sc->w, N, &c0, &c2);
  ts_write_ext(ts, c0, 1);
  ts_write_ext(ts, c2, 1);
  ext r = ts_draw_ext(ts);
  fix_lo(sc->poly, N, r);
  fix_lo(sc->w, N, r);
  sc->k--;
  sc->sum = extrapolate012(c0, ext_sub(sc->sum, c0), c2, r);
  return r;
}

/* SumcheckProver::fold (prover.rs:378-397) with combine_claims (combine.rs:38-64) */
static void sc_fold(sumcheck *sc, wo_ts *ts, int d, const ext *eq_pts, const ext *eq_evals,
                    int n_eq, const fe *pow_vars, const ext *pow_evals, int n_pow, ext *rs_out) {
  sc->alpha = ts_draw_ext(ts);
  ext *ev = ext_alloc(n_eq + n_pow);
  memcpy(ev, eq_evals, n_eq * sizeof(ext));
  memcpy(ev + n_eq, pow_evals, n_pow * sizeof(ext));
  sc->sum = ext_add(sc->sum, horner(ev, n_eq + n_pow, sc->alpha));
  free(ev);
  combine_eqs(sc->w, sc->k, eq_pts, n_eq, sc->alpha);
  combine_pows(sc->w, sc->k, pow_vars, n_pow, sc->alpha, n_eq);
  for (int i = 0; i < d; i++) {
    ext r = sc_round(sc, ts);
    rs_out[i] = r;
    sc->rs[sc->n_rs++] = r;
  }
}

/* recursion g of fold_with_code (prover.rs:437-461) */
typedef struct { size_t *idx; ext *val; size_t n; } evalmap;
static ext em_get(const evalmap *m, size_t index) {
  size_t lo = 0, hi = m->n;
  while (lo < hi) {
    size_t mid = (lo + hi) / 2;
    if (m->idx[mid] < index) lo = mid + 1; else hi = mid;
  }
  if (lo < m->n && m->idx[lo] == index) return m->val[lo];
  fprintf(stderr, "oracle: missing eval index %zu\n", index);
  abort();
}
static ext g_rec(int k, const evalmap *m, int round, size_t index, const ext *rs, fe two_inv) {
  if (round == 0) return em_get(m, index);
  size_t l = (size_t)1 << (k - (round - 1)), mid = l / 2;
  size_t i_lo = index & (mid - 1), i_hi = i_lo + mid;
  ext glo = g_rec(k, m, round - 1, i_lo, rs, two_inv);
  ext ghi = g_rec(k, m, round - 1, i_hi, rs, two_inv);
  fe om = fe_two_adic(k - (round - 1));
  ext even = ext_scale(ext_add(glo, ghi), two_inv);
  ext odd = ext_scale(ext_scale(ext_sub(glo, ghi), two_inv), fe_inv(fe_pow(om, i_lo)));
  return ext_add(even, ext_mul(rs[round - 1], ext_sub(odd, even)));
}
static int cmp_size(const void *a, const void *b) {
  size_t x = *(const size_t *)a, y = *(const size_t *)b;
  return (x > y) - (x < y);
}

/* SumcheckProver::fold_with_code (prover.rs:400-561) */
static void sc_fold_with_code(sumcheck *sc, wo_ts *ts, int d, const ext *eq_pts,
                              const ext *eq_evals, int n_eq, const size_t *indexes, int n_idx,
                              const fe *data, int k_data, size_t row_len, ext *rs_out) {
  sc->alpha = ts_draw_ext(ts);
  ext alpha = sc->alpha;
  sc->sum = ext_add(sc->sum, horner(eq_evals, n_eq, alpha));
  combine_eqs(sc->w, sc->k, eq_pts, n_eq, alpha);

  ext *scales = ext_alloc(n_idx);
  ext a = ext_pow(alpha, (uint64_t)n_eq);
  for (int i = 0; i < n_idx; i++) { scales[i] = a; a = ext_mul(a, alpha); }
  size_t nz = (size_t)1 << sc->n_rs;
  ext *eq = ext_alloc(nz);
  eq_table(sc->rs, sc->n_rs, ext_one(), eq);
  for (int i = 0; i < n_idx; i++) {
    ext dot = ext_zero();
    for (size_t j = 0; j < row_len; j++) dot = ext_add(dot, ext_scale(eq[j], data[indexes[i] * row_len + j]));
    sc->sum = ext_add(sc->sum, ext_mul(scales[i], dot));
  }
  fe omega = fe_two_adic(k_data);
  fe *ws = malloc(n_idx * sizeof(fe)), *tsw = malloc(n_idx * sizeof(fe));
  size_t mid0 = ((size_t)1 << k_data) / 2;
  for (int i = 0; i < n_idx; i++) {
    ws[i] = fe_pow(omega, indexes[i]);
    tsw[i] = fe_inv(fe_pow(omega, indexes[i] & (mid0 - 1)));
  }
  /* recursive indexes (prover.rs:483-495) and their evals (497-506) */
  size_t cap = 0;
  for (int round = 0; round < d; round++) cap += (size_t)n_idx << (round + 1);
  size_t *ri = malloc((cap ? cap : 1) * sizeof(size_t)), nri = 0;
  for (int round = 0; round < d; round++) {
    size_t stride = (size_t)1 << (k_data - round - 1), count = (size_t)1 << (round + 1);
    for (int i = 0; i < n_idx; i++) {
      size_t base = indexes[i] & (stride - 1);
      for (size_t t = 0; t < count; t++) ri[nri++] = base + t * stride;
    }
  }
  qsort(ri, nri, sizeof(size_t), cmp_size);
  size_t u = 0;
  for (size_t i = 0; i < nri; i++) if (!u || ri[u - 1] != ri[i]) ri[u++] = ri[i];
  evalmap em = {ri, ext_alloc(u), u};
  for (size_t i = 0; i < u; i++) {
    ext dot = ext_zero();
    for (size_t j = 0; j < row_len; j++) dot = ext_add(dot, ext_scale(eq[j], data[ri[i] * row_len + j]));
    em.val[i] = dot;
  }
  free(eq);

  fe two_inv = fe_inv(fe_from(2));
  ext rs_cur[32];
  for (int round = 0; round < d; round++) {
    size_t N = (size_t)1 << sc->k;
    ext c0, c2;
    coeffs(sc->poly, sc->w, N, &c0, &c2);
    size_t l = (size_t)1 << (k_data - round), mid = l / 2;
    for (int i = 0; i < n_idx; i++) {
      size_t i_lo = indexes[i] & (mid - 1), i_hi = i_lo + mid;
      ext glo = g_rec(k_data, &em, round, i_lo, rs_cur, two_inv);
      ext ghi = g_rec(k_data, &em, round, i_hi, rs_cur, two_inv);
      ext even = ext_scale(ext_add(glo, ghi), two_inv);
      ext odd = ext_scale(ext_scale(ext_sub(glo, ghi), two_inv), tsw[i]);
      c0 = ext_add(c0, ext_mul(scales[i], even));
      fe wt = fe_sub(fe_dbl(ws[i]), WO_ONE);
      c2 = ext_add(c2, ext_scale(ext_mul(scales[i], ext_sub(ext_dbl(odd), even)), wt));
    }
    ts_write_ext(ts, c0, 1);
    ts_write_ext(ts, c2, 1);
    ext r = ts_draw_ext(ts);
    sc->sum = extrapolate012(c0, ext_sub(sc->sum, c0), c2, r);
    rs_cur[round] = r;
    fix_lo(sc->poly, N, r);
    fix_lo(sc->w, N, r);
    sc->k--;
    for (int i = 0; i < n_idx; i++) {
      ext f = ext_add(ext_one(), ext_mul(r, ext_add(ext_neg(ext_one()), ext_from_fe(ws[i]))));
      scales[i] = ext_mul(scales[i], f);
      ws[i] = fe_mul(ws[i], ws[i]);
      tsw[i] = fe_mul(tsw[i], tsw[i]);
      if ((indexes[i] >> (k_data - round - 2)) & 1) tsw[i] = fe_neg(tsw[i]);
    }
  }
  combine_pows_scaled(sc->w, sc->k, ws, n_idx, scales);
  for (int round = 0; round < d; round++) { rs_out[round] = rs_cur[round]; sc->rs[sc->n_rs++] = rs_cur[round]; }
  free(scales); free(ws); free(tsw); free(ri); free(em.val);
}

/* ---------------- WHIR (whir.rs) ---------------- */
static void round_params(const wo_params *p, int round, int *kfd, int *this_rate, int *prev_rate) {
  int prev_red = round == 0 ? 0 : p->initial_reduction + round - 1;
  int this_red = p->initial_reduction + round;
  int k_domain = p->rate + p->k - prev_red;
  *kfd = k_domain - p->folding;
  *prev_rate = p->rate + round * p->folding - prev_red;
  *this_rate = p->rate + (round + 1) * p->folding - this_red;
}
/* stir_indexes (whir.rs:64-77): draw, sort, dedup */
static int stir_indexes(wo_ts *ts, int bits, int n, size_t *out) {
  for (int i = 0; i < n; i++) out[i] = ts_draw_bits(ts, bits);
  qsort(out, n, sizeof(size_t), cmp_size);
  int m = 0;
  for (int i = 0; i < n; i++) if (!m || out[m - 1] != out[i]) out[m++] = out[i];
  return m;
}

typedef struct { fe *codeword; wo_tree tree; } commitment;

/* commit_base / commit_ext (whir.rs:20-61): rows of 2^folding (Ext) coefficients,
 * zero-padded to 2^(k + rate - folding) rows, DFT per column, Merkle commit. */
static void commit_rows(commitment *c, wo_ts *ts, const fe *poly, int k, int rate, int folding,
                        int dim) {
  int log_h = k + rate - folding;
  size_t width = ((size_t)dim) << folding, h_in = (size_t)1 << (k - folding);
  c->codeword = malloc(((size_t)1 << log_h) * width * sizeof(fe));
  dft_batch(poly, h_in, width, log_h, c->codeword);
  tree_build(&c->tree, c->codeword, log_h, width);
  ts_write_digest(ts, tree_node(&c->tree, log_h, 0), 1);
}
static void commit_free(commitment *c) { free(c->codeword); tree_free(&c->tree); }

static int whir_open(const wo_params *p, wo_ts *ts, commitment *c0, prover_layout *L) {
  int n_ood = wo_n_ood_queries(p->soundness, p->security_level, p->k, p->rate, EXT_BITS);
  if (n_ood < 0) return -10;
  for (int i = 0; i < n_ood; i++) write_virtual_eval(L, ts);
  sumcheck sc;
  new_prover(L, ts, &sc);
  int n_rounds, final_rounds;
  wo_number_of_rounds(p->folding, p->k, &n_rounds, &final_rounds);
  commitment prev = {0}, cur = {0};
  int have_prev = 0;
  ext round_point[32];
  size_t *idx = malloc(4096 * sizeof(size_t));
  for (int round = 0; round < n_rounds; round++) {
    int kfd, this_rate, prev_rate;
    round_params(p, round, &kfd, &this_rate, &prev_rate);
    int kp = sc.k;
    commit_rows(&cur, ts, (const fe *)sc.poly, kp, this_rate, p->folding, 4);
    int n_o = wo_n_ood_queries(p->soundness, p->security_level, kp, this_rate, EXT_BITS);
    ext *pts = ext_alloc((size_t)n_o * kp), *evs = ext_alloc(n_o);
    for (int i = 0; i < n_o; i++) {
      expand(pts + (size_t)i * kp, kp, ts_draw_ext(ts));
      evs[i] = eval_extp(sc.poly, kp, pts + (size_t)i * kp);
      ts_write_ext(ts, evs[i], 1);
    }
    int n_s = wo_n_stir_queries(p->soundness, p->security_level, prev_rate);
    int m = stir_indexes(ts, kfd, n_s, idx);
    fe omega = fe_two_adic(kfd);
    ext rs_new[32];
    if (round == 0) {
      for (int i = 0; i < m; i++) tree_query(&c0->tree, ts, idx[i]);
      sc_fold_with_code(&sc, ts, p->folding, pts, evs, n_o, idx, m, c0->codeword,
                        c0->tree.log_h, c0->tree.row_len, rs_new);
    } else {
      fe *vars = malloc(m * sizeof(fe));
      ext *pev = ext_alloc(m);
      for (int i = 0; i < m; i++) {
        tree_query(&prev.tree, ts, idx[i]);
        vars[i] = fe_pow(omega, idx[i]);
        pev[i] = eval_extp((const ext *)(prev.codeword + idx[i] * prev.tree.row_len), p->folding,
                           round_point);
      }
      sc_fold(&sc, ts, p->folding, pts, evs, n_o, vars, pev, m, rs_new);
      free(vars); free(pev);
    }
    memcpy(round_point, rs_new, p->folding * sizeof(ext));
    if (have_prev) commit_free(&prev);
    prev = cur;
    have_prev = 1;
    free(pts); free(evs);
  }
  for (size_t i = 0; i < ((size_t)1 << sc.k); i++) ts_write_ext(ts, sc.poly[i], 1);
  int kfd, this_rate, prev_rate;
  round_params(p, n_rounds, &kfd, &this_rate, &prev_rate);
  int n_s = wo_n_stir_queries(p->soundness, p->security_level, prev_rate);
  int m = stir_indexes(ts, kfd, n_s, idx);
  for (int i = 0; i < m; i++) tree_query(have_prev ? &prev.tree : &c0->tree, ts, idx[i]);
  if (have_prev) commit_free(&prev);
  int ok = sc.k == final_rounds ? 0 : -11;
  free(idx); free(sc.rs); free(sc.poly); free(sc.w);
  return ok;
}

/* Parameter sets the reference can run: its round shapes are usize
 * arithmetic (params.rs:186-202, whir.rs:150-166) that panics when a result
 * would be negative, every codeword fits the 2^24 two-adic subgroup, and
 * every round's and the final STIR query count is within MAX_STIR. */
static int stir_counts_ok(const wo_params *p) {
  if (p->folding < 1 || p->k < p->folding || p->security_level < 0) return 0;
  if (p->k + p->rate - p->folding > 24) return 0; /* two-adicity of KoalaBear */
  int n_rounds, final_rounds;
  wo_number_of_rounds(p->folding, p->k, &n_rounds, &final_rounds);
  if (final_rounds < 0) return 0;
  for (int round = 0; round <= n_rounds; round++) {
    int kfd, this_rate, prev_rate;
    round_params(p, round, &kfd, &this_rate, &prev_rate);
    if (kfd < 0 || this_rate < 0 || prev_rate < 0) return 0;
    if (round < n_rounds && p->k - p->folding * (round + 1) + this_rate - p->folding > 24) return 0;
    if (wo_n_stir_queries(p->soundness, p->security_level, prev_rate) < 0) return 0;
  }
  return 1;
}

static int group_offset(const wo_claims *cl, int g) {
  int o = 0;
  for (int i = 0; i < g; i++) o += cl->group_n[i];
  return o;
}

/* a group's point is expanded to the size of its first polynomial, so every
 * member must have that size (and every id must name a polynomial) */
static int groups_ok(const wo_claims *cl) {
  int o = 0;
  for (int g = 0; g < cl->n_groups; g++) {
    if (cl->group_n[g] < 1) return 0;
    for (int j = 0; j < cl->group_n[g]; j++) {
      int id = cl->group_ids[o + j];
      if (id < 0 || id >= cl->n_polys) return 0;
      if (cl->poly_k[id] != cl->poly_k[cl->group_ids[o]]) return 0;
    }
    o += cl->group_n[g];
  }
  return 1;
}

/* every stacked polynomial has at least `folding` variables: the
 * reference's expression build fixes the low `folding` variables of each
 * (compress_stacked, crates/whir/src/sumcheck/prover.rs:211-222, asserts
 * rs.k() <= k_poly with rs.k() = folding, whir.rs:184), and its claims split
 * off that many (SvoPoint::new, svo.rs:64-69, asserts k_svo <= point.k()) */
static int sizes_ok(const wo_params *prm, const wo_claims *cl) {
  if (cl->n_polys < 1) return 0;
  for (int i = 0; i < cl->n_polys; i++)
    if (cl->poly_k[i] < prm->folding) return 0;
  return 1;
}

int wo_prove(const wo_params *prm, const wo_claims *cl, const uint32_t *polys, uint8_t *proof,
             size_t cap, size_t *len, uint32_t *checkpoint) {
  if (!stir_counts_ok(prm)) return -1;  /* parameters the reference cannot run */
  if (!groups_ok(cl) || !sizes_ok(prm, cl)) return -1;
  wo_ts ts;
  ts_writer(&ts, proof, cap);
  prover_layout L;
  memset(&L, 0, sizeof L);
  L.prm = prm;
  L.n_polys = cl->n_polys;
  L.pk = cl->poly_k;
  L.polys = malloc(cl->n_polys * sizeof(fe *));
  size_t off = 0;
  for (int i = 0; i < cl->n_polys; i++) { L.polys[i] = polys + off; off += (size_t)1 << cl->poly_k[i]; }
  L.lay = malloc(cl->n_polys * sizeof(lay_entry));
  L.k = make_layout(cl->n_polys, cl->poly_k, L.lay);
  L.k_svo = prm->folding;
  if (L.k != prm->k) return -1;
  L.stacked = calloc((size_t)1 << L.k, sizeof(fe));
  for (int e = 0; e < L.n_polys; e++) {
    int id = L.lay[e].poly;
    memcpy(L.stacked + (sel_index(&L.lay[e]) << L.pk[id]), L.polys[id], 4 * ((size_t)1 << L.pk[id]));
  }
  commitment c0;
  commit_rows(&c0, &ts, L.stacked, L.k, prm->rate, prm->folding, 1);
  int total = group_offset(cl, cl->n_groups);
  L.claims = calloc(total ? total : 1, sizeof(svo_claim));
  L.claim_poly = malloc((total ? total : 1) * sizeof(int));
  for (int g = 0; g < cl->n_groups; g++) {
    int o = group_offset(cl, g);
    int kg = L.pk[cl->group_ids[o]];
    ext z = ts_draw_ext(&ts);
    ext pt[32];
    expand(pt, kg, z);
    for (int j = 0; j < cl->group_n[g]; j++) {
      int id = cl->group_ids[o + j];
      svo_claim *c = &L.claims[L.n_claims];
      svo_claim_make(c, L.k_svo, pt, L.pk[id], L.polys[id]);
      L.claim_poly[L.n_claims++] = id;
      ts_write_ext(&ts, c->eval, 1);
    }
  }
  int rc = whir_open(prm, &ts, &c0, &L);
  *checkpoint = ts_draw_fe(&ts);
  *len = ts.len;
  commit_free(&c0);
  for (int i = 0; i < L.n_claims; i++) svo_claim_free(&L.claims[i]);
  for (int v = 0; v < L.n_virt; v++) { free(L.virt[v].point); free(L.virt[v].acc); }
  free(L.claims); free(L.claim_poly); free(L.lay); free(L.polys); free(L.stacked);
  if (ts.err) return -2;
  return rc;
}

/* ---------------- verifier (sumcheck/verifier.rs, whir.rs:361-522) ---------------- */
typedef struct {
  int n_eq, n_pow, kfull;
  ext *eq_pts;  /* n_eq x kfull */
  fe *pow_vars; /* n_pow */
  ext rs[64];
  int n_rs;
  ext alpha;
} folding_rounds;

static ext fr_eval(const folding_rounds *f, const ext *poly, int kp) {
  int n = f->n_eq + f->n_pow;
  ext *w = ext_alloc(n);
  for (int i = 0; i < f->n_eq; i++) {
    const ext *z = f->eq_pts + (size_t)i * f->kfull;
    w[i] = ext_mul(eval_eq_xy(z, f->rs, f->n_rs), eval_extp(poly, kp, z + f->n_rs));
  }
  for (int i = 0; i < f->n_pow; i++) {
    fe pt[64];
    fe v = f->pow_vars[i];
    for (int j = 0; j < f->kfull; j++) { pt[j] = v; v = fe_mul(v, v); }
    ext e = eval_univariate(poly, (size_t)1 << kp, ext_from_fe(pt[f->n_rs]));
    w[f->n_eq + i] = ext_mul(eval_pow_xy_f(pt, f->rs, f->n_rs), e);
  }
  ext r = horner(w, n, f->alpha);
  free(w);
  return r;
}

static int reduce_round(wo_ts *ts, ext *sum, ext *r) {
  ext v0 = ts_read_ext(ts, 1), v2 = ts_read_ext(ts, 1);
  *r = ts_draw_ext(ts);
  *sum = extrapolate012(v0, ext_sub(*sum, v0), v2, *r);
  return ts->err ? -1 : 0;
}

int wo_verify(const wo_params *p, const wo_claims *cl, const uint8_t *proof, size_t len,
              uint32_t *checkpoint) {
  if (!stir_counts_ok(p) || !groups_ok(cl) || !sizes_ok(p, cl)) return -1;
  wo_ts ts;
  ts_reader(&ts, proof, len);
  int rc = 0;
  size_t row_len_base = (size_t)1 << p->folding, row_len_ext = row_len_base * 4;
  fe *row = malloc(row_len_ext * sizeof(fe));
  lay_entry *lay = malloc(cl->n_polys * sizeof(lay_entry));
  int k = make_layout(cl->n_polys, cl->poly_k, lay);
  if (k != p->k) { free(lay); free(row); return -1; }
  fe comm[8];
  ts_read_digest(&ts, comm, 1);
  int total = group_offset(cl, cl->n_groups);
  ext *cpts = ext_alloc((size_t)total * 32), *cev = ext_alloc(total);
  int *cpoly = malloc((total ? total : 1) * sizeof(int));
  int nc = 0;
  for (int g = 0; g < cl->n_groups; g++) {
    int o = group_offset(cl, g);
    int kg = cl->poly_k[cl->group_ids[o]];
    ext z = ts_draw_ext(&ts);
    for (int j = 0; j < cl->group_n[g]; j++) {
      expand(cpts + (size_t)nc * 32, kg, z);
      cev[nc] = ts_read_ext(&ts, 1);
      cpoly[nc++] = cl->group_ids[o + j];
    }
  }
  /* claims in layout order, lifted with selector bits (verifier.rs:199-217) */
  int n_ood = wo_n_ood_queries(p->soundness, p->security_level, p->k, p->rate, EXT_BITS);
  int nmax = total + n_ood;
  folding_rounds fr[64];
  int n_fr = 0;
  folding_rounds *f0 = &fr[n_fr++];
  memset(f0, 0, sizeof *f0);
  f0->kfull = k;
  f0->eq_pts = ext_alloc((size_t)nmax * k);
  ext *evals = ext_alloc(nmax);
  int m = 0;
  for (int e = 0; e < cl->n_polys; e++)
    for (int c = 0; c < nc; c++)
      if (cpoly[c] == lay[e].poly) {
        int kp = cl->poly_k[lay[e].poly];
        ext *dst = f0->eq_pts + (size_t)m * k;
        memcpy(dst, cpts + (size_t)c * 32, kp * sizeof(ext));
        for (int b = 0; b < lay[e].nbits; b++) dst[kp + b] = lay[e].bits[b] ? ext_one() : ext_zero();
        evals[m++] = cev[c];
      }
  for (int i = 0; i < n_ood; i++) { /* read_virtual_eval */
    expand(f0->eq_pts + (size_t)m * k, k, ts_draw_ext(&ts));
    evals[m++] = ts_read_ext(&ts, 1);
  }
  f0->n_eq = m;
  ext alpha = ts_draw_ext(&ts);
  f0->alpha = alpha;
  ext sum = horner(evals, m, alpha);
  for (int i = 0; i < p->folding; i++) {
    ext r;
    if (reduce_round(&ts, &sum, &r)) { rc = -2; goto done; }
    f0->rs[f0->n_rs++] = r;
  }
  int kcur = k - p->folding;
  ext round_point[32];
  memcpy(round_point, f0->rs, p->folding * sizeof(ext));
  int n_rounds, final_rounds;
  wo_number_of_rounds(p->folding, p->k, &n_rounds, &final_rounds);
  fe round_comm[8];
  int have_rc = 0;
  size_t idx[4096];
  for (int round = 0; round < n_rounds; round++) {
    int kfd, this_rate, prev_rate;
    round_params(p, round, &kfd, &this_rate, &prev_rate);
    fe rcomm[8];
    ts_read_digest(&ts, rcomm, 1);
    int n_o = wo_n_ood_queries(p->soundness, p->security_level, kcur, this_rate, EXT_BITS);
    folding_rounds *f = &fr[n_fr];
    memset(f, 0, sizeof *f);
    f->kfull = kcur;
    ext *oev = ext_alloc(n_o + 4096);
    f->eq_pts = ext_alloc((size_t)(n_o ? n_o : 1) * kcur);
    for (int i = 0; i < n_o; i++) {
      ext z = ts_draw_ext(&ts);
      oev[i] = ts_read_ext(&ts, 1);
      expand(f->eq_pts + (size_t)i * kcur, kcur, z);
    }
    f->n_eq = n_o;
    int n_s = wo_n_stir_queries(p->soundness, p->security_level, prev_rate);
    int mm = stir_indexes(&ts, kfd, n_s, idx);
    fe omega = fe_two_adic(kfd);
    f->pow_vars = malloc((mm ? mm : 1) * sizeof(fe));
    for (int i = 0; i < mm; i++) {
      ext e;
      if (round == 0) {
        if (tree_verify(&ts, comm, idx[i], row_len_base, kfd, row)) { rc = -3; goto done; }
        e = eval_base(row, p->folding, round_point);
      } else {
        if (tree_verify(&ts, round_comm, idx[i], row_len_ext, kfd, row)) { rc = -3; goto done; }
        e = eval_extp((const ext *)row, p->folding, round_point);
      }
      f->pow_vars[i] = fe_pow(omega, idx[i]);
      oev[n_o + i] = e;
    }
    f->n_pow = mm;
    memcpy(round_comm, rcomm, 32);
    have_rc = 1;
    /* SumcheckVerifier::fold (verifier.rs:262-306) */
    ext a = ts_draw_ext(&ts);
    f->alpha = a;
    sum = ext_add(sum, horner(oev, n_o + mm, a));
    free(oev);
    ext rsn[32];
    for (int i = 0; i < p->folding; i++)
      if (reduce_round(&ts, &sum, &rsn[i])) { rc = -2; goto done; }
    for (int j = 0; j < n_fr; j++)
      for (int i = 0; i < p->folding; i++) fr[j].rs[fr[j].n_rs++] = rsn[i];
    for (int i = 0; i < p->folding; i++) f->rs[f->n_rs++] = rsn[i];
    n_fr++;
    kcur -= p->folding;
    memcpy(round_point, rsn, p->folding * sizeof(ext));
  }
  if (kcur != final_rounds) { rc = -4; goto done; }
  {
    size_t nf = (size_t)1 << kcur;
    ext *fp = ext_alloc(nf);
    for (size_t i = 0; i < nf; i++) fp[i] = ts_read_ext(&ts, 1);
    int kfd, this_rate, prev_rate;
    round_params(p, n_rounds, &kfd, &this_rate, &prev_rate);
    int n_s = wo_n_stir_queries(p->soundness, p->security_level, prev_rate);
    int mm = stir_indexes(&ts, kfd, n_s, idx);
    fe omega = fe_two_adic(kfd);
    for (int i = 0; i < mm && !rc; i++) {
      ext e;
      if (have_rc) {
        if (tree_verify(&ts, round_comm, idx[i], row_len_ext, kfd, row)) { rc = -3; break; }
        e = eval_extp((const ext *)row, p->folding, round_point);
      } else {
        if (tree_verify(&ts, comm, idx[i], row_len_base, kfd, row)) { rc = -3; break; }
        e = eval_base(row, p->folding, round_point);
      }
      ext want = eval_univariate(fp, nf, ext_from_fe(fe_pow(omega, idx[i])));
      if (!ext_eq(e, want)) rc = -5;
    }
    if (!rc) { /* SumcheckVerifier::finalize (verifier.rs:308-323) */
      ext tot = ext_zero();
      for (int j = 0; j < n_fr; j++) tot = ext_add(tot, fr_eval(&fr[j], fp, kcur));
      if (!ext_eq(tot, sum)) rc = -6;
    }
    free(fp);
  }
  if (!rc) *checkpoint = ts_draw_fe(&ts);
  if (!rc && ts.err) rc = -7;
done:
  for (int j = 0; j < n_fr; j++) { free(fr[j].eq_pts); free(fr[j].pow_vars); }
  free(row); free(lay); free(cpts); free(cev); free(cpoly); free(evals);
  return rc;
}
