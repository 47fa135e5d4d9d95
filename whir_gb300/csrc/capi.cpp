// extern "C" boundary (include/whir_gb300.h): argument checks, exception to
// status-code translation, and the kernel-level entry points.
#include "../../include/whir_gb300.h"

#include <string.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <memory>
#include <mutex>
#include <thread>

#include <new>
#include <string>
#include <vector>

#include "kernels.h"
#include "poseidon2_host.h"
#include "batch.h"
#include "batch_prover.h"
#include "debug.h"
#include "prover.h"
#include "tune.h"
#include "verifier.h"
#include "verify_batch.h"
#include "transcript.h"

using whir::Context;
using whir::DeviceBuffer;
using whir::WhirError;
using kb::E4;

struct whir_ctx {
  Context ctx;
  DeviceBuffer scratch, eq, acc, small;
  // the node buffer of the last freed tree, reused by the next commit (a
  // fresh reservation and its release cost ~0.3 ms at 2^21 leaves)
  std::unique_ptr<DeviceBuffer> spare_nodes;
  std::mutex spare_mu;
  std::unique_ptr<whir::BatchProver> batch;  // whir_prove_batch's prover, made on first use
  std::unique_ptr<whir::BatchVerifier> verifier;  // whir_verify_batch's, made on first use
  explicit whir_ctx(int dev) : ctx(dev) {}
};
struct whir_transcript {
  whir::Transcript t;
};
struct whir_prover {
  whir_ctx *ctx;
  whir::Prover p;
  whir_prover(whir_ctx *c, const whir::Params &prm) : ctx(c), p(&c->ctx, prm) {}
};
struct whir_tree {
  whir_ctx *ctx;
  std::unique_ptr<DeviceBuffer> nodes;
  whir::DeviceTree t;
};

static thread_local std::string g_err;

#define API_BEGIN try {
#define API_END                                          \
  return WHIR_OK;                                        \
  }                                                      \
  catch (const WhirError &e) {                           \
    g_err = e.what();                                    \
    return e.code == -2 ? WHIR_ERR_CUDA                  \
           : e.code == -3 ? WHIR_ERR_NOMEM               \
           : e.code == -4 ? WHIR_ERR_CAPACITY            \
                          : WHIR_ERR_ARG;                \
  }                                                      \
  catch (const std::bad_alloc &) {                       \
    g_err = "host allocation failed";                    \
    return WHIR_ERR_NOMEM;                               \
  }                                                      \
  catch (const std::exception &e) {                      \
    g_err = e.what();                                    \
    return WHIR_ERR_INTERNAL;                            \
  }

// error text for entry points defined outside this file
void whir_record_error(const char *msg) { g_err = msg; }

static void need(bool ok, const char *what) {
  if (!ok) throw WhirError(-1, what);
}
static E4 ext_in(const uint32_t *v) {
  E4 e;
  for (int i = 0; i < 4; i++) e.c[i] = v[i];
  for (int i = 0; i < 4; i++) need(v[i] < kb::P, "non-canonical field element");
  return e;
}
static void ext_out(const E4 &e, uint32_t *v) { memcpy(v, e.c, 16); }
static whir::gpu::Point point_in(const uint32_t *pt, int k) {
  need(k >= 0 && k <= whir::gpu::MAX_VARS, "point has too many variables");
  need(pt != nullptr || k == 0, "null point");
  whir::gpu::Point z;
  z.k = k;
  for (int i = 0; i < k; i++) z.z[i] = ext_in(pt + 4 * i);
  return z;
}
static unsigned long long *acc_buf(whir_ctx *c, size_t words) {
  c->acc.reserve(8 * words);
  unsigned long long *a = c->acc.as<unsigned long long>();
  whir::cuda_check(cudaMemsetAsync(a, 0, 8 * words, c->ctx.stream()), "memset");
  return a;
}
static void read_acc(whir_ctx *c, unsigned long long *a, size_t words, uint32_t *out) {
  std::vector<unsigned long long> h(words);
  whir::cuda_check(cudaMemcpyAsync(h.data(), a, 8 * words, cudaMemcpyDeviceToHost, c->ctx.stream()),
                   "d2h");
  c->ctx.sync();
  for (size_t i = 0; i < words; i++) out[i] = (uint32_t)(h[i] % kb::P);
}

extern "C" {

const char *whir_last_error(void) { return g_err.c_str(); }

int whir_ctx_create(int device, whir_ctx **out) {
  API_BEGIN
  need(out != nullptr, "null out");
  *out = new whir_ctx(device);
  API_END
}
int whir_ctx_destroy(whir_ctx *ctx) {
  API_BEGIN
  delete ctx;
  API_END
}
int whir_ctx_stream(whir_ctx *ctx, void **stream) {
  API_BEGIN
  need(ctx && stream, "null argument");
  *stream = (void *)ctx->ctx.stream();
  API_END
}
int whir_device_alloc(whir_ctx *ctx, size_t bytes, void **out) {
  API_BEGIN
  need(ctx && out, "null argument");
  cudaError_t e = cudaMalloc(out, bytes ? bytes : 16);
  if (e != cudaSuccess) throw WhirError(-3, cudaGetErrorString(e));
  API_END
}
int whir_device_free(whir_ctx *ctx, void *ptr) {
  API_BEGIN
  need(ctx != nullptr, "null context");
  ctx->ctx.sync();
  whir::cuda_check(cudaFree(ptr), "cudaFree");
  API_END
}
int whir_copy_to_device(whir_ctx *ctx, void *dst, const void *src, size_t bytes) {
  API_BEGIN
  need(ctx && dst && src, "null argument");
  whir::cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->ctx.stream()),
                   "h2d");
  ctx->ctx.sync();
  API_END
}
int whir_copy_to_host(whir_ctx *ctx, void *dst, const void *src, size_t bytes) {
  API_BEGIN
  need(ctx && dst && src, "null argument");
  whir::cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->ctx.stream()),
                   "d2h");
  ctx->ctx.sync();
  API_END
}

int whir_dft_batch(whir_ctx *ctx, const uint32_t *in, size_t h_in, size_t width, int log_h,
                   uint32_t *out) {
  API_BEGIN
  need(ctx && in && out, "null argument");
  need(log_h >= 0 && log_h <= 24, "log_h must be in [0, 24] (two-adicity of KoalaBear)");
  need(width > 0 && h_in <= ((size_t)1 << log_h), "bad matrix shape");
  if (log_h > 11) ctx->scratch.reserve(4 * (width << log_h));
  whir::cuda_check(whir::gpu::dft_batch(in, h_in, width, log_h, out,
                                        log_h > 11 ? ctx->scratch.as<uint32_t>() : nullptr,
                                        ctx->ctx.stream()),
                   "dft_batch");
  ctx->ctx.sync();
  API_END
}

int whir_merkle_commit(whir_ctx *ctx, const uint32_t *rows, int log_h, size_t row_len,
                       whir_tree **out, uint32_t root[8]) {
  API_BEGIN
  need(ctx && rows && out && root, "null argument");
  need(log_h >= 0 && log_h <= 30 && row_len > 0 && row_len < (1u << 20), "bad tree shape");
  whir_tree *t = new whir_tree();
  t->ctx = ctx;
  try {
    {
      std::lock_guard<std::mutex> lock(ctx->spare_mu);
      t->nodes = std::move(ctx->spare_nodes);
    }
    if (!t->nodes) t->nodes.reset(new DeviceBuffer());
    t->nodes->reserve(4 * whir::gpu::tree_words(log_h));
    cudaStream_t st = ctx->ctx.stream();
    size_t n = (size_t)1 << log_h;
    whir::cuda_check(whir::gpu::hash_rows(rows, n, (int)row_len, t->nodes->as<uint32_t>(), st),
                     "hash_rows");
    whir::cuda_check(whir::gpu::build_tree(t->nodes->as<uint32_t>(), log_h, st), "build_tree");
    uint32_t h[8];
    whir::cuda_check(cudaMemcpyAsync(h, t->nodes->as<uint32_t>() + whir::gpu::tree_words(log_h) - 8,
                                     32, cudaMemcpyDeviceToHost, st),
                     "d2h");
    ctx->ctx.sync();
    t->t.rows = rows;
    t->t.nodes = t->nodes->as<uint32_t>();
    t->t.log_h = log_h;
    t->t.row_len = (int)row_len;
    memcpy(t->t.root, h, 32);
    memcpy(root, h, 32);
  } catch (...) {
    delete t;
    throw;
  }
  *out = t;
  API_END
}
int whir_merkle_levels(whir_tree *tree, uint32_t *out) {
  API_BEGIN
  need(tree && out, "null argument");
  size_t words = whir::gpu::tree_words(tree->t.log_h);
  whir::cuda_check(cudaMemcpyAsync(out, tree->t.nodes, 4 * words, cudaMemcpyDeviceToHost,
                                   tree->ctx->ctx.stream()),
                   "d2h");
  tree->ctx->ctx.sync();
  API_END
}
int whir_merkle_open(whir_tree *tree, const size_t *idx, size_t n, uint32_t *out) {
  API_BEGIN
  need(tree && (idx || !n) && (out || !n), "null argument");
  if (!n) return WHIR_OK;
  whir_ctx *c = tree->ctx;
  size_t h = (size_t)1 << tree->t.log_h;
  std::vector<uint32_t> i32(n);
  for (size_t i = 0; i < n; i++) {
    need(idx[i] < h, "query index out of range");
    i32[i] = (uint32_t)idx[i];
  }
  size_t per = (size_t)tree->t.row_len + 8 * (size_t)tree->t.log_h;
  c->small.reserve(4 * n + 4 * per * n);
  uint32_t *d = c->small.as<uint32_t>();
  cudaStream_t st = c->ctx.stream();
  whir::cuda_check(cudaMemcpyAsync(d, i32.data(), 4 * n, cudaMemcpyHostToDevice, st), "h2d");
  whir::cuda_check(whir::gpu::gather_openings(tree->t.rows, tree->t.row_len, tree->t.nodes,
                                              tree->t.log_h, d, (int)n, d + n, st),
                   "gather");
  whir::cuda_check(cudaMemcpyAsync(out, d + n, 4 * per * n, cudaMemcpyDeviceToHost, st), "d2h");
  c->ctx.sync();
  API_END
}
int whir_merkle_free(whir_tree *tree) {
  API_BEGIN
  if (tree) {
    whir_ctx *c = tree->ctx;
    c->ctx.sync();
    std::lock_guard<std::mutex> lock(c->spare_mu);
    if (tree->nodes && (!c->spare_nodes || c->spare_nodes->bytes() < tree->nodes->bytes()))
      c->spare_nodes = std::move(tree->nodes);
  }
  delete tree;
  API_END
}

int whir_eq_table(whir_ctx *ctx, const uint32_t *point, int k, const uint32_t scale[4],
                  uint32_t *out) {
  API_BEGIN
  need(ctx && out && scale, "null argument");
  need(k <= 24, "k too large");
  whir::gpu::Point z = point_in(point, k);
  ctx->eq.reserve(sizeof(E4) * (((size_t)1 << (k / 2)) + ((size_t)1 << (k - k / 2))));
  whir::cuda_check(whir::gpu::eq_full(z, ext_in(scale), reinterpret_cast<E4 *>(out),
                                      ctx->eq.as<E4>(), ctx->ctx.stream()),
                   "eq_full");
  ctx->ctx.sync();
  API_END
}

int whir_compress_hi(whir_ctx *ctx, const uint32_t *poly, int k, const uint32_t *point, int kz,
                     uint32_t *out) {
  API_BEGIN
  need(ctx && poly && out, "null argument");
  need(kz >= 0 && kz <= k && k - kz <= 8, "compress_hi keeps at most 8 variables");
  whir::gpu::Point z = point_in(point, kz);
  int ks = k - kz;
  int s_lo = kz < 10 ? kz : 10;
  ctx->eq.reserve(sizeof(E4) * (((size_t)1 << s_lo) + ((size_t)1 << (kz - s_lo))));
  E4 *lo = ctx->eq.as<E4>(), *hi = lo + ((size_t)1 << s_lo);
  cudaStream_t st = ctx->ctx.stream();
  whir::cuda_check(whir::gpu::eq_split(z, s_lo, kb::e_one(), lo, hi, st), "eq_split");
  size_t words = (size_t)4 << ks;
  unsigned long long *a = acc_buf(ctx, words);
  whir::cuda_check(whir::gpu::compress_hi(poly, k, ks, lo, s_lo, hi, a, st), "compress_hi");
  read_acc(ctx, a, words, out);
  API_END
}

int whir_compress_lo(whir_ctx *ctx, const uint32_t *poly, int k, const uint32_t *point, int kz,
                     uint32_t *out) {
  API_BEGIN
  need(ctx && poly && out, "null argument");
  need(kz >= 0 && kz <= k && kz <= 8, "compress_lo fixes at most 8 variables");
  whir::gpu::Point z = point_in(point, kz);
  whir::cuda_check(whir::gpu::compress_lo(poly, k, z, reinterpret_cast<E4 *>(out),
                                          ctx->ctx.stream()),
                   "compress_lo");
  ctx->ctx.sync();
  API_END
}

int whir_eval_ext(whir_ctx *ctx, const uint32_t *poly, int k, const uint32_t *point,
                  uint32_t out[4]) {
  API_BEGIN
  need(ctx && poly && out, "null argument");
  need(k >= 0 && k <= 30, "bad k");
  whir::gpu::Point z = point_in(point, k);
  int s_lo = k < 10 ? k : 10;
  ctx->eq.reserve(sizeof(E4) * (((size_t)1 << s_lo) + ((size_t)1 << (k - s_lo))));
  E4 *lo = ctx->eq.as<E4>(), *hi = lo + ((size_t)1 << s_lo);
  cudaStream_t st = ctx->ctx.stream();
  whir::cuda_check(whir::gpu::eq_split(z, s_lo, kb::e_one(), lo, hi, st), "eq_split");
  unsigned long long *a = acc_buf(ctx, 4);
  whir::cuda_check(whir::gpu::eval_ext(reinterpret_cast<const E4 *>(poly), k, lo, s_lo, hi, a, st),
                   "eval_ext");
  read_acc(ctx, a, 4, out);
  API_END
}

int whir_sumcheck_coeffs(whir_ctx *ctx, const uint32_t *poly, const uint32_t *weights, int k,
                         uint32_t c0[4], uint32_t c2[4]) {
  API_BEGIN
  need(ctx && poly && weights && c0 && c2, "null argument");
  need(k >= 1 && k <= 30, "coeffs needs k >= 1");
  unsigned long long *a = acc_buf(ctx, 8);
  whir::cuda_check(whir::gpu::sumcheck_round(reinterpret_cast<const E4 *>(poly),
                                             reinterpret_cast<const E4 *>(weights),
                                             (size_t)1 << k, false, kb::e_zero(), nullptr,
                                             nullptr, true, a, ctx->ctx.stream()),
                   "round");
  uint32_t h[8];
  read_acc(ctx, a, 8, h);
  memcpy(c0, h, 16);
  memcpy(c2, h + 4, 16);
  API_END
}

int whir_sumcheck_fold(whir_ctx *ctx, const uint32_t *poly, const uint32_t *weights, int k,
                       const uint32_t r[4], uint32_t *poly_out, uint32_t *weights_out) {
  API_BEGIN
  need(ctx && poly && weights && r && poly_out && weights_out, "null argument");
  need(k >= 1 && k <= 30, "fold needs k >= 1");
  whir::cuda_check(whir::gpu::sumcheck_round(reinterpret_cast<const E4 *>(poly),
                                             reinterpret_cast<const E4 *>(weights),
                                             (size_t)1 << k, true, ext_in(r),
                                             reinterpret_cast<E4 *>(poly_out),
                                             reinterpret_cast<E4 *>(weights_out), false, nullptr,
                                             ctx->ctx.stream()),
                   "fold");
  ctx->ctx.sync();
  API_END
}

int whir_combine_eqs(whir_ctx *ctx, uint32_t *weights, int k, const uint32_t *points, int n,
                     const uint32_t alpha[4]) {
  API_BEGIN
  need(ctx && weights && alpha && (points || !n) && n >= 0, "bad argument");
  need(k >= 0 && k <= 24, "bad k");
  if (n == 0) return WHIR_OK;
  E4 a = ext_in(alpha), s = kb::e_one();
  int sl = k / 2;
  size_t per = ((size_t)1 << sl) + ((size_t)1 << (k - sl));
  ctx->eq.reserve(sizeof(E4) * per * n);
  cudaStream_t st = ctx->ctx.stream();
  for (int t = 0; t < n; t++) {
    whir::gpu::Point z = point_in(points + (size_t)4 * k * t, k);
    E4 *tab = ctx->eq.as<E4>() + per * t;
    whir::cuda_check(whir::gpu::eq_split(z, sl, s, tab, tab + ((size_t)1 << sl), st), "eq_split");
    s = kb::e_mul(s, a);
  }
  whir::cuda_check(whir::gpu::add_eq(reinterpret_cast<E4 *>(weights), k, ctx->eq.as<E4>(), n, st),
                   "add_eq");
  ctx->ctx.sync();
  API_END
}

static void combine_pows_impl(whir_ctx *ctx, uint32_t *weights, int k, const uint32_t *vars, int n,
                              const std::vector<E4> &scales) {
  for (int i = 0; i < n; i++) need(vars[i] < kb::P, "non-canonical field element");
  size_t bytes = 16 * (size_t)n + 4 * (size_t)n;
  ctx->small.reserve(bytes);
  std::vector<uint8_t> h(bytes);
  memcpy(h.data(), scales.data(), 16 * (size_t)n);
  memcpy(h.data() + 16 * (size_t)n, vars, 4 * (size_t)n);
  cudaStream_t st = ctx->ctx.stream();
  whir::cuda_check(cudaMemcpyAsync(ctx->small.as<uint8_t>(), h.data(), bytes,
                                   cudaMemcpyHostToDevice, st),
                   "h2d");
  ctx->eq.reserve(4 * whir::gpu::add_pows_scratch_words(k, n));
  whir::cuda_check(whir::gpu::add_pows(reinterpret_cast<E4 *>(weights), k,
                                       reinterpret_cast<const uint32_t *>(ctx->small.as<uint8_t>() +
                                                                          16 * (size_t)n),
                                       ctx->small.as<E4>(), n, ctx->eq.as<uint32_t>(), st),
                   "add_pows");
  ctx->ctx.sync();
}

int whir_combine_pows(whir_ctx *ctx, uint32_t *weights, int k, const uint32_t *vars, int n,
                      const uint32_t alpha[4], int shift) {
  API_BEGIN
  need(ctx && weights && alpha && (vars || !n) && n >= 0 && shift >= 0, "bad argument");
  need(k >= 0 && k <= 30, "bad k");
  if (n == 0) return WHIR_OK;
  E4 a = ext_in(alpha);
  std::vector<E4> sc(n);
  E4 s = kb::e_pow(a, (uint64_t)shift);
  for (int i = 0; i < n; i++) {
    sc[i] = s;
    s = kb::e_mul(s, a);
  }
  combine_pows_impl(ctx, weights, k, vars, n, sc);
  API_END
}

int whir_combine_pows_scaled(whir_ctx *ctx, uint32_t *weights, int k, const uint32_t *vars,
                             int n, const uint32_t *scales) {
  API_BEGIN
  need(ctx && weights && (vars || !n) && (scales || !n) && n >= 0, "bad argument");
  need(k >= 0 && k <= 30, "bad k");
  if (n == 0) return WHIR_OK;
  std::vector<E4> sc(n);
  for (int i = 0; i < n; i++) sc[i] = ext_in(scales + 4 * i);
  combine_pows_impl(ctx, weights, k, vars, n, sc);
  API_END
}

int whir_fold_code_rounds(whir_ctx *ctx, const uint32_t *codeword, int k_data, int folding,
                          const size_t *idx, int n, const uint32_t *scales, const uint32_t *rs,
                          const uint32_t *r, uint32_t *out) {
  API_BEGIN
  need(ctx && codeword && out && rs && (r || folding <= 1), "null argument");
  need(folding >= 1 && folding <= 8 && k_data >= folding && k_data <= 24, "bad shape");
  need(n >= 1 && idx && scales, "no queries");
  const int d = folding, lS = k_data - d;
  const size_t S = (size_t)1 << lS, T = (size_t)1 << d;
  for (int i = 0; i < n; i++) need(idx[i] < ((size_t)1 << k_data), "index out of range");
  whir::gpu::Point rsp = point_in(rs, d);
  std::vector<E4> rr(d > 1 ? d - 1 : 0);
  for (int i = 0; i + 1 < d; i++) rr[i] = ext_in(r + 4 * i);
  // device state (Prover's fold_with_code layout): G | scales | idx | ws | tw | B | wd | rows
  const size_t un = (size_t)n;
  std::vector<uint32_t> hrows(un * T), hidx(un), hwd(T);
  std::vector<E4> hsc(un);
  for (size_t i = 0; i < un; i++) {
    hidx[i] = (uint32_t)idx[i];
    hsc[i] = ext_in(scales + 4 * i);
    for (size_t t = 0; t < T; t++) hrows[i * T + t] = (uint32_t)((idx[i] & (S - 1)) + t * S);
  }
  whir::gpu::CodeState cs;
  cs.n = n;
  cs.d = d;
  cs.k_data = k_data;
  cs.omega = whir::two_adic_generator(k_data);
  cs.winv = kb::inv(cs.omega);
  cs.two_inv = kb::inv(kb::from_canonical(2));
  const uint32_t wdv = kb::pow(cs.winv, S);
  hwd[0] = kb::ONE;
  for (size_t t = 1; t < T; t++) hwd[t] = kb::mul(hwd[t - 1], wdv);
  const size_t words = 4 * un * T + 4 * un + 5 * un + T + un * T;
  ctx->scratch.reserve(4 * words + 64);
  uint32_t *base = ctx->scratch.as<uint32_t>();
  cs.G = reinterpret_cast<E4 *>(base);
  cs.scales = reinterpret_cast<E4 *>(base + 4 * un * T);
  uint32_t *u = base + 4 * un * T + 4 * un;
  cs.idx = u;
  cs.ws = u + un;
  cs.tw = u + 2 * un;
  cs.B = u + 3 * un;
  uint32_t *dwd = u + 4 * un, *drows = dwd + T;
  cs.wd = dwd;
  cudaStream_t st = ctx->ctx.stream();
  whir::cuda_check(cudaMemcpyAsync(const_cast<uint32_t *>(cs.idx), hidx.data(), 4 * un,
                                   cudaMemcpyHostToDevice, st), "h2d");
  whir::cuda_check(cudaMemcpyAsync(cs.scales, hsc.data(), 16 * un, cudaMemcpyHostToDevice, st), "h2d");
  whir::cuda_check(cudaMemcpyAsync(dwd, hwd.data(), 4 * T, cudaMemcpyHostToDevice, st), "h2d");
  whir::cuda_check(cudaMemcpyAsync(drows, hrows.data(), 4 * un * T, cudaMemcpyHostToDevice, st),
                   "h2d");
  // G_0: the 2^d rows of each query's recursion at eq(rs) (prover.rs:497-506)
  whir::cuda_check(whir::gpu::row_evals(codeword, (int)T, drows, (int)(un * T), rsp, cs.G, st),
                   "row_evals");
  unsigned long long *a = acc_buf(ctx, 12);
  for (int round = 0; round < d; round++) {
    whir::cuda_check(whir::gpu::code_round(cs, round, round ? rr[round - 1] : kb::e_zero(), a, st),
                     "code_round");
    uint32_t got[12];
    read_acc(ctx, a, 12, got);
    memcpy(out + 8 * round, got, 32);
    if (round == 0) memcpy(out + 8 * d, got + 8, 16);
    whir::cuda_check(cudaMemsetAsync(a, 0, 8 * 12, st), "memset");
  }
  ctx->ctx.sync();
  API_END
}

int whir_debug_set(unsigned flags) {
  API_BEGIN
  need((flags & ~7u) == 0, "unknown debug flags");
  whir::set_debug(flags);
  API_END
}

int whir_poseidon2_permute(int width, uint32_t *state) {
  API_BEGIN
  need(state != nullptr, "null state");
  need(width == 16 || width == 24, "width must be 16 or 24");
  for (int i = 0; i < width; i++) need(state[i] < kb::P, "non-canonical field element");
  whir::poseidon2_permute_host(whir::poseidon2_constants(width), state);
  API_END
}

int whir_random_field(uint64_t seed, uint32_t *out, size_t n) {
  API_BEGIN
  need(out != nullptr || n == 0, "null out");
  whir::std_rng_fill_field(seed, out, n);
  API_END
}

int whir_transcript_new(whir_transcript **out) {
  API_BEGIN
  need(out != nullptr, "null out");
  *out = new whir_transcript();
  API_END
}
int whir_transcript_free(whir_transcript *t) {
  API_BEGIN
  delete t;
  API_END
}
int whir_transcript_write(whir_transcript *t, const uint32_t e[4]) {
  API_BEGIN
  need(t && e, "null argument");
  t->t.write_ext(ext_in(e));
  API_END
}
int whir_transcript_write_base(whir_transcript *t, uint32_t v) {
  API_BEGIN
  need(t != nullptr, "null transcript");
  need(v < kb::P, "non-canonical field element");
  t->t.write_fe(v);
  API_END
}
int whir_transcript_draw(whir_transcript *t, uint32_t out[4]) {
  API_BEGIN
  need(t && out, "null argument");
  ext_out(t->t.draw_ext(), out);
  API_END
}
int whir_transcript_draw_base(whir_transcript *t, uint32_t *out) {
  API_BEGIN
  need(t && out, "null argument");
  *out = t->t.draw_fe();
  API_END
}
int whir_transcript_draw_bits(whir_transcript *t, int bits, size_t *out) {
  API_BEGIN
  need(t && out, "null argument");
  need(bits >= 0 && bits < 31, "bits must satisfy 2^bits < p");
  *out = t->t.draw_bits(bits);
  API_END
}
int whir_transcript_size(whir_transcript *t, size_t *len) {
  API_BEGIN
  need(t && len, "null argument");
  *len = t->t.bytes().size();
  API_END
}
int whir_transcript_bytes(whir_transcript *t, uint8_t *out, size_t cap) {
  API_BEGIN
  need(t && (out || !cap), "null argument");
  const auto &b = t->t.bytes();
  if (b.size() > cap) throw WhirError(-4, "proof buffer too small");
  memcpy(out, b.data(), b.size());
  API_END
}

int whir_prover_new(whir_ctx *ctx, const whir_params *params, whir_prover **out) {
  API_BEGIN
  need(ctx && params && out, "null argument");
  whir::Params p{params->k,         params->folding,   params->rate,
                 params->initial_reduction, params->soundness, params->security_level};
  *out = new whir_prover(ctx, p);
  API_END
}
int whir_prover_free(whir_prover *p) {
  API_BEGIN
  if (p) p->ctx->ctx.sync();
  delete p;
  API_END
}
static std::vector<int> ks_in(const int32_t *poly_k, int n_polys) {
  need(poly_k && n_polys > 0 && n_polys < (1 << 20), "bad polynomial list");
  std::vector<int> v(poly_k, poly_k + n_polys);
  for (int k : v) need(k >= 0 && k <= 30, "bad polynomial size");
  return v;
}
int whir_commit(whir_prover *p, whir_transcript *t, const uint32_t *polys, int on_device,
                const int32_t *poly_k, int n_polys) {
  API_BEGIN
  need(p && t && polys, "null argument");
  std::vector<int> ks = ks_in(poly_k, n_polys);
  p->p.commit(t->t, polys, on_device != 0, ks);
  API_END
}
int whir_stack_eval(whir_prover *p, whir_transcript *t, int id, const uint32_t *point,
                    uint32_t eval[4]) {
  API_BEGIN
  need(p && t && point && eval, "null argument");
  need(id >= 0, "bad id");
  ext_out(p->p.eval(t->t, id, reinterpret_cast<const E4 *>(point)), eval);
  API_END
}
int whir_open(whir_prover *p, whir_transcript *t) {
  API_BEGIN
  need(p && t, "null argument");
  p->p.open(t->t);
  API_END
}
int whir_prove(whir_prover *p, whir_transcript *t, const uint32_t *polys, int on_device,
               const int32_t *poly_k, int n_polys, const int32_t *group_n, int n_groups,
               const int32_t *group_ids) {
  API_BEGIN
  need(p && t && polys, "null argument");
  std::vector<int> ks = ks_in(poly_k, n_polys);
  need(n_groups >= 0 && (group_n || !n_groups), "bad claim groups");
  std::vector<std::vector<int>> groups;
  size_t off = 0;
  for (int g = 0; g < n_groups; g++) {
    need(group_n[g] > 0, "empty claim group");
    std::vector<int> ids(group_ids + off, group_ids + off + group_n[g]);
    for (int id : ids) need(id >= 0 && id < n_polys, "claim id out of range");
    off += group_n[g];
    groups.push_back(ids);
  }
  p->p.prove(t->t, polys, on_device != 0, ks, groups);
  API_END
}

static whir::Params params_in(const whir_params *q) {
  need(q != nullptr, "null parameters");
  return whir::Params{q->k, q->folding, q->rate, q->initial_reduction, q->soundness,
                      q->security_level};
}

int whir_prove_batch(whir_ctx *ctx, const whir_params *params, const uint32_t *const *polys,
                     int on_device, int batch, int n_claims, int commit_only, uint8_t *proofs,
                     size_t proof_cap, size_t *proof_len, uint32_t *checkpoints) {
  API_BEGIN
  need(ctx && polys && proof_len && checkpoints, "null argument");
  need(proof_cap == 0 || proofs != nullptr, "proof buffer missing");
  need(n_claims >= 0 && n_claims <= 64, "claims per instance out of range");
  whir::Params p = params_in(params);
  need(batch >= 1 && batch <= whir::BatchProver::max_batch(p), "batch size out of range");
  for (int b = 0; b < batch; b++) need(polys[b] != nullptr, "null polynomial");
  if (!ctx->batch)
    ctx->batch.reset(new whir::BatchProver(&ctx->ctx, p, (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
  else
    ctx->batch->set_params(p);
  std::vector<whir::Transcript> ts(batch);
  std::vector<whir::Transcript *> tp(batch);
  std::vector<const uint32_t *> pp(polys, polys + batch);
  for (int b = 0; b < batch; b++) tp[b] = &ts[b];
  // each instance's read-out runs on the prover's host pool
  ctx->batch->prove(tp, pp, on_device != 0, n_claims, commit_only != 0, [&](int b) {
    checkpoints[b] = ts[b].draw_fe();
    const std::vector<uint8_t> &bytes = ts[b].bytes();
    proof_len[b] = bytes.size();
    if (proof_cap)
      memcpy(proofs + (size_t)b * proof_cap, bytes.data(), std::min(proof_cap, bytes.size()));
  });
  API_END
}

int whir_batch_max(const whir_params *params, int32_t *max_batch) {
  API_BEGIN
  need(max_batch != nullptr, "null argument");
  *max_batch = whir::BatchProver::max_batch(params_in(params));
  API_END
}

struct whir_server {
  whir::Server s;
  whir_server(int device, int workers, size_t budget) : s(device, workers, budget) {}
};

static void run_on(whir::Server &srv, whir_job *jobs, int n_jobs, whir_run_stats *stats,
                   bool honor_arrival) {
  need(n_jobs >= 0 && (jobs || n_jobs == 0), "bad job list");
  std::vector<whir::Job> js(n_jobs);
  for (int i = 0; i < n_jobs; i++) {
    const whir_job &q = jobs[i];
    need(q.poly != nullptr, "job without a polynomial");
    need(q.proof_cap == 0 || q.proof != nullptr, "proof buffer missing");
    js[i].params = params_in(&q.params);
    js[i].poly = q.poly;
    js[i].on_device = q.poly_on_device != 0;
    js[i].n_claims = q.commit_only ? 0 : q.n_claims;
    js[i].commit_only = q.commit_only != 0;
    js[i].arrival = honor_arrival ? q.arrival_s : 0.0;
  }
  whir::RunStats rs = srv.run(js, honor_arrival);
  for (int i = 0; i < n_jobs; i++) {
    whir_job &q = jobs[i];
    const whir::Job &j = js[i];
    q.proof_len = j.proof.size();
    if (q.proof) memcpy(q.proof, j.proof.data(), std::min(q.proof_cap, j.proof.size()));
    q.checkpoint = j.checkpoint;
    q.status = j.status == 0 ? WHIR_OK
               : j.status == -2 ? WHIR_ERR_CUDA
               : j.status == -3 ? WHIR_ERR_NOMEM
               : j.status == -4 ? WHIR_ERR_CAPACITY
               : j.status == -5 ? WHIR_ERR_INTERNAL
                                : WHIR_ERR_ARG;
    q.worker = j.worker;
    q.start_s = j.start;
    q.done_s = j.done;
  }
  if (stats) {
    stats->seconds = rs.seconds;
    stats->peak_device_bytes = rs.peak_bytes;
  }
}

int whir_server_new(int device, int n_workers, uint64_t budget, whir_server **out) {
  API_BEGIN
  need(out != nullptr, "null argument");
  need(n_workers >= 1 && n_workers <= 256, "workers out of range");
  *out = new whir_server(device, n_workers, (size_t)budget);
  API_END
}
int whir_server_run(whir_server *s, whir_job *jobs, int n_jobs, int honor_arrival,
                    whir_run_stats *stats) {
  API_BEGIN
  need(s != nullptr, "null server");
  run_on(s->s, jobs, n_jobs, stats, honor_arrival != 0);
  API_END
}
int whir_server_set_lockstep(whir_server *s, int max_group) {
  API_BEGIN
  need(s != nullptr && max_group >= 0, "bad argument");
  s->s.set_lockstep(max_group);
  API_END
}
int whir_server_free(whir_server *s) {
  API_BEGIN
  delete s;
  API_END
}

int whir_batch_prove(int device, whir_job *jobs, int n_jobs, int n_workers, uint64_t budget,
                     whir_run_stats *stats) {
  API_BEGIN
  need(n_workers >= 1 && n_workers <= 256, "workers out of range");
  whir::Server srv(device, n_workers, (size_t)budget);
  run_on(srv, jobs, n_jobs, stats, false);
  API_END
}
int whir_serve(int device, whir_job *jobs, int n_jobs, int n_workers, uint64_t budget,
               whir_run_stats *stats) {
  API_BEGIN
  need(n_workers >= 1 && n_workers <= 256, "workers out of range");
  whir::Server srv(device, n_workers, (size_t)budget);
  run_on(srv, jobs, n_jobs, stats, true);
  API_END
}

int whir_workspace_bytes(const whir_params *params, uint64_t *bytes) {
  API_BEGIN
  need(bytes != nullptr, "null argument");
  *bytes = whir::Prover::workspace_bytes(params_in(params));
  API_END
}

int whir_proof_bytes_max(const whir_params *params, int n_claims, uint64_t *bytes) {
  API_BEGIN
  need(bytes != nullptr && n_claims >= 0, "bad argument");
  whir::Params p = params_in(params);
  whir::Prover::workspace_bytes(p);  // validates
  *bytes = whir::proof_bytes_max(p, n_claims);
  API_END
}

// whir_serve's scheduler with host sleeps for proofs; shape (optional):
// jobs of equal shape id may be grouped, up to max_group per group, a group
// holding its size times one job's bytes and taking the head job's time.  A
// negative duration is a proof that fails after |duration| seconds (a
// transcript or I/O error), its worker's buffers already grown for it.
static void simulate(const double *arrival_s, const uint64_t *need_b, const double *duration_s,
                     const int32_t *shape, int max_group, int n_jobs, int n_workers,
                     uint64_t budget, double *start_s, double *done_s, int32_t *worker,
                     int32_t *status) {
  need(n_jobs >= 0 && n_workers >= 1 && n_workers <= 256, "bad sizes");
  need(n_jobs == 0 || (arrival_s && need_b && duration_s && start_s && done_s && worker && status),
       "null argument");
  std::vector<whir::Job> js(n_jobs);
  std::vector<size_t> nb(n_jobs);
  for (int i = 0; i < n_jobs; i++) {
    need(duration_s[i] >= -10 && duration_s[i] <= 10, "duration out of range");
    js[i].arrival = arrival_s[i];
    js[i].params.k = i;  // carries the job index to need()
    nb[i] = (size_t)need_b[i];
  }
  auto needf = [&](const whir::Params &p) { return nb[p.k]; };
  // a worker's buffers only grow, as a prover's do
  auto make = [](int) -> void * { return new size_t(0); };
  auto exec = [&](void *state, std::vector<whir::Job *> &group) -> size_t {
    const int h = group[0]->params.k;
    size_t *held = static_cast<size_t *>(state);
    *held = std::max(*held, nb[h] * group.size());
    std::this_thread::sleep_for(std::chrono::duration<double>(std::fabs(duration_s[h])));
    if (duration_s[h] < 0) throw whir::WhirError(-5, "injected failure");
    return *held;
  };
  auto held_of = [](void *state) -> size_t { return *static_cast<size_t *>(state); };
  std::vector<void *> states(n_workers, nullptr);
  std::vector<size_t> held(n_workers, 0);
  whir::Grouping grouping;
  grouping.compatible = [&](size_t h, size_t j) { return shape[h] == shape[j]; };
  grouping.max_group = [&](size_t) { return max_group; };
  grouping.grow = [&](int w, const std::vector<int> &group) -> size_t {
    const size_t have = states[w] ? *static_cast<size_t *>(states[w]) : 0;
    const size_t want = nb[group[0]] * group.size();
    return want > have ? want - have : 0;
  };
  whir::run_jobs(js, states, held, budget, true, needf, make, exec, nullptr,
                 shape && max_group > 1 ? &grouping : nullptr, held_of);
  for (void *st : states) delete static_cast<size_t *>(st);
  for (int i = 0; i < n_jobs; i++) {
    start_s[i] = js[i].start;
    done_s[i] = js[i].done;
    worker[i] = js[i].worker;
    status[i] = js[i].status == 0 ? WHIR_OK : js[i].status == -4 ? WHIR_ERR_CAPACITY : WHIR_ERR_INTERNAL;
  }
}

int whir_serve_simulate(const double *arrival_s, const uint64_t *need_b, const double *duration_s,
                        int n_jobs, int n_workers, uint64_t budget, double *start_s,
                        double *done_s, int32_t *worker, int32_t *status) {
  API_BEGIN
  simulate(arrival_s, need_b, duration_s, nullptr, 1, n_jobs, n_workers, budget, start_s, done_s,
           worker, status);
  API_END
}

int whir_serve_simulate_groups(const double *arrival_s, const uint64_t *need_b,
                               const double *duration_s, const int32_t *shape, int max_group,
                               int n_jobs, int n_workers, uint64_t budget, double *start_s,
                               double *done_s, int32_t *worker, int32_t *status) {
  API_BEGIN
  need(max_group >= 1 && (shape || n_jobs == 0), "bad grouping");
  simulate(arrival_s, need_b, duration_s, shape, max_group, n_jobs, n_workers, budget, start_s,
           done_s, worker, status);
  API_END
}

static std::vector<std::vector<int>> groups_in(const int32_t *group_n, int n_groups,
                                               const int32_t *group_ids) {
  need(n_groups >= 0 && (group_n || !n_groups), "bad claim groups");
  std::vector<std::vector<int>> groups;
  size_t off = 0;
  for (int g = 0; g < n_groups; g++) {
    need(group_n[g] > 0 && group_ids, "empty claim group");
    groups.emplace_back(group_ids + off, group_ids + off + group_n[g]);
    off += group_n[g];
  }
  return groups;
}

int whir_verify(const whir_params *params, const int32_t *poly_k, int n_polys,
                const int32_t *group_n, int n_groups, const int32_t *group_ids,
                const uint8_t *proof, size_t len, int32_t *result, uint32_t *checkpoint) {
  API_BEGIN
  need(result != nullptr, "null result");
  std::vector<int> ks = ks_in(poly_k, n_polys);
  std::vector<std::vector<int>> groups = groups_in(group_n, n_groups, group_ids);
  uint32_t cp = 0;
  if (whir::debug_flags() & whir::DEBUG_VERIFY_INLINE) {
    *result = (int32_t)whir::verify(params_in(params), ks, groups, proof, len, &cp);
  } else {
    // the transcript pass with the openings deferred, then the openings
    // hashed here: the same pass structure as whir_verify_batch
    whir::DeferredPaths d;
    whir::VerifyResult r = whir::verify(params_in(params), ks, groups, proof, len, &cp, &d);
    std::vector<uint8_t> ok = whir::deferred_paths_ok(proof, len, d);
    *result = (int32_t)whir::verify_resolve(r, d, ok.data());
  }
  if (checkpoint) *checkpoint = *result == 0 ? cp : 0;
  API_END
}

int whir_verify_batch(whir_ctx *ctx, const whir_params *params, const int32_t *poly_k,
                      int n_polys, const int32_t *group_n, int n_groups,
                      const int32_t *group_ids, int n_proofs, const uint8_t *const *proofs,
                      const size_t *lens, int32_t *results, uint32_t *checkpoints) {
  API_BEGIN
  need(ctx != nullptr, "null context");
  need(n_proofs >= 0 && (n_proofs == 0 || (proofs && lens && results && checkpoints)),
       "bad proof list");
  std::vector<int> ks = ks_in(poly_k, n_polys);
  std::vector<std::vector<int>> groups = groups_in(group_n, n_groups, group_ids);
  if (!ctx->verifier)
    ctx->verifier.reset(new whir::BatchVerifier(
        &ctx->ctx, (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
  ctx->verifier->verify(params_in(params), ks, groups, n_proofs, proofs, lens, results,
                        checkpoints);
  API_END
}

int whir_autotune(whir_ctx *ctx, int log_h_lo, int log_h_hi, char *report, size_t cap) {
  API_BEGIN
  need(ctx != nullptr, "null context");
  std::string r = whir::autotune(ctx->ctx, log_h_lo, log_h_hi);
  if (report && cap) {
    size_t n = std::min(cap - 1, r.size());
    memcpy(report, r.data(), n);
    report[n] = 0;
  }
  API_END
}
int whir_tune_tree(int log_h, int wide_log, int split) {
  API_BEGIN
  whir::gpu::TreeTune t;
  t.wide_log = wide_log;
  t.split = split;
  need(whir::gpu::tree_tune_valid(log_h, t), "tree split out of range");
  whir::gpu::set_tree_tune(log_h, t);
  API_END
}
int whir_tune_dft(int log_h, size_t width, int l1_bias) {
  API_BEGIN
  whir::gpu::DftTune t;
  t.l1_bias = l1_bias;
  need(log_h >= 0 && log_h <= 24 && whir::gpu::dft_tune_valid(log_h, t), "DFT split out of range");
  whir::gpu::set_dft_tune(log_h, width, t);
  API_END
}
int whir_tune_reset(void) {
  API_BEGIN
  whir::tune_reset();
  API_END
}

int whir_prof_enable(whir_ctx *ctx, int on) {
  API_BEGIN
  need(ctx != nullptr, "null context");
  ctx->ctx.prof_enable(on != 0);
  API_END
}
int whir_prof_enable_classes(whir_ctx *ctx, unsigned mask) {
  API_BEGIN
  need(ctx != nullptr, "null context");
  ctx->ctx.prof_enable_classes(mask);
  API_END
}
int whir_prof_read(whir_ctx *ctx, int klass, double *ms, long *launches, double *bytes) {
  API_BEGIN
  need(ctx && ms && launches && bytes, "null argument");
  need(klass >= 0 && klass < Context::K_NCLASS, "bad kernel class");
  ctx->ctx.prof_read(klass, ms, launches, bytes);
  API_END
}

int whir_counters(whir_ctx *ctx, uint64_t *kernel_launches, uint64_t *h2d_bytes,
                  uint64_t *d2h_bytes) {
  API_BEGIN
  need(ctx && kernel_launches && h2d_bytes && d2h_bytes, "null argument");
  *kernel_launches = whir::gpu::launch_count();
  *h2d_bytes = ctx->ctx.h2d_bytes();
  *d2h_bytes = ctx->ctx.d2h_bytes();
  API_END
}

}  // extern "C"
