// Lock-step proving of many same-shape instances (see batch_prover.h).
//
// Device layout for `B` instances: the polynomials back to back
// (stacked: B x 2^k words); the sumcheck arrays back to back at the current
// size (B x 2^kc extension elements, halving with each fold); codewords and
// trees batched as kernels.h describes (row r of instance b is row r B + b,
// trees halves-paired up to the level of B roots).  Reductions publish all
// instances' sums in one go (instance b at b times the per-instance words).
// Per-instance challenges reach the device through a pinned staging area
// copied once before the launches that read it.
#include "batch_prover.h"

#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <exception>
#include <mutex>
#include <thread>

#include "host_math.h"
#include "svo_host.h"

namespace whir {

using kb::E4;
using namespace kb;

// ---------------- host pool ----------------
// A run wakes only as many helpers as its work needs (run's `parts`).  A
// helper that took part spins on the generation counter for a short while
// before sleeping on the condition variable (a round trip's host work comes
// every few tens of microseconds, and waking sleeping threads costs about as
// much); helpers that were not needed go straight back to sleep, so that
// many small groups proving side by side do not keep the host cores busy.
struct HostPool::State {
  std::mutex mu;
  std::condition_variable cv;
  const std::function<void(int)> *fn = nullptr;
  int n = 0;
  int helpers = 0;  // helpers taking part in the current generation
  std::atomic<int> next{0};
  std::atomic<int> active{0};  // taking part and not yet finished
  std::atomic<unsigned long> gen{0};
  std::atomic<bool> stop{false};
  std::exception_ptr err;
  std::vector<std::thread> th;
  void work() {
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= n) return;
      try {
        (*fn)(i);
      } catch (...) {
        std::lock_guard<std::mutex> l(mu);
        if (!err) err = std::current_exception();
      }
    }
  }
};

HostPool::HostPool(int threads) : s_(new State), threads_(std::max(1, threads)) {
  for (int t = 1; t < threads_; t++)
    s_->th.emplace_back([s = s_, t] {
      unsigned long seen = 0;
      bool spin = false;  // took part in the last generation
      for (;;) {
        if (spin) {
          auto t0 = std::chrono::steady_clock::now();
          unsigned spins = 0;
          while (s->gen.load(std::memory_order_acquire) == seen && !s->stop.load()) {
            if ((++spins & 63) == 0 &&
                std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(50))
              break;
            std::this_thread::yield();
          }
        }
        int helpers;
        {
          std::unique_lock<std::mutex> l(s->mu);
          s->cv.wait(l, [&] { return s->stop.load() || s->gen.load() != seen; });
          if (s->stop.load()) return;
          seen = s->gen.load();
          helpers = s->helpers;
        }
        spin = t <= helpers;
        if (!spin) continue;
        s->work();
        s->active.fetch_sub(1, std::memory_order_acq_rel);
      }
    });
}

HostPool::~HostPool() {
  {
    std::lock_guard<std::mutex> l(s_->mu);
    s_->stop.store(true);
  }
  s_->cv.notify_all();
  for (auto &t : s_->th) t.join();
  delete s_;
}

void HostPool::run(int n, const std::function<void(int)> &fn, int parts) {
  if (n <= 0) return;
  const int helpers = std::min({threads_, std::max(1, parts), n}) - 1;
  if (helpers <= 0) {
    for (int i = 0; i < n; i++) fn(i);
    return;
  }
  {
    std::lock_guard<std::mutex> l(s_->mu);
    s_->fn = &fn;
    s_->n = n;
    s_->helpers = helpers;
    s_->next.store(0);
    s_->err = nullptr;
    s_->active.store(helpers);
    s_->gen.fetch_add(1, std::memory_order_acq_rel);
  }
  s_->cv.notify_all();
  s_->work();
  // every helper has left this generation's work before fn goes out of scope
  while (s_->active.load(std::memory_order_acquire) != 0) std::this_thread::yield();
  std::exception_ptr err;
  {
    std::lock_guard<std::mutex> l(s_->mu);
    err = s_->err;
  }
  if (err) std::rethrow_exception(err);
}

// ---------------- sizes ----------------
namespace {

struct BatchSizes {
  size_t stacked, inter, cw0, tree0, scratch, cw, tree, sumcheck, eqbuf, tab, acc, code, rbuf;
  size_t pub, defer, stage, codepin;  // pinned host bytes
  size_t device() const {
    return stacked + inter + cw0 + tree0 + scratch + 2 * (cw + tree + 2 * sumcheck) + eqbuf + tab +
           acc + code + rbuf + stage;
  }
};

int max_stir(const Params &p) {
  int n_rounds, fin;
  number_of_rounds(p.folding, p.k, &n_rounds, &fin);
  int nq = 0;
  for (int r = 0; r <= n_rounds; r++) {
    int kfd, this_rate, prev_rate;
    round_params(p, r, &kfd, &this_rate, &prev_rate);
    nq = std::max(nq, n_stir_queries(p.soundness, p.security_level, prev_rate));
  }
  return nq;
}

BatchSizes batch_sizes(const Params &p, int B, int n_claims) {
  BatchSizes z;
  const int k = p.k, f = p.folding;
  const size_t Bz = (size_t)B, T = (size_t)1 << f;
  const Workspace w = workspace_plan(p);
  const int n_ood0 = n_ood_queries(p.soundness, p.security_level, k, p.rate, EXT_BITS);
  const int nq = max_stir(p);
  z.stacked = Bz * w.stacked;
  // the largest DFT input: the base polynomial or a round's folded one
  z.inter = B > 1 ? Bz * std::max(w.stacked, 16 * ((size_t)1 << (k - f))) : 0;
  z.cw0 = Bz * w.cw0;
  z.tree0 = Bz * w.tree0;
  z.scratch = Bz * w.scratch;
  z.cw = Bz * w.cw;
  z.tree = Bz * w.tree;
  z.sumcheck = Bz * w.sumcheck;
  // eq tables: one claim's compress_hi tables, an OOD evaluation's, or the
  // expression's combined points (claims and OOD samples) per instance
  const int kc0 = k - f, n_pts = n_claims + n_ood0 + 4;
  const int nz = k - f, s_lo = std::min(8, nz);
  size_t per_inst = ((size_t)1 << s_lo) + ((size_t)1 << (nz - s_lo));
  per_inst = std::max(per_inst, ((size_t)1 << std::min(10, kc0)) + ((size_t)1 << (kc0 - std::min(10, kc0))));
  per_inst = std::max(per_inst, (size_t)n_pts * (((size_t)1 << (kc0 / 2)) + ((size_t)1 << (kc0 - kc0 / 2))));
  z.eqbuf = 16 * Bz * per_inst;
  z.tab = 4 * gpu::add_pows_scratch_words(kc0, std::max(1, nq) * B);
  z.acc = 8 * (Bz * std::max((size_t)4 << f, (size_t)12) + 2);
  const size_t nt = (size_t)nq * Bz;
  z.code = 16 * nt * T + 16 * nt + 4 * 4 * nt + 4 * (T + 4) + 4 * (Bz + 4) + 256;
  z.rbuf = 16 * Bz;
  z.pub = 8 * Bz * std::max((size_t)4 << f, (size_t)12) + 64;
  z.defer = Bz * proof_bytes_max(p, n_claims) + 4096;
  // staging per round trip: points of the claims or of the expression's eq
  // additions, the SVO challenges, fold_with_code's row lists, query indexes
  z.stage = Bz * (16 * (size_t)n_pts * (k + 1) + 16 * (size_t)f + (size_t)nq * (4 * T + 48) + 64) +
            4 * (Bz + 1) + 4096;
  z.codepin = z.code;
  return z;
}

}  // namespace

int BatchProver::max_batch(const Params &p) {
  check_params(p);
  const int f = p.folding;
  size_t cap = 1024;
  auto limit = [&](int log_h, size_t w) {
    cap = std::min(cap, (size_t)65535 / w);                         // DFT width < 2^16 words
    cap = std::min(cap, (((size_t)1 << 32) - 1) / (w << log_h));   // words < 2^32
  };
  limit(p.k + p.rate - f, (size_t)1 << f);
  int n_rounds, fin;
  number_of_rounds(f, p.k, &n_rounds, &fin);
  for (int r = 0; r < n_rounds; r++) {
    int kfd, this_rate, prev_rate;
    round_params(p, r, &kfd, &this_rate, &prev_rate);
    limit(p.k - f * (r + 1) + this_rate - f, (size_t)4 << f);
  }
  return (int)std::max<size_t>(1, cap);
}

size_t BatchProver::workspace_bytes(const Params &p, int batch) {
  check_params(p);
  return batch_sizes(p, batch, 16).device();
}

// ---------------- the prover ----------------
struct BatchProver::Impl {
  Context *ctx;
  Params p;
  int ks = 0;
  int B = 0;
  HostPool pool;
  SvoTables svo;
  DeviceBuffer stacked, inter, cw0, tree0, scratch, cw[2], trees[2], sp[2], sw[2], eqbuf, tab, acc,
      code, rbuf, stage_dev;
  PinnedBuffer pub_pin, defer_pin, stage_pin, code_pin, r_pin, roots_pin;

  struct Tree {
    const uint32_t *rows = nullptr;
    uint32_t *nodes = nullptr;
    int log_h = 0, row_len = 0;
  };
  Tree t0, tr[2];
  int cur_tree = -1;

  struct PendingHint {
    size_t ts_off, pin_off, words;
  };
  struct Inst {
    Transcript *ts = nullptr;
    std::vector<SvoClaim> claims;
    std::vector<VirtClaim> virt;
    E4 sum, alpha;
    std::vector<E4> rs;
    std::vector<PendingHint> hints;
    std::vector<E4> pt;  // the point being evaluated
    std::vector<std::vector<E4>> ood_pts;
    std::vector<E4> ood_evs;
    std::vector<size_t> idx;
    size_t rows_off = 0;  // words into the deferred area: this instance's first opened row
    std::vector<E4> round_point, rc;
    E4 r;
    E4 c0, c2, extra;
  };
  std::vector<Inst> in;
  int kc = 0, ping = 0;
  bool pending = false;
  size_t defer_off = 0;  // words

  // staging: bump offsets into stage_pin / stage_dev
  size_t stage_off = 0, stage_copied = 0, stage_mark = 0;
  unsigned int pub_seq = 0;

  Impl(Context *c, const Params &pp, int threads) : ctx(c), p(pp), ks(pp.folding), pool(threads) {}

  cudaStream_t st() const { return ctx->stream(); }
  // per-instance host work on the pool: one thread per 4 instances
  void par(const std::function<void(int)> &fn) { pool.run(B, fn, (B + 3) / 4); }

  // ---- staging ----
  size_t stage_alloc(size_t bytes) {
    bytes = (bytes + 15) & ~(size_t)15;
    if (stage_off + bytes > stage_pin.bytes())
      throw WhirError(-5, "batched prover: staging area too small");
    size_t o = stage_off;
    stage_off += bytes;
    return o;
  }
  template <class T>
  T *stage_host(size_t off) {
    return reinterpret_cast<T *>(stage_pin.data() + off);
  }
  template <class T>
  T *stage_devp(size_t off) {
    return reinterpret_cast<T *>(stage_dev.as<uint8_t>() + off);
  }
  void stage_upload() {
    if (stage_off == stage_copied) return;
    cuda_check(copy_async(*ctx, stage_dev.as<uint8_t>() + stage_copied,
                          stage_pin.data() + stage_copied, stage_off - stage_copied,
                          cudaMemcpyHostToDevice),
               "h2d");
    stage_copied = stage_off;
  }
  // a full wait on the stream: every staged copy has been read
  void sync() {
    ctx->sync();
    stage_off = stage_copied = 0;
  }

  // ---- reductions published to pinned memory ----
  gpu::Publish publish(size_t words) {
    if (8 * words > pub_pin.bytes()) throw WhirError(-5, "reduction too wide to publish");
    gpu::Publish pb;
    pb.counter = reinterpret_cast<unsigned int *>(acc.as<unsigned long long>() + acc.bytes() / 8 - 1);
    pb.host = reinterpret_cast<unsigned long long *>(pub_pin.data());
    pb.words = (int)words;
    pb.flag = ctx->flag();
    pb.seq = pub_seq = ctx->next_seq();
    stage_mark = stage_off;
    return pb;
  }
  // the publishing launch and everything before it have completed; the
  // staging area is free again unless something was staged after it
  void wait_published() {
    ctx->wait_flag(pub_seq);
    if (stage_off == stage_mark) stage_off = stage_copied = 0;
  }
  const unsigned long long *published() const {
    return reinterpret_cast<const unsigned long long *>(pub_pin.data());
  }

  // ---- buffers ----
  void reserve(int batch, int n_claims) {
    BatchSizes z = batch_sizes(p, batch, n_claims);
    stacked.reserve(z.stacked);
    inter.reserve(z.inter);
    cw0.reserve(z.cw0);
    tree0.reserve(z.tree0);
    scratch.reserve(z.scratch);
    for (int i = 0; i < 2; i++) {
      cw[i].reserve(z.cw);
      trees[i].reserve(z.tree);
      sp[i].reserve(z.sumcheck);
      sw[i].reserve(z.sumcheck);
    }
    eqbuf.reserve(z.eqbuf);
    tab.reserve(z.tab);
    acc.reserve(z.acc);
    code.reserve(z.code);
    rbuf.reserve(z.rbuf);
    stage_dev.reserve(z.stage);
    pub_pin.reserve(z.pub);
    defer_pin.reserve(z.defer);
    stage_pin.reserve(z.stage);
    code_pin.reserve(z.codepin);
    r_pin.reserve(z.rbuf);
    roots_pin.reserve(32 * (size_t)batch + 64);
  }
  size_t device_bytes() const {
    size_t s = 0;
    const DeviceBuffer *bufs[] = {&stacked, &inter, &cw0,  &tree0, &scratch, &cw[0], &cw[1],
                                  &trees[0], &trees[1], &sp[0], &sp[1], &sw[0], &sw[1],
                                  &eqbuf,   &tab,     &acc,  &code,  &rbuf,   &stage_dev};
    for (auto b : bufs) s += b->bytes();
    return s;
  }

  // ---- encode + commit of all instances ----
  // src: B polynomials of 2^k_src elements of `dim` words, back to back
  void encode_commit(const uint32_t *src, int k_src, int rate, int dim, uint32_t *codeword,
                     uint32_t *nodes, Tree *out) {
    const int f = p.folding;
    const int log_h = k_src + rate - f;
    const size_t w = (size_t)dim << f, h_in = (size_t)1 << (k_src - f), rows = (size_t)1 << log_h;
    const size_t Bz = (size_t)B;
    const uint32_t *din = src;
    ctx->prof_begin(Context::K_DFT);
    if (B > 1) {
      cuda_check(gpu::interleave_rows(src, h_in, w, B, inter.as<uint32_t>(), st()), "interleave");
      din = inter.as<uint32_t>();
    }
    cuda_check(gpu::dft_batch(din, h_in, w * Bz, log_h, codeword, scratch.as<uint32_t>(), st()),
               "dft_batch");
    ctx->prof_end(Context::K_DFT, 4.0 * (double)(Bz * (h_in * w + rows * w)));
    ctx->prof_begin(Context::K_LEAF);
    cuda_check(gpu::hash_rows(codeword, rows * Bz, (int)w, nodes, st()), "hash_rows");
    ctx->prof_end(Context::K_LEAF, 4.0 * (double)(Bz * (rows * w + rows * 8)));
    ctx->prof_begin(Context::K_TREE);
    cuda_check(gpu::build_tree_batch(nodes, log_h, B, st()), "build_tree");
    ctx->prof_end(Context::K_TREE, 32.0 * (double)(Bz * (2 * rows - 2 + rows - 1)));
    cuda_check(copy_async(*ctx, roots_pin.data(), nodes + Bz * gpu::level_offset_words(log_h, log_h),
                          32 * Bz, cudaMemcpyDeviceToHost),
               "roots");
    sync();
    out->rows = codeword;
    out->nodes = nodes;
    out->log_h = log_h;
    out->row_len = (int)w;
    const uint32_t *roots = reinterpret_cast<const uint32_t *>(roots_pin.data());
    par([&](int b) { in[b].ts->write_digest(roots + 8 * (size_t)b); });
  }

  // ---- SVO claims of every instance at in[b].pt (SvoPoint::new + eval) ----
  void svo_claims(std::vector<SvoClaim> &cs) {
    const int k = p.k, nz = k - ks, s_lo = std::min(8, nz);
    const size_t per = ((size_t)1 << s_lo) + ((size_t)1 << (nz - s_lo));
    const size_t Bz = (size_t)B;
    const size_t po = stage_alloc(16 * Bz * (size_t)std::max(nz, 1)), so = stage_alloc(16 * Bz);
    E4 *hp = stage_host<E4>(po), *hs = stage_host<E4>(so);
    for (int b = 0; b < B; b++) {
      std::copy(in[b].pt.begin() + ks, in[b].pt.begin() + k, hp + (size_t)b * nz);
      hs[b] = e_one();
    }
    stage_upload();
    E4 *lo = eqbuf.as<E4>();
    cuda_check(gpu::eq_tables(stage_devp<E4>(po), stage_devp<E4>(so), B, nz, s_lo, lo, st()),
               "eq_tables");
    const size_t na = (size_t)4 << ks;
    gpu::HiStrides sd;
    sd.poly = (size_t)1 << k;
    sd.tab = per;
    sd.acc = na;
    ctx->prof_begin(Context::K_SUMCHECK);
    cuda_check(gpu::compress_hi_batch(stacked.as<uint32_t>(), k, ks, lo, s_lo, lo + ((size_t)1 << s_lo),
                                      acc.as<unsigned long long>(), B, sd, st(), publish(na * Bz)),
               "compress_hi");
    ctx->prof_end(Context::K_SUMCHECK, 4.0 * (double)(Bz << k));
    wait_published();
    const unsigned long long *h = published();
    par([&](int b) {
      SvoClaim &c = cs[b];
      c.k = k;
      c.point = in[b].pt;
      svo_finish(c, ks, h + na * (size_t)b);
    });
  }

  // ---- write_virtual_eval (prover.rs:232-277), one polynomial per instance ----
  void write_virtual_eval() {
    const int k = p.k;
    par([&](int b) {
      in[b].pt.resize(k);
      expand(in[b].pt.data(), k, in[b].ts->draw_ext());
    });
    std::vector<SvoClaim> cs(B);
    svo_claims(cs);
    svo.build(ks);
    const size_t na = svo_acc_size(ks);
    par([&](int b) {
      VirtClaim v;
      v.point = in[b].pt;
      v.acc.assign(na, e_zero());
      const E4 weight = eval_eq_xy(nullptr, v.point.data() + k, 0);  // no selector bits
      v.eval = e_add(e_zero(), e_mul(weight, cs[b].eval));
      svo.accumulate(v.acc, cs[b], weight, ks);
      in[b].ts->write_ext(v.eval);
      in[b].virt.push_back(std::move(v));
    });
  }

  // ---- sumcheck arrays ----
  E4 *P() { return sp[ping].as<E4>(); }
  E4 *W() { return sw[ping].as<E4>(); }

  // upload the instances' latest challenges (in[b].r) for the next fold
  void upload_r() {
    E4 *h = reinterpret_cast<E4 *>(r_pin.data());
    for (int b = 0; b < B; b++) h[b] = in[b].r;
    cuda_check(copy_async(*ctx, rbuf.as<E4>(), h, 16 * (size_t)B, cudaMemcpyHostToDevice), "h2d");
  }
  void defer_fold() {  // Expression::fix_var (expr.rs:101-104)
    upload_r();
    pending = true;
    kc -= 1;
  }
  void flush() {
    if (!pending) return;
    const size_t n = (size_t)1 << kc;
    cuda_check(gpu::sumcheck_round_batch(P(), W(), 2 * n, true, rbuf.as<E4>(), sp[1 - ping].as<E4>(),
                                         sw[1 - ping].as<E4>(), false, nullptr, 0, B, st()),
               "fold");
    ping = 1 - ping;
    pending = false;
  }
  // (c0, c2) of every instance's arrays, applying a pending fold in the same
  // pass; with code, fold_with_code's per-query pass of this round adds into
  // the same slots (and its round-0 sum term into slots 8..12)
  void coeffs_begin(const gpu::CodeState *code = nullptr, int code_round = 0) {
    if (code && code->n == 0) code = nullptr;
    const size_t Bz = (size_t)B;
    gpu::Publish pub = publish(12 * Bz), none;
    const size_t n = (size_t)1 << kc;
    unsigned long long *a = acc.as<unsigned long long>();
    ctx->prof_begin(Context::K_SUMCHECK);
    if (pending) {
      cuda_check(gpu::sumcheck_round_batch(P(), W(), 2 * n, true, rbuf.as<E4>(),
                                           sp[1 - ping].as<E4>(), sw[1 - ping].as<E4>(), true, a,
                                           12, B, st(), code ? none : pub),
                 "round");
      ping = 1 - ping;
      pending = false;
      ctx->prof_end(Context::K_SUMCHECK, 3.0 * 2 * 16 * (double)(n * Bz));
    } else {
      cuda_check(gpu::sumcheck_round_batch(P(), W(), n, false, nullptr, nullptr, nullptr, true, a,
                                           12, B, st(), code ? none : pub),
                 "round");
      ctx->prof_end(Context::K_SUMCHECK, 2 * 16 * (double)(n * Bz));
    }
    if (code) cuda_check(gpu::code_round(*code, code_round, e_zero(), a, st(), pub), "code_round");
  }
  void coeffs_end() {
    wait_published();
    const unsigned long long *h = published();
    for (int b = 0; b < B; b++) {
      in[b].c0 = reduce_acc(h + 12 * (size_t)b);
      in[b].c2 = reduce_acc(h + 12 * (size_t)b + 4);
      in[b].extra = reduce_acc(h + 12 * (size_t)b + 8);
    }
  }

  // w[off ..] += eq(point) * scale for each instance's points (the same
  // count per instance), one table launch and one addition launch
  void add_eqs(E4 *w, int kt, const std::vector<std::vector<std::vector<E4>>> &pts,
               const std::vector<std::vector<E4>> &scales) {
    const int nt = (int)pts[0].size();
    if (nt == 0) return;
    const int s = kt / 2;
    const size_t per = ((size_t)1 << s) + ((size_t)1 << (kt - s));
    if (16 * per * nt * (size_t)B > eqbuf.bytes()) {
      sync();
      eqbuf.reserve(16 * per * nt * (size_t)B);
    }
    const size_t Bz = (size_t)B;
    const size_t po = stage_alloc(16 * Bz * nt * (size_t)std::max(kt, 1)), so = stage_alloc(16 * Bz * nt);
    E4 *hp = stage_host<E4>(po), *hs = stage_host<E4>(so);
    for (int b = 0; b < B; b++)
      for (int t = 0; t < nt; t++) {
        std::copy(pts[b][t].begin(), pts[b][t].begin() + kt, hp + ((size_t)b * nt + t) * kt);
        hs[(size_t)b * nt + t] = scales[b][t];
      }
    stage_upload();
    cuda_check(gpu::eq_tables(stage_devp<E4>(po), stage_devp<E4>(so), B * nt, kt, s, eqbuf.as<E4>(),
                              st()),
               "eq_tables");
    cuda_check(gpu::add_eq_batch(w, kt, eqbuf.as<E4>(), nt, B, st()), "add_eq");
  }

  // w += sum_t scales_t var_t^i per instance (ragged counts)
  void add_pows(const std::vector<std::vector<uint32_t>> &vars,
                const std::vector<std::vector<E4>> &scales) {
    const size_t Bz = (size_t)B;
    size_t total = 0, mx = 0;
    for (int b = 0; b < B; b++) {
      total += vars[b].size();
      mx = std::max(mx, vars[b].size());
    }
    if (total == 0) return;
    const size_t vo = stage_alloc(4 * total), so = stage_alloc(16 * total), oo = stage_alloc(4 * (Bz + 1));
    uint32_t *hv = stage_host<uint32_t>(vo);
    E4 *hs = stage_host<E4>(so);
    int *ho = stage_host<int>(oo);
    size_t o = 0;
    for (int b = 0; b < B; b++) {
      ho[b] = (int)o;
      std::copy(vars[b].begin(), vars[b].end(), hv + o);
      std::copy(scales[b].begin(), scales[b].end(), hs + o);
      o += vars[b].size();
    }
    ho[B] = (int)o;
    stage_upload();
    add_pows_dev(stage_devp<uint32_t>(vo), stage_devp<E4>(so), stage_devp<int>(oo), (int)total, (int)mx);
  }
  void add_pows_dev(const uint32_t *vars, const E4 *scales, const int *off, int total, int mx) {
    if (total == 0) return;
    const size_t words = gpu::add_pows_scratch_words(kc, total);
    if (4 * words > tab.bytes()) {
      sync();
      tab.reserve(4 * words);
    }
    cuda_check(gpu::add_pows_batch(W(), kc, vars, scales, off, total, mx, B, tab.as<uint32_t>(), st()),
               "add_pows");
  }

  // ---- new_prover (prover.rs:280-354) incl. expression (185-229) ----
  void new_prover() {
    const int k = p.k;
    svo.build(ks);
    const size_t na = svo_acc_size(ks);
    // the expression's eq points and scales, per instance
    std::vector<std::vector<std::vector<E4>>> pts(B);
    std::vector<std::vector<E4>> scl(B);
    par([&](int b) {
      Inst &I = in[b];
      I.alpha = I.ts->draw_ext();
      const int n = (int)I.claims.size();
      std::vector<E4> alphas(n), evals;
      E4 a = e_one();
      for (int c = 0; c < n; c++) {  // one polynomial: layout order is claim order
        alphas[c] = a;
        evals.push_back(I.claims[c].eval);
        a = e_mul(a, I.alpha);
      }
      for (auto &v : I.virt) evals.push_back(v.eval);
      I.sum = horner(evals.data(), evals.size(), I.alpha);
      std::vector<E4> accv(na, e_zero());
      for (int c = 0; c < n; c++) svo.accumulate(accv, I.claims[c], alphas[c], ks);
      E4 av = e_pow(I.alpha, (uint64_t)n);
      for (auto &v : I.virt) {
        for (size_t i = 0; i < accv.size(); i++) accv[i] = e_add(accv[i], e_mul(av, v.acc[i]));
        av = e_mul(av, I.alpha);
      }
      I.rs.clear();
      svo_rounds(*I.ts, accv, ks, I.sum, I.rs);
      a = e_one();
      for (int c = 0; c < n; c++) {
        const SvoClaim &cl = I.claims[c];
        pts[b].emplace_back(cl.point.begin() + ks, cl.point.end());
        scl[b].push_back(e_mul(a, eval_eq_xy(cl.point.data(), I.rs.data(), ks)));
        a = e_mul(a, I.alpha);
      }
      for (auto &v : I.virt) {
        pts[b].emplace_back(v.point.begin() + ks, v.point.end());
        scl[b].push_back(e_mul(a, eval_eq_xy(v.point.data(), I.rs.data(), ks)));
        a = e_mul(a, I.alpha);
      }
    });
    kc = k - ks;
    ping = 0;
    pending = false;
    const size_t N = (size_t)1 << kc, Bz = (size_t)B;
    const size_t ro = stage_alloc(16 * Bz * (size_t)std::max(ks, 1));
    E4 *hr = stage_host<E4>(ro);
    for (int b = 0; b < B; b++) std::copy(in[b].rs.begin(), in[b].rs.end(), hr + (size_t)b * ks);
    stage_upload();
    cuda_check(gpu::compress_lo_batch(stacked.as<uint32_t>(), k, ks, stage_devp<E4>(ro), B,
                                      (size_t)1 << k, P(), st()),
               "compress_lo");
    cuda_check(cudaMemsetAsync(W(), 0, Bz * N * sizeof(E4), st()), "memset");
    add_eqs(W(), kc, pts, scl);
  }

  // ---- queries (MerkleTree::query, poseidon_packed.rs:145-233) ----
  // Gathers every instance's opened rows and sibling paths (in[b].idx) into
  // the deferred pinned area and reserves their hints in the transcripts;
  // in[b].rows_off is the instance's first row there.
  void query(const Tree &t) {
    const size_t per = (size_t)t.row_len + 8 * (size_t)t.log_h;
    size_t total = 0;
    std::vector<size_t> qoff(B + 1);
    for (int b = 0; b < B; b++) {
      qoff[b] = total;
      total += in[b].idx.size();
    }
    qoff[B] = total;
    if (4 * (defer_off + per * total) > defer_pin.bytes())
      throw WhirError(-5, "batched prover: deferred area too small");
    const size_t base = defer_off;
    defer_off += per * total;
    par([&](int b) {
      Inst &I = in[b];
      I.rows_off = base + qoff[b] * per;
      for (size_t q = 0; q < I.idx.size(); q++)
        I.hints.push_back(PendingHint{I.ts->hint_reserve(per), I.rows_off + q * per, per});
    });
    if (total == 0) return;
    const size_t io = stage_alloc(4 * total), no = stage_alloc(4 * total);
    uint32_t *hi = stage_host<uint32_t>(io);
    int *hn = stage_host<int>(no);
    for (int b = 0; b < B; b++)
      for (size_t q = 0; q < in[b].idx.size(); q++) {
        hi[qoff[b] + q] = (uint32_t)in[b].idx[q];
        hn[qoff[b] + q] = b;
      }
    stage_upload();
    cuda_check(gpu::gather_openings_batch(t.rows, t.row_len, t.nodes, t.log_h, B,
                                          stage_devp<uint32_t>(io), stage_devp<int>(no), (int)total,
                                          reinterpret_cast<uint32_t *>(defer_pin.data()) + base, st()),
               "gather");
    ctx->count_copy(4 * per * total, cudaMemcpyDeviceToHost);
  }
  const uint32_t *defer_ptr(size_t off) const {
    return reinterpret_cast<const uint32_t *>(defer_pin.data()) + off;
  }

  static std::vector<size_t> stir_indexes(Transcript &ts, int bits, int n) {  // whir.rs:64-77
    std::vector<size_t> v(n);
    for (int i = 0; i < n; i++) v[i] = ts.draw_bits(bits);
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    return v;
  }

  // ---- fold (prover.rs:378-397) ----
  void fold(const Tree &prev, int kfd) {
    const size_t per = (size_t)prev.row_len + 8 * (size_t)prev.log_h;
    const uint32_t omega = two_adic_generator(kfd);
    par([&](int b) { in[b].alpha = in[b].ts->draw_ext(); });
    flush();
    std::vector<std::vector<E4>> sc(B), ps(B);
    std::vector<std::vector<uint32_t>> vars(B);
    par([&](int b) {
      Inst &I = in[b];
      E4 a = e_one();
      for (size_t i = 0; i < I.ood_pts.size(); i++) {
        sc[b].push_back(a);
        a = e_mul(a, I.alpha);
      }
      for (size_t i = 0; i < I.idx.size(); i++) {
        vars[b].push_back(kb::pow(omega, I.idx[i]));
        ps[b].push_back(a);
        a = e_mul(a, I.alpha);
      }
    });
    std::vector<std::vector<std::vector<E4>>> pts(B);
    for (int b = 0; b < B; b++) pts[b] = in[b].ood_pts;
    add_eqs(W(), kc, pts, sc);
    add_pows(vars, ps);
    for (int i = 0; i < p.folding; i++) {
      coeffs_begin();
      coeffs_end();
      par([&](int b) {
        Inst &I = in[b];
        if (i == 0) {  // combine_claims' sum update (combine.rs:49-53)
          std::vector<E4> ev(I.ood_evs);
          for (size_t q = 0; q < I.idx.size(); q++)
            ev.push_back(eval_ext_small(reinterpret_cast<const E4 *>(defer_ptr(I.rows_off + per * q)),
                                        p.folding, I.round_point.data()));
          I.sum = e_add(I.sum, horner(ev.data(), ev.size(), I.alpha));
        }
        I.ts->write_ext(I.c0);
        I.ts->write_ext(I.c2);
        I.r = I.ts->draw_ext();
        I.sum = extrapolate012(I.c0, e_sub(I.sum, I.c0), I.c2, I.r);
        I.rc.push_back(I.r);
        I.rs.push_back(I.r);
      });
      defer_fold();
    }
  }

  // ---- fold_with_code (prover.rs:400-561) ----
  void fold_with_code() {
    const int d = p.folding, k_data = t0.log_h;
    if (k_data < d) throw WhirError(-1, "codeword shorter than the folding");
    par([&](int b) {
      Inst &I = in[b];
      I.alpha = I.ts->draw_ext();
      I.sum = e_add(I.sum, horner(I.ood_evs.data(), I.ood_evs.size(), I.alpha));
    });
    flush();
    std::vector<std::vector<E4>> sc(B), scales(B);
    par([&](int b) {
      Inst &I = in[b];
      E4 a = e_one();
      for (size_t i = 0; i < I.ood_pts.size(); i++) {
        sc[b].push_back(a);
        a = e_mul(a, I.alpha);
      }
      for (size_t i = 0; i < I.idx.size(); i++) {
        scales[b].push_back(a);
        a = e_mul(a, I.alpha);
      }
    });
    std::vector<std::vector<std::vector<E4>>> pts(B);
    for (int b = 0; b < B; b++) pts[b] = in[b].ood_pts;
    add_eqs(W(), kc, pts, sc);
    // the per-query state of the recursion g (prover.rs:437-461) for every
    // instance's queries, flat in instance order (see gpu::code_round)
    const int lS = k_data - d;
    const size_t S = (size_t)1 << lS, T = (size_t)1 << d, Bz = (size_t)B;
    std::vector<int> qoff(B + 1);
    size_t n = 0, mx = 0;
    for (int b = 0; b < B; b++) {
      qoff[b] = (int)n;
      n += in[b].idx.size();
      mx = std::max(mx, in[b].idx.size());
    }
    qoff[B] = (int)n;
    gpu::CodeState cs;
    cs.n = (int)n;
    cs.d = d;
    cs.k_data = k_data;
    cs.omega = two_adic_generator(k_data);
    cs.winv = inv(cs.omega);
    cs.two_inv = inv(from_canonical(2));
    // layout in `code` (mirrored in code_pin): G | scales | idx | ws | tw | B | inst | wd | qoff
    const size_t g_b = 16 * n * T, s_b = 16 * n, u_b = 4 * ((n + 3) & ~(size_t)3);
    const size_t wd_b = 4 * ((T + 3) & ~(size_t)3), q_b = 4 * ((Bz + 4) & ~(size_t)3);
    const size_t need = g_b + s_b + 5 * u_b + wd_b + q_b + 64;
    if (need > code.bytes() || need > code_pin.bytes()) {
      sync();
      code.reserve(need);
      code_pin.reserve(need);
    }
    uint8_t *cd = code.as<uint8_t>(), *ch = code_pin.data();
    size_t o = 0;
    auto place = [&](size_t bytes) {
      size_t at = o;
      o += bytes;
      return at;
    };
    const size_t oG = place(g_b), oS = place(s_b), oI = place(u_b), oW = place(u_b), oT = place(u_b),
                 oB = place(u_b), oN = place(u_b), oD = place(wd_b), oQ = place(q_b);
    cs.G = reinterpret_cast<E4 *>(cd + oG);
    cs.scales = reinterpret_cast<E4 *>(cd + oS);
    cs.idx = reinterpret_cast<uint32_t *>(cd + oI);
    cs.ws = reinterpret_cast<uint32_t *>(cd + oW);
    cs.tw = reinterpret_cast<uint32_t *>(cd + oT);
    cs.B = reinterpret_cast<uint32_t *>(cd + oB);
    cs.inst = reinterpret_cast<int *>(cd + oN);
    cs.wd = reinterpret_cast<uint32_t *>(cd + oD);
    cs.r_b = rbuf.as<E4>();
    cs.acc_stride = 12;
    const int *d_qoff = reinterpret_cast<int *>(cd + oQ);
    {
      E4 *hs = reinterpret_cast<E4 *>(ch + oS);
      uint32_t *hi = reinterpret_cast<uint32_t *>(ch + oI), *hw = reinterpret_cast<uint32_t *>(ch + oD);
      int *hn = reinterpret_cast<int *>(ch + oN), *hq = reinterpret_cast<int *>(ch + oQ);
      for (int b = 0; b < B; b++) {
        hq[b] = qoff[b];
        for (size_t i = 0; i < in[b].idx.size(); i++) {
          hi[qoff[b] + i] = (uint32_t)in[b].idx[i];
          hs[qoff[b] + i] = scales[b][i];
          hn[qoff[b] + i] = b;
        }
      }
      hq[B] = (int)n;
      const uint32_t wd = kb::pow(cs.winv, S);
      hw[0] = ONE;
      for (size_t t = 1; t < T; t++) hw[t] = mul(hw[t - 1], wd);
      // scales .. qoff in one copy (G is written on the device)
      cuda_check(copy_async(*ctx, cd + oS, ch + oS, o - oS, cudaMemcpyHostToDevice), "h2d");
    }
    // G_0: the row evaluations at eq(rs) of each query's 2^d rows base + t S
    const size_t ro = stage_alloc(4 * n * T + 4), fo = stage_alloc(4 * (Bz + 1)),
                 rso = stage_alloc(16 * Bz * (size_t)std::max(ks, 1));
    uint32_t *hr = stage_host<uint32_t>(ro);
    int *hf = stage_host<int>(fo);
    E4 *hrs = stage_host<E4>(rso);
    par([&](int b) {
      hf[b] = (int)(qoff[b] * T);
      for (size_t i = 0; i < in[b].idx.size(); i++)
        for (size_t t = 0; t < T; t++)
          hr[(qoff[b] + i) * T + t] = (uint32_t)((in[b].idx[i] & (S - 1)) + t * S);
      std::copy(in[b].rs.begin(), in[b].rs.end(), hrs + (size_t)b * ks);
    });
    hf[B] = (int)(n * T);
    stage_upload();
    if ((int)in[0].rs.size() != ks) throw WhirError(-5, "fold_with_code after the SVO rounds only");
    cuda_check(gpu::row_evals_batch(t0.rows, t0.row_len, stage_devp<uint32_t>(ro), stage_devp<int>(fo),
                                    (int)(mx * T), ks, stage_devp<E4>(rso), B, cs.G, st()),
               "row_evals");
    for (int round = 0; round < d; round++) {
      coeffs_begin(&cs, round);
      coeffs_end();
      par([&](int b) {
        Inst &I = in[b];
        if (round == 0) I.sum = e_add(I.sum, I.extra);  // prover.rs:426-435
        I.ts->write_ext(I.c0);
        I.ts->write_ext(I.c2);
        I.r = I.ts->draw_ext();
        I.sum = extrapolate012(I.c0, e_sub(I.sum, I.c0), I.c2, I.r);
        I.rc.push_back(I.r);
      });
      defer_fold();
    }
    cuda_check(gpu::code_finish(cs, e_zero(), st()), "code_finish");
    flush();
    // combine_pows_scaled (combine.rs:441-468)
    add_pows_dev(cs.ws, cs.scales, d_qoff, (int)n, (int)mx);
    par([&](int b) {
      for (auto &r : in[b].rc) in[b].rs.push_back(r);
    });
  }

  // ---- OOD evaluations of every instance's expression poly ----
  void ood(int n_o) {
    const size_t Bz = (size_t)B;
    for (int i = 0; i < n_o; i++) {
      par([&](int b) {
        in[b].pt.resize(kc);
        expand(in[b].pt.data(), kc, in[b].ts->draw_ext());
      });
      const unsigned long long *h = nullptr;
      std::vector<E4> direct;
      if (kc == 0) {
        E4 *hp = reinterpret_cast<E4 *>(pub_pin.data());
        cuda_check(copy_async(*ctx, hp, P(), 16 * Bz, cudaMemcpyDeviceToHost), "d2h");
        sync();
        direct.assign(hp, hp + B);
      } else {
        const int s_lo = std::min(10, kc);
        const size_t per = ((size_t)1 << s_lo) + ((size_t)1 << (kc - s_lo));
        const size_t po = stage_alloc(16 * Bz * kc), so = stage_alloc(16 * Bz);
        E4 *hp = stage_host<E4>(po), *hs = stage_host<E4>(so);
        for (int b = 0; b < B; b++) {
          std::copy(in[b].pt.begin(), in[b].pt.end(), hp + (size_t)b * kc);
          hs[b] = e_one();
        }
        stage_upload();
        E4 *lo = eqbuf.as<E4>();
        cuda_check(gpu::eq_tables(stage_devp<E4>(po), stage_devp<E4>(so), B, kc, s_lo, lo, st()),
                   "eq_tables");
        cuda_check(gpu::eval_ext_batch(P(), kc, lo, s_lo, lo + ((size_t)1 << s_lo), per, B,
                                       acc.as<unsigned long long>(), st(), publish(4 * Bz)),
                   "eval_ext");
        wait_published();
        h = published();
      }
      par([&](int b) {
        Inst &I = in[b];
        const E4 e = h ? reduce_acc(h + 4 * (size_t)b) : direct[b];
        I.ts->write_ext(e);
        I.ood_pts.push_back(I.pt);
        I.ood_evs.push_back(e);
      });
    }
  }

  // ---- Whir::open (whir.rs:168-359) ----
  void open() {
    const int f = p.folding;
    defer_off = 0;
    int n_ood = n_ood_queries(p.soundness, p.security_level, p.k, p.rate, EXT_BITS);
    for (int i = 0; i < n_ood; i++) write_virtual_eval();
    new_prover();
    int n_rounds, final_rounds;
    number_of_rounds(f, p.k, &n_rounds, &final_rounds);
    cur_tree = -1;
    for (int round = 0; round < n_rounds; round++) {
      int kfd, this_rate, prev_rate;
      whir::round_params(p, round, &kfd, &this_rate, &prev_rate);
      flush();
      const int slot = cur_tree < 0 ? 0 : 1 - cur_tree;
      encode_commit(reinterpret_cast<const uint32_t *>(P()), kc, this_rate, 4,
                    cw[slot].as<uint32_t>(), trees[slot].as<uint32_t>(), &tr[slot]);
      const int n_o = n_ood_queries(p.soundness, p.security_level, kc, this_rate, EXT_BITS);
      par([&](int b) {
        in[b].ood_pts.clear();
        in[b].ood_evs.clear();
      });
      ood(n_o);
      const int n_s = n_stir_queries(p.soundness, p.security_level, prev_rate);
      par([&](int b) {
        in[b].idx = stir_indexes(*in[b].ts, kfd, n_s);
        in[b].rc.clear();
      });
      if (round == 0) {
        query(t0);
        fold_with_code();
      } else {
        query(tr[cur_tree]);
        fold(tr[cur_tree], kfd);
      }
      par([&](int b) { in[b].round_point = in[b].rc; });
      cur_tree = slot;
    }
    flush();
    const size_t nf = (size_t)1 << kc, Bz = (size_t)B;
    if (16 * nf * Bz > pub_pin.bytes()) pub_pin.reserve(16 * nf * Bz);
    E4 *hf = reinterpret_cast<E4 *>(pub_pin.data());
    cuda_check(copy_async(*ctx, hf, P(), 16 * nf * Bz, cudaMemcpyDeviceToHost), "d2h");
    sync();
    int kfd, this_rate, prev_rate;
    whir::round_params(p, n_rounds, &kfd, &this_rate, &prev_rate);
    const int n_s = n_stir_queries(p.soundness, p.security_level, prev_rate);
    par([&](int b) {
      for (size_t i = 0; i < nf; i++) in[b].ts->write_ext(hf[(size_t)b * nf + i]);
      in[b].idx = stir_indexes(*in[b].ts, kfd, n_s);
    });
    query(cur_tree >= 0 ? tr[cur_tree] : t0);
    sync();
    par([&](int b) {
      Inst &I = in[b];
      for (auto &h : I.hints) I.ts->hint_fill(h.ts_off, defer_ptr(h.pin_off), h.words);
      I.hints.clear();
    });
    if (kc != final_rounds) throw WhirError(-1, "final sumcheck size mismatch");
  }

  void prove(const std::vector<Transcript *> &ts, const std::vector<const uint32_t *> &polys,
             bool on_device, int n_claims, bool commit_only,
             const std::function<void(int)> &finish) {
    B = (int)ts.size();
    if (B < 1 || polys.size() != ts.size()) throw WhirError(-1, "batch of no instances");
    if (B > BatchProver::max_batch(p)) throw WhirError(-1, "batch too large for these parameters");
    if (n_claims < 0) throw WhirError(-1, "negative claim count");
    reserve(B, n_claims);
    in.assign(B, Inst());
    for (int b = 0; b < B; b++) {
      if (!ts[b] || !polys[b]) throw WhirError(-1, "null transcript or polynomial");
      in[b].ts = ts[b];
    }
    stage_off = stage_copied = 0;
    defer_off = 0;
    const size_t cap = commit_only ? 64 : proof_bytes_max(p, n_claims) + 64;
    par([&](int b) { in[b].ts->reserve(cap); });
    // reductions publish and re-zero their accumulators; start from zero
    cuda_check(cudaMemsetAsync(acc.as<void>(), 0, acc.bytes(), st()), "memset");
    const size_t n = (size_t)1 << p.k;
    for (int b = 0; b < B; b++)
      cuda_check(copy_async(*ctx, stacked.as<uint32_t>() + (size_t)b * n, polys[b], 4 * n,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice),
                 "poly copy");
    encode_commit(stacked.as<uint32_t>(), p.k, p.rate, 1, cw0.as<uint32_t>(), tree0.as<uint32_t>(), &t0);
    if (commit_only) {
      if (finish) par(finish);
      return;
    }
    for (int c = 0; c < n_claims; c++) {  // the harness's claim groups (test.rs:225-231)
      par([&](int b) {
        in[b].pt.resize(p.k);
        expand(in[b].pt.data(), p.k, in[b].ts->draw_ext());
      });
      std::vector<SvoClaim> cs(B);
      svo_claims(cs);
      par([&](int b) {
        cs[b].poly = 0;
        in[b].ts->write_ext(cs[b].eval);
        in[b].claims.push_back(std::move(cs[b]));
      });
    }
    open();
    if (finish) par(finish);
  }
};

BatchProver::BatchProver(Context *ctx, const Params &p, int host_threads)
    : m_(nullptr), p_(p) {
  check_params(p);
  m_ = new Impl(ctx, p, host_threads);
}
BatchProver::~BatchProver() { delete m_; }
void BatchProver::set_params(const Params &p) {
  check_params(p);
  p_ = p;
  m_->p = p;
  m_->ks = p.folding;
}
void BatchProver::reserve(int batch) { m_->reserve(batch, 16); }
size_t BatchProver::device_bytes() const { return m_->device_bytes(); }
void BatchProver::prove(const std::vector<Transcript *> &ts,
                        const std::vector<const uint32_t *> &polys, bool on_device, int n_claims,
                        bool commit_only, const std::function<void(int)> &finish) {
  m_->prove(ts, polys, on_device, n_claims, commit_only, finish);
}

}  // namespace whir
