// GPU WHIR prover host orchestration (see prover.h).
#include "prover.h"
#include "debug.h"
#include "host_math.h"
#include "svo_host.h"
#include "verifier.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <functional>
#include <map>
#include <thread>
#include <unordered_map>

namespace whir {

using kb::E4;
using namespace kb;

// ---------------- params (crates/whir/src/params.rs) ----------------
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
  double eta = ::pow(2., log_eta(s, lir));
  double rate = 1. / (double)(1u << lir);
  double delta = s == 0 ? 0.5 * (1. - rate) : s == 1 ? 1. - sqrt(rate) - eta : 1. - rate - eta;
  return log2(1. - delta);
}
// params.rs:118-122 converts with Rust's `as usize`, which saturates: NaN
// and negative values (rate 1, log_inv_rate 0, where log(1 - delta) is 0 or
// positive) give 0 queries.  Counts above MAX_STIR_QUERIES are refused (the
// pow-claim combination keeps one extension element per query in shared
// memory: 48 KB).
constexpr int MAX_STIR_QUERIES = 3072;
int n_stir_queries(int s, int security, int lir) {
  const double q = ceil(-(double)security / log_1_delta(s, lir));
  if (!(q > 0.)) return 0;
  if (q > (double)MAX_STIR_QUERIES) throw WhirError(-1, "STIR query count above 3072");
  return (int)q;
}
int n_ood_queries(int s, int security, int log_degree, int lir, int field_bits) {
  if (s == 0) return 0;
  for (int n = 1; n < 64; n++) {
    double err = 2. * list_size_bits(s, log_degree, lir) + (double)(log_degree * n);
    if ((double)(n * field_bits) + 1. - err >= (double)security) return n;
  }
  throw WhirError(-1, "could not find an appropriate number of OOD samples");
}
void number_of_rounds(int folding, int k, int *n_rounds, int *final_rounds) {
  if (k <= 6) {
    *n_rounds = 0;
    *final_rounds = k - folding;
    return;
  }
  int nr = (k - 6 + folding - 1) / folding;
  *final_rounds = k - nr * folding;
  *n_rounds = nr - 1;
}

uint32_t two_adic_generator(int bits) {
  uint32_t g = from_canonical(0x6ac49f88u);  // 3^127, order 2^24
  for (int i = bits; i < 24; i++) g = mul(g, g);
  return g;
}

static std::atomic<unsigned> g_debug{0};
void set_debug(unsigned flags) { g_debug.store(flags, std::memory_order_relaxed); }
unsigned debug_flags() { return g_debug.load(std::memory_order_relaxed); }

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess)
    throw WhirError(-2, std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------- device buffers, context ----------------
DeviceBuffer::~DeviceBuffer() {
  if (ptr_) cudaFree(ptr_);
}
void DeviceBuffer::reserve(size_t bytes) {
  if (bytes <= bytes_) return;
  if (ptr_) cudaFree(ptr_);
  ptr_ = nullptr;
  bytes_ = 0;
  cudaError_t e = cudaMalloc(&ptr_, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    ptr_ = nullptr;
    throw WhirError(-3, std::string("device allocation failed: ") + cudaGetErrorString(e));
  }
  bytes_ = bytes;
}

Context::Context(int device) : device_(device) {
  cuda_check(cudaSetDevice(device), "cudaSetDevice");
  int least = 0, greatest = 0;
  cuda_check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
  cuda_check(cudaStreamCreateWithPriority(&streams_[0], cudaStreamNonBlocking, least),
             "cudaStreamCreate");
  cuda_check(cudaStreamCreateWithPriority(&streams_[1], cudaStreamNonBlocking, greatest),
             "cudaStreamCreate");
  stream_ = streams_[0];
  cuda_check(gpu::init_device_tables(), "device tables");
  cuda_check(cudaMallocHost(&flag_, 64), "cudaMallocHost");
  *flag_ = 0;
}
Context::~Context() {
  cudaSetDevice(device_);
  for (auto &e : evs_) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  for (auto e : free_events_) cudaEventDestroy(e);
  if (block_ev_) cudaEventDestroy(block_ev_);
  if (flag_) cudaFreeHost(flag_);
  if (pinned_) cudaFreeHost(pinned_);
  for (auto s : streams_)
    if (s) cudaStreamDestroy(s);
}
void *Context::pinned(size_t bytes) {
  if (bytes > pinned_bytes_) {
    cuda_check(cudaStreamSynchronize(stream_), "sync");
    if (pinned_) cudaFreeHost(pinned_);
    pinned_ = nullptr;
    size_t n = std::max(bytes, (size_t)1 << 20);
    cuda_check(cudaMallocHost(&pinned_, n), "cudaMallocHost");
    pinned_bytes_ = n;
  }
  return pinned_;
}
void Context::wait_stream() {
  if (!yield_) {
    cuda_check(cudaStreamSynchronize(stream_), "stream sync");
    return;
  }
  // poll briefly, giving the core to other runnable threads between polls;
  // then sleep on a blocking-sync event so a waiting worker holds no core
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(stream_);
    if (e == cudaSuccess) return;
    if (e != cudaErrorNotReady) cuda_check(e, "stream sync");
    if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(20)) break;
    std::this_thread::yield();
  }
  if (!block_ev_)
    cuda_check(cudaEventCreateWithFlags(&block_ev_, cudaEventBlockingSync | cudaEventDisableTiming),
               "cudaEventCreate");
  cuda_check(cudaEventRecord(block_ev_, stream_), "cudaEventRecord");
  cuda_check(cudaEventSynchronize(block_ev_), "stream sync");
}
void Context::set_high_priority(bool on) {
  cudaStream_t want = streams_[on ? 1 : 0];
  if (want == stream_) return;
  cuda_check(cudaStreamSynchronize(stream_), "stream sync");
  stream_ = want;
}

void Context::wait_flag(unsigned int seq) {
  auto t0 = std::chrono::steady_clock::now();
  unsigned long spins = 0;
  while (__atomic_load_n(flag_, __ATOMIC_ACQUIRE) != seq) {
    // now and then make sure the stream is alive: a failed launch never
    // raises the flag, and a finished stream must have raised it
    if ((++spins & 4095) == 0) {
      cudaError_t e = cudaStreamQuery(stream_);
      if (e != cudaSuccess && e != cudaErrorNotReady) cuda_check(e, "stream");
      if (e == cudaSuccess && __atomic_load_n(flag_, __ATOMIC_ACQUIRE) != seq)
        throw WhirError(-5, "stream finished without raising the result flag");
    }
    if (yield_) std::this_thread::yield();
  }
  if (prof_on(K_SYNC)) {
    acc_ms_[K_SYNC] +=
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    acc_n_[K_SYNC] += 1;
  }
}

void Context::sync() {
  if (!prof_on(K_SYNC)) {
    wait_stream();
    return;
  }
  auto t0 = std::chrono::steady_clock::now();
  wait_stream();
  acc_ms_[K_SYNC] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  acc_n_[K_SYNC] += 1;
}

cudaEvent_t Context::take_event() {
  if (!free_events_.empty()) {
    cudaEvent_t e = free_events_.back();
    free_events_.pop_back();
    return e;
  }
  cudaEvent_t e;
  cuda_check(cudaEventCreate(&e), "cudaEventCreate");
  return e;
}
void Context::prof_begin(int klass) {
  if (!prof_on(klass)) return;
  open_klass_ = klass;
  open_ev_ = take_event();
  cudaEventRecord(open_ev_, stream_);
}
void Context::prof_end(int klass, double bytes) {
  if (!prof_on(klass) || open_klass_ != klass) return;
  cudaEvent_t b = take_event();
  cudaEventRecord(b, stream_);
  evs_.push_back(Ev{open_ev_, b, klass, bytes});
  open_klass_ = -1;
}
void Context::prof_read(int klass, double *ms, long *launches, double *bytes) {
  if (!evs_.empty()) {
    cuda_check(cudaStreamSynchronize(stream_), "stream sync");
    for (auto &e : evs_) {
      float t = 0;
      cudaEventElapsedTime(&t, e.a, e.b);
      acc_ms_[e.klass] += t;
      acc_n_[e.klass] += 1;
      acc_bytes_[e.klass] += e.bytes;
      free_events_.push_back(e.a);
      free_events_.push_back(e.b);
    }
    evs_.clear();
  }
  *ms = acc_ms_[klass];
  *launches = acc_n_[klass];
  *bytes = acc_bytes_[klass];
  acc_ms_[klass] = 0;
  acc_n_[klass] = 0;
  acc_bytes_[klass] = 0;
}

cudaError_t copy_async(Context &c, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind) {
  c.count_copy(bytes, kind);
  return cudaMemcpyAsync(dst, src, bytes, kind, c.stream());
}
void Context::count_copy(size_t bytes, int kind) {
  if (kind == cudaMemcpyHostToDevice) h2d_bytes_ += bytes;
  if (kind == cudaMemcpyDeviceToHost) d2h_bytes_ += bytes;
}


// ---------------- encode + commit ----------------
void encode_commit(Context &ctx, const uint32_t *src, int k, int rate, int folding, int dim,
                   uint32_t *codeword, uint32_t *scratch, uint32_t *nodes, DeviceTree *out) {
  Span span(dim == 1 ? "commit_base" : "commit_ext");  // whir.rs:19, 38
  cudaStream_t st = ctx.stream();
  int log_h = k + rate - folding;
  size_t width = (size_t)dim << folding, h_in = (size_t)1 << (k - folding);
  size_t rows = (size_t)1 << log_h;
  {
    Span dft(dim == 1 ? "dft-base" : "dft-ext");  // whir.rs:33, 58
    ctx.prof_begin(Context::K_DFT);
    cuda_check(gpu::dft_batch(src, h_in, width, log_h, codeword, scratch, st), "dft_batch");
    ctx.prof_end(Context::K_DFT, 4.0 * (double)(h_in * width + rows * width));
  }
  ctx.prof_begin(Context::K_LEAF);
  cuda_check(gpu::hash_rows(codeword, rows, (int)width, nodes, st), "hash_rows");
  ctx.prof_end(Context::K_LEAF, 4.0 * (double)(rows * width + rows * 8));
  // the last tree launch writes the root straight into pinned host memory
  uint32_t *h = (uint32_t *)ctx.pinned(64);
  unsigned int seq = ctx.next_seq();
  ctx.prof_begin(Context::K_TREE);
  cuda_check(gpu::build_tree(nodes, log_h, st, h, ctx.flag(), seq), "build_tree");
  ctx.prof_end(Context::K_TREE, 32.0 * (double)(2 * rows - 2 + rows - 1));
  if (log_h == 0) {  // a single leaf is the root; no tree launch ran
    cuda_check(copy_async(ctx, h, nodes, 32, cudaMemcpyDeviceToHost), "root copy");
    ctx.sync();
  } else {
    ctx.wait_flag(seq);  // the last tree launch raised it after writing the root
  }
  out->rows = codeword;
  out->nodes = nodes;
  out->log_h = log_h;
  out->row_len = (int)width;
  memcpy(out->root, h, 32);
}

// ---------------- prover state ----------------

// ProverStack::layout (crates/whir/src/sumcheck/prover.rs:92-124): polys
// placed largest first, each at an aligned offset; entries sorted by their
// selector bits as BTreeMap<Selector, _> orders them (Vec<bool>
// lexicographic).  Shared by the prover and the verifier.
std::vector<LayEntry> stack_layout(const std::vector<int> &pk, int k_expect, int folding) {
  int n = (int)pk.size();
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return pk[a] < pk[b]; });
  size_t total = 0;
  for (int i = 0; i < n; i++) total += (size_t)1 << pk[i];
  int k = 0;
  while (((size_t)1 << k) < total) k++;
  if (k != k_expect) throw WhirError(-1, "stacked layout size does not match params.k");
  if (k < folding) throw WhirError(-1, "k smaller than folding");
  // the reference's expression build fixes the low `folding` variables of
  // every stacked polynomial (compress_stacked, sumcheck/prover.rs:211-222,
  // asserts rs.k() <= k_poly with rs.k() = folding, whir.rs:184)
  for (int i = 0; i < n; i++)
    if (pk[i] < folding)
      throw WhirError(-1, "a stacked polynomial has fewer variables than the folding factor");
  std::vector<LayEntry> lay(n);
  size_t off = 0;
  for (int t = 0; t < n; t++) {
    int id = order[n - 1 - t];
    LayEntry &e = lay[t];
    e.poly = id;
    e.nbits = k - pk[id];
    e.index = off >> pk[id];
    for (int b = 0; b < e.nbits; b++) e.bits[b] = (e.index >> b) & 1;
    off += (size_t)1 << pk[id];
  }
  std::sort(lay.begin(), lay.end(), [](const LayEntry &a, const LayEntry &b) {
    int m = std::min(a.nbits, b.nbits);
    for (int i = 0; i < m; i++)
      if (a.bits[i] != b.bits[i]) return a.bits[i] < b.bits[i];
    return a.nbits < b.nbits;
  });
  return lay;
}

// crates/whir/src/whir.rs:150-166: the domain, folding and rates of round r
void round_params(const Params &p, int round, int *kfd, int *this_rate, int *prev_rate) {
  int prev_red = round == 0 ? 0 : p.initial_reduction + round - 1;
  int this_red = p.initial_reduction + round;
  int k_domain = p.rate + p.k - prev_red;
  *kfd = k_domain - p.folding;
  *prev_rate = p.rate + round * p.folding - prev_red;
  *this_rate = p.rate + (round + 1) * p.folding - this_red;
}

// Device buffers (bytes) a prover holds for one polynomial of 2^p.k
// evaluations: the base codeword and tree, the two alternating round
// codewords and trees, the DFT scratch, the sumcheck arrays, and small
// argument and reduction areas.
Workspace workspace_plan(const Params &p) {
  Workspace w;
  int k = p.k, f = p.folding;
  size_t cw0_words = ((size_t)1 << (k + p.rate - f)) << f;
  w.stacked = 4 * ((size_t)1 << k);
  w.cw0 = 4 * cw0_words;
  w.tree0 = 4 * gpu::tree_words(k + p.rate - f);
  int n_rounds, fin;
  number_of_rounds(f, k, &n_rounds, &fin);
  size_t max_cw = 16, max_tree = 8;
  for (int r = 0; r < n_rounds; r++) {
    int kfd, this_rate, prev_rate;
    round_params(p, r, &kfd, &this_rate, &prev_rate);
    int kp = k - f * (r + 1);
    int log_h = kp + this_rate - f;
    size_t words = ((size_t)4 << f) << log_h;
    max_cw = std::max(max_cw, words);
    max_tree = std::max(max_tree, gpu::tree_words(log_h));
  }
  w.scratch = 4 * std::max(cw0_words, max_cw);
  w.cw = 4 * max_cw;
  w.tree = 4 * max_tree;
  w.sumcheck = sizeof(kb::E4) * ((size_t)1 << (k - f));
  w.eqbuf = sizeof(kb::E4) * (size_t)64 * 8192;
  w.acc = 8 * 4096;
  w.small = 1 << 20;
  w.gather = (size_t)4 * 4096 * (((size_t)4 << f) + 8 * 32);
  // fold_with_code's per-query state (Impl::fold_with_code's layout) for
  // the most STIR queries any round draws, so that no proof grows it: a
  // cudaFree in the middle of a run synchronises every stream of the device
  size_t nq = 0;
  for (int r = 0; r <= n_rounds; r++) {
    int kfd, this_rate, prev_rate;
    round_params(p, r, &kfd, &this_rate, &prev_rate);
    nq = std::max(nq, (size_t)n_stir_queries(p.soundness, p.security_level, prev_rate));
  }
  const size_t T = (size_t)1 << f;
  w.code = 16 * nq * T + 16 * nq + 16 * ((nq + 3) & ~(size_t)3) + 4 * ((T + 3) & ~(size_t)3) +
           4 * nq * T + 64;
  return w;
}

// Upper bound of the proof length (the byte order of Whir::open,
// whir.rs:168-359): query hints counted before deduplication.
size_t proof_bytes_max(const Params &p, int n_claims) {
  size_t b = 32 + 16 * (size_t)n_claims;
  b += 16 * (size_t)n_ood_queries(p.soundness, p.security_level, p.k, p.rate, EXT_BITS);
  b += 32 * (size_t)p.folding;  // SVO rounds
  int n_rounds, fin;
  number_of_rounds(p.folding, p.k, &n_rounds, &fin);
  size_t prev_log_h = (size_t)(p.k + p.rate - p.folding), prev_row = (size_t)1 << p.folding;
  for (int r = 0; r <= n_rounds; r++) {
    int kfd, this_rate, prev_rate;
    round_params(p, r, &kfd, &this_rate, &prev_rate);
    int kc = p.k - p.folding * (r + 1);
    if (r < n_rounds) {
      b += 32 + 16 * (size_t)n_ood_queries(p.soundness, p.security_level, kc, this_rate, EXT_BITS);
    } else {
      b += (size_t)16 << fin;  // final polynomial
    }
    b += (size_t)n_stir_queries(p.soundness, p.security_level, prev_rate) * 4 *
         (prev_row + 8 * prev_log_h);
    if (r < n_rounds) {
      b += 32 * (size_t)p.folding;
      prev_log_h = (size_t)(kc + this_rate - p.folding);
      prev_row = (size_t)4 << p.folding;
    }
  }
  return b;
}

size_t workspace_union_bytes(const std::vector<Params> &ps) {
  Workspace u{};
  for (const Params &p : ps) {
    Workspace w = workspace_plan(p);
    u.stacked = std::max(u.stacked, w.stacked);
    u.cw0 = std::max(u.cw0, w.cw0);
    u.tree0 = std::max(u.tree0, w.tree0);
    u.scratch = std::max(u.scratch, w.scratch);
    u.cw = std::max(u.cw, w.cw);
    u.tree = std::max(u.tree, w.tree);
    u.sumcheck = std::max(u.sumcheck, w.sumcheck);
    u.eqbuf = std::max(u.eqbuf, w.eqbuf);
    u.acc = std::max(u.acc, w.acc);
    u.small = std::max(u.small, w.small);
    u.gather = std::max(u.gather, w.gather);
    u.code = std::max(u.code, w.code);
  }
  return u.total();
}

size_t Workspace::total() const {
  return stacked + cw0 + tree0 + scratch + 2 * (cw + tree + 2 * sumcheck) + eqbuf + acc + small +
         gather + code;
}

struct Prover::Impl {
  Context *ctx;
  Params p;
  int ks;
  // layout
  int n_polys = 0;
  std::vector<int> pk;
  std::vector<LayEntry> lay;
  std::vector<size_t> poly_off;  // word offset of each poly inside the stacked poly
  // device memory
  DeviceBuffer stacked, cw0, tree0, scratch, cw[2], trees[2], sp[2], sw[2], eqbuf, acc, small,
      gather, ptsbuf, codebuf;
  DeviceTree t0, tr[2];
  int cur_tree = -1;  // index into tr of the latest round commitment
  SvoTables svo;  // eq tables of the {0,1,2} grid per SVO round
  // pinned staging: `args` holds host->device arguments and is reused after
  // every sync; `defer` receives opening rows and row evaluations whose
  // device->host copies complete at a later sync (hints are filled into the
  // transcript at the end of the proof)
  PinnedBuffer args_pin, defer_pin;
  size_t args_off = 0, defer_off = 0;
  struct PendingHint {
    size_t ts_off, pin_off, words;
    // the opening's tree, for the debug check of its path
    uint32_t root[8];
    size_t index;
    int log_h, row_len;
  };
  std::vector<PendingHint> pending_hints;
  // claims
  std::vector<SvoClaim> claims;
  std::vector<VirtClaim> virt;
  // sumcheck state
  E4 sum, alpha;
  std::vector<E4> rs;
  int kc = 0;           // variables of the expression
  int ping = 0;         // sp[ping]/sw[ping] hold the arrays
  bool pending = false; // fold by pending_r not applied yet
  E4 pending_r;

  cudaStream_t st() const { return ctx->stream(); }

  size_t acc_size() const { return svo_acc_size(ks); }

  void sync() {
    ctx->sync();
    args_off = 0;
  }
  // reduction results land in the context's pinned area (see gpu::Publish);
  // the counter is the last word of acc
  static constexpr size_t PUB_WORDS = 1024;
  gpu::Publish publish(int words) {
    gpu::Publish p;
    p.counter = reinterpret_cast<unsigned int *>(acc.as<unsigned long long>() + acc.bytes() / 8 - 1);
    p.host = published();
    p.words = words;
    if ((size_t)words > PUB_WORDS) throw WhirError(-5, "reduction too wide to publish");
    p.flag = ctx->flag();
    p.seq = pub_seq = ctx->next_seq();
    args_mark = args_off;
    return p;
  }
  // waits for the last publish (its flag) instead of the stream; everything
  // queued before that launch has completed, so the argument space is free
  // again unless arguments were queued after it
  unsigned int pub_seq = 0;
  size_t args_mark = 0;
  void wait_published() {
    ctx->wait_flag(pub_seq);
    if (args_off == args_mark) args_off = 0;
  }
  unsigned long long *published() { return (unsigned long long *)ctx->pinned(8 * PUB_WORDS); }
  // pinned argument space for host->device copies issued before the next sync
  uint8_t *args_alloc(size_t bytes) {
    bytes = (bytes + 15) & ~(size_t)15;
    if (args_off + bytes > args_pin.bytes()) {
      sync();
      if (bytes > args_pin.bytes()) args_pin.reserve(std::max(bytes, (size_t)1 << 20));
    }
    uint8_t *p = args_pin.data() + args_off;
    args_off += bytes;
    return p;
  }
  // copy host bytes to `dst` (device) through the argument space
  void upload(void *dst, const void *src, size_t bytes) {
    if (bytes == 0) return;
    uint8_t *h = args_alloc(bytes);
    memcpy(h, src, bytes);
    cuda_check(copy_async(*ctx, dst, h, bytes, cudaMemcpyHostToDevice), "h2d");
  }
  // split eq tables of n points (k variables each, lo over the first s) with
  // per-table scales, written back to back at `out` (one upload, one launch)
  void make_eq_tables(const std::vector<const E4 *> &pts, int k, const std::vector<E4> &scales,
                      int s, E4 *out) {
    size_t n = pts.size();
    if (n == 0) return;
    if (n <= (size_t)gpu::EqArgs::N && k <= gpu::EqArgs::K) {  // by value: no upload
      gpu::EqArgs a;
      for (size_t t = 0; t < n; t++) {
        std::copy(pts[t], pts[t] + k, a.z + t * gpu::EqArgs::K);
        a.scale[t] = scales[t];
      }
      cuda_check(gpu::eq_tables_val(a, (int)n, k, s, out, st()), "eq_tables");
      return;
    }
    std::vector<E4> host(n * k + n);
    for (size_t t = 0; t < n; t++) {
      std::copy(pts[t], pts[t] + k, host.begin() + t * k);
      host[n * k + t] = scales[t];
    }
    size_t bytes = host.size() * sizeof(E4);
    if (bytes > ptsbuf.bytes()) ptsbuf.reserve(2 * bytes);
    upload(ptsbuf.as<E4>(), host.data(), bytes);
    cuda_check(gpu::eq_tables(ptsbuf.as<E4>(), ptsbuf.as<E4>() + n * k, (int)n, k, s, out, st()),
               "eq_tables");
  }
  void fill_pending_hints(Transcript &ts) {
    for (auto &h : pending_hints) {
      const uint32_t *w = reinterpret_cast<const uint32_t *>(defer_pin.data()) + h.pin_off;
      // MerkleTree::query's debug self-check (poseidon_packed.rs:158-230)
      if (debug_checks() &&
          !merkle_path_ok(h.root, h.index, w, (size_t)h.row_len, w + h.row_len, h.log_h))
        throw WhirError(-5, "debug check: an opened Merkle path does not hash to its root");
      ts.hint_fill(h.ts_off, w, h.words);
    }
    pending_hints.clear();
    defer_off = 0;
  }
  // Expression::prod == sum (prover.rs:346,558, expr.rs:68): the device
  // arrays' inner product against the running claimed sum, in debug mode
  void check_sum(const char *where) {
    if (!debug_checks()) return;
    flush();
    unsigned long long *a = acc.as<unsigned long long>();
    cuda_check(gpu::dot_ext(P(), W(), (size_t)1 << kc, a, st(), publish(4)), "dot");
    const unsigned long long *h = published();
    wait_published();
    if (!e_eq(reduce_acc(h), sum))
      throw WhirError(-5, std::string("debug check: <poly, weights> != sum after ") + where);
  }
  // The reference's debug-build STIR checks (crates/whir/src/whir.rs:263-264,
  // 287-288, 331-352): every opened row, folded at the round point, equals
  // the current polynomial evaluated at omega^index (omega of order 2^kfd).
  // In debug mode only: waits for the gathered rows and reads the polynomial
  // back (poly_host: the final polynomial, already on the host).
  void check_stir(const std::vector<size_t> &idx, int kfd, size_t rows_off, size_t per,
                  int row_len, bool base_rows, const std::vector<E4> &point,
                  const std::vector<E4> *poly_host) {
    if (!debug_checks() || idx.empty()) return;
    if (point.size() > 30 ||
        ((size_t)1 << point.size()) * (base_rows ? 1 : 4) != (size_t)row_len)
      throw WhirError(-5, "debug check: the round point does not match the opened rows");
    sync();
    std::vector<E4> poly;
    if (!poly_host) {
      poly.resize((size_t)1 << kc);
      E4 *h = (E4 *)ctx->pinned(16 * poly.size());
      cuda_check(copy_async(*ctx, h, P(), 16 * poly.size(), cudaMemcpyDeviceToHost), "d2h");
      sync();
      std::copy(h, h + poly.size(), poly.begin());
      poly_host = &poly;
    }
    const size_t n = (size_t)1 << point.size();
    std::vector<E4> eq(n);
    eq_host(point.data(), (int)point.size(), e_one(), eq.data());
    const uint32_t omega = two_adic_generator(kfd);
    for (size_t i = 0; i < idx.size(); i++) {
      const uint32_t *row = defer_ptr(rows_off + per * i);
      const E4 e = base_rows ? dot_eq_base(eq.data(), row, n)
                             : dot_eq_ext(eq.data(), reinterpret_cast<const E4 *>(row), n);
      const E4 want = horner_base(poly_host->data(), poly_host->size(), kb::pow(omega, idx[i]));
      if (!e_eq(e, want))
        throw WhirError(-5, "debug check: an opened row does not fold to the polynomial's "
                            "value at its point");
    }
  }
  // pinned space (in words) for device->host results read after a later sync
  size_t defer_alloc(size_t words, Transcript &ts) {
    words = (words + 3) & ~(size_t)3;
    if (4 * (defer_off + words) > defer_pin.bytes()) {
      sync();  // everything pending has landed: emit it and start over
      fill_pending_hints(ts);
      if (4 * words > defer_pin.bytes()) defer_pin.reserve(std::max(4 * words, (size_t)16 << 20));
    }
    size_t off = defer_off;
    defer_off += words;
    return off;
  }
  uint32_t *defer_ptr(size_t off) { return reinterpret_cast<uint32_t *>(defer_pin.data()) + off; }

  // ---- layout (ProverStack::layout, prover.rs:92-124) ----
  void make_layout() {
    lay = stack_layout(pk, p.k, ks);
    poly_off.assign(n_polys, 0);
    for (auto &e : lay) poly_off[e.poly] = e.index << pk[e.poly];
  }

  // ---- workspace ----
  void reserve() {
    Workspace w = workspace_plan(p);
    stacked.reserve(w.stacked);
    cw0.reserve(w.cw0);
    tree0.reserve(w.tree0);
    scratch.reserve(w.scratch);
    for (int i = 0; i < 2; i++) {
      cw[i].reserve(w.cw);
      trees[i].reserve(w.tree);
      sp[i].reserve(w.sumcheck);
      sw[i].reserve(w.sumcheck);
    }
    eqbuf.reserve(w.eqbuf);
    args_pin.reserve((size_t)1 << 20);
    ptsbuf.reserve(64 << 10);
    defer_pin.reserve((size_t)16 << 20);
    acc.reserve(w.acc);
    small.reserve(w.small);
    gather.reserve(w.gather);
    codebuf.reserve(w.code);
  }

  void round_params(int round, int *kfd, int *this_rate, int *prev_rate) const {
    whir::round_params(p, round, kfd, this_rate, prev_rate);
  }

  // ---- SVO claim (SvoPoint::new + eval, svo.rs:64-91) ----
  void svo_claim(SvoClaim &c, const uint32_t *poly_dev, int kp, const E4 *point) {
    c.k = kp;
    c.point.assign(point, point + kp);
    int nz = kp - ks;
    int s_lo = std::min(8, nz);  // 2^(nz-8) CTAs: enough loads in flight
    E4 *lo = eqbuf.as<E4>(), *hi = lo + ((size_t)1 << s_lo);
    make_eq_tables({point + ks}, nz, {e_one()}, s_lo, lo);
    size_t na = (size_t)4 << ks;
    unsigned long long *a = acc.as<unsigned long long>();
    ctx->prof_begin(Context::K_SUMCHECK);
    cuda_check(gpu::compress_hi(poly_dev, kp, ks, lo, s_lo, hi, a, st(), publish((int)na)),
               "compress_hi");
    ctx->prof_end(Context::K_SUMCHECK, 4.0 * (double)((size_t)1 << kp));
    const unsigned long long *h = published();
    wait_published();
    svo_finish(c, ks, h);
  }

  const uint32_t *poly_dev(int id) const { return stacked.as<uint32_t>() + poly_off[id]; }

  // claims in layout order: (claim index, layout entry)
  std::vector<std::pair<int, int>> claims_layout_order() const {
    std::vector<std::pair<int, int>> v;
    for (int e = 0; e < n_polys; e++)
      for (int c = 0; c < (int)claims.size(); c++)
        if (claims[c].poly == lay[e].poly) v.push_back({c, e});
    return v;
  }

  // ---- write_virtual_eval (prover.rs:232-277) ----
  void write_virtual_eval(Transcript &ts) {
    Span span("write_virtual_eval");  // sumcheck/prover.rs:231
    VirtClaim v;
    v.point.resize(p.k);
    expand(v.point.data(), p.k, ts.draw_ext());
    v.eval = e_zero();
    v.acc.assign(acc_size(), e_zero());
    for (int e = 0; e < n_polys; e++) {
      int id = lay[e].poly, kp = pk[id];
      E4 sel[32];
      for (int b = 0; b < lay[e].nbits; b++) sel[b] = lay[e].bits[b] ? e_one() : e_zero();
      E4 weight = eval_eq_xy(sel, v.point.data() + kp, lay[e].nbits);
      SvoClaim c;
      svo_claim(c, poly_dev(id), kp, v.point.data());
      v.eval = e_add(v.eval, e_mul(weight, c.eval));
      svo.accumulate(v.acc, c, weight, ks);
    }
    // the debug-build check of ProverLayout::write_virtual_eval
    // (crates/whir/src/sumcheck/prover.rs:257-266): the same claim made
    // directly on the stacked polynomial gives the same evaluation and SVO
    // accumulators
    if (debug_checks()) {
      SvoClaim d;
      svo_claim(d, stacked.as<uint32_t>(), p.k, v.point.data());
      std::vector<E4> acc2(acc_size(), e_zero());
      svo.accumulate(acc2, d, e_one(), ks);
      bool same = e_eq(d.eval, v.eval);
      for (size_t i = 0; same && i < acc2.size(); i++) same = e_eq(acc2[i], v.acc[i]);
      if (!same)
        throw WhirError(-5, "debug check: the virtual claim differs from the claim on the "
                            "stacked polynomial");
    }
    ts.write_ext(v.eval);
    virt.push_back(std::move(v));
  }

  // ---- sumcheck arrays on the device ----
  E4 *P() { return sp[ping].as<E4>(); }
  E4 *W() { return sw[ping].as<E4>(); }

  // (c0, c2) of the current arrays, applying a pending fold in the same pass;
  // coeffs_begin queues the pass and the read-back, coeffs_end waits for them
  // (host work in between overlaps the pass)
  void coeffs(E4 *c0, E4 *c2) {
    coeffs_begin();
    coeffs_end(c0, c2);
  }
  void coeffs_end(E4 *c0, E4 *c2, E4 *extra = nullptr) {
    const unsigned long long *h = published();
    wait_published();
    *c0 = reduce_acc(h);
    *c2 = reduce_acc(h + 4);
    if (extra) *extra = reduce_acc(h + 8);
  }
  // code: fold_with_code's per-query pass of this round, added into the same
  // slots (and its round-0 sum term into slots 8..12)
  void coeffs_begin(const gpu::CodeState *code = nullptr, int code_round = 0,
                    E4 code_r = E4{}) {
    unsigned long long *a = acc.as<unsigned long long>();
    // the last reducing launch publishes the sums to pinned memory and
    // re-zeroes them (no memset, no copy); with no queries (rate 1) there is
    // no code pass and the round pass publishes
    if (code && code->n == 0) code = nullptr;
    gpu::Publish pub = publish(12);
    gpu::Publish none;
    size_t n = (size_t)1 << kc;
    ctx->prof_begin(Context::K_SUMCHECK);
    if (pending) {
      cuda_check(gpu::sumcheck_round(P(), W(), 2 * n, true, pending_r, sp[1 - ping].as<E4>(),
                                     sw[1 - ping].as<E4>(), true, a, st(), code ? none : pub),
                 "round");
      ping = 1 - ping;
      pending = false;
      ctx->prof_end(Context::K_SUMCHECK, 3.0 * 2 * 16 * (double)n);
    } else {
      cuda_check(gpu::sumcheck_round(P(), W(), n, false, e_zero(), nullptr, nullptr, true, a, st(),
                                     code ? none : pub),
                 "round");
      ctx->prof_end(Context::K_SUMCHECK, 2 * 16 * (double)n);
    }
    if (code) cuda_check(gpu::code_round(*code, code_round, code_r, a, st(), pub), "code_round");
  }
  void flush() {
    if (!pending) return;
    size_t n = (size_t)1 << kc;
    cuda_check(gpu::sumcheck_round(P(), W(), 2 * n, true, pending_r, sp[1 - ping].as<E4>(),
                                   sw[1 - ping].as<E4>(), false, nullptr, st()),
               "fold");
    ping = 1 - ping;
    pending = false;
  }
  void defer_fold(const E4 &r) {  // Expression::fix_var (expr.rs:101-104)
    pending = true;
    pending_r = r;
    kc -= 1;
  }
  // Expression::round (expr.rs:52-70)
  E4 round(Transcript &ts) {
    E4 c0, c2;
    coeffs(&c0, &c2);
    ts.write_ext(c0);
    ts.write_ext(c2);
    E4 r = ts.draw_ext();
    defer_fold(r);
    sum = extrapolate012(c0, e_sub(sum, c0), c2, r);
    return r;
  }

  // w[off .. off + 2^kt) += eq(point) * scale for several points sharing the range
  void add_eqs(E4 *w, int kt, const std::vector<std::vector<E4>> &pts, const std::vector<E4> &scales) {
    if (pts.empty()) return;
    int s = kt / 2;
    size_t per = ((size_t)1 << s) + ((size_t)1 << (kt - s));
    if (per * pts.size() * sizeof(E4) > eqbuf.bytes())
      eqbuf.reserve(per * pts.size() * sizeof(E4));
    std::vector<const E4 *> pp;
    for (auto &q : pts) pp.push_back(q.data());
    make_eq_tables(pp, kt, scales, s, eqbuf.as<E4>());
    cuda_check(gpu::add_eq(w, kt, eqbuf.as<E4>(), (int)pts.size(), st()), "add_eq");
  }

  // w += sum_t scales_t var_t^i; arguments go through the pinned argument
  // space, so no sync is needed here
  void add_pows(const std::vector<uint32_t> &vars, const std::vector<E4> &scales) {
    if (vars.empty()) return;
    if (vars.size() <= (size_t)gpu::PowArgs::N) {  // by value: no upload
      static thread_local gpu::PowArgs a;
      std::copy(vars.begin(), vars.end(), a.vars);
      std::copy(scales.begin(), scales.end(), a.scales);
      size_t tw = gpu::add_pows_scratch_words(kc, (int)vars.size());
      if (4 * tw > eqbuf.bytes()) eqbuf.reserve(4 * tw);
      cuda_check(gpu::add_pows_val(W(), kc, a, (int)vars.size(), eqbuf.as<uint32_t>(), st()),
                 "add_pows");
      return;
    }
    size_t bytes = vars.size() * 4 + scales.size() * 16;
    std::vector<uint8_t> h(bytes);
    memcpy(h.data(), scales.data(), scales.size() * 16);
    memcpy(h.data() + scales.size() * 16, vars.data(), vars.size() * 4);
    if (bytes > small.bytes()) small.reserve(2 * bytes);
    upload(small.as<uint8_t>(), h.data(), bytes);
    size_t tw = gpu::add_pows_scratch_words(kc, (int)vars.size());
    if (4 * tw > eqbuf.bytes()) eqbuf.reserve(4 * tw);
    cuda_check(gpu::add_pows(W(), kc, (const uint32_t *)(small.as<uint8_t>() + scales.size() * 16),
                             small.as<E4>(), (int)vars.size(), eqbuf.as<uint32_t>(), st()),
               "add_pows");
  }

  // add_pows with vars and scales already on the device
  void add_pows_dev(const uint32_t *vars, const E4 *scales, int n) {
    if (n == 0) return;
    size_t tw = gpu::add_pows_scratch_words(kc, n);
    if (4 * tw > eqbuf.bytes()) eqbuf.reserve(4 * tw);
    cuda_check(gpu::add_pows(W(), kc, vars, scales, n, eqbuf.as<uint32_t>(), st()), "add_pows");
  }

  // ---- new_prover (prover.rs:280-354) incl. expression (185-229) ----
  void new_prover(Transcript &ts) {
    Span span("new_prover");  // sumcheck/prover.rs:279
    alpha = ts.draw_ext();
    auto order = claims_layout_order();
    int n = (int)claims.size();
    std::vector<E4> alphas(n), evals;
    E4 a = e_one();
    for (auto &oe : order) {
      alphas[oe.first] = a;
      evals.push_back(claims[oe.first].eval);
      a = e_mul(a, alpha);
    }
    for (auto &v : virt) evals.push_back(v.eval);
    sum = horner(evals.data(), evals.size(), alpha);
    std::vector<E4> accv(acc_size(), e_zero());
    for (int c = 0; c < n; c++) svo.accumulate(accv, claims[c], alphas[c], ks);
    E4 av = e_pow(alpha, (uint64_t)n);
    for (auto &v : virt) {
      for (size_t i = 0; i < accv.size(); i++) accv[i] = e_add(accv[i], e_mul(av, v.acc[i]));
      av = e_mul(av, alpha);
    }
    rs.clear();
    svo_rounds(ts, accv, ks, sum, rs);
    // expression: compress_stacked (compress_lo_into per poly) + combine_eqs
    kc = p.k - ks;
    ping = 0;
    pending = false;
    size_t N = (size_t)1 << kc;
    gpu::Point rsp;
    rsp.k = ks;
    for (int i = 0; i < ks; i++) rsp.z[i] = rs[i];
    if (n_polys > 1) cuda_check(cudaMemsetAsync(P(), 0, N * sizeof(E4), st()), "memset");
    for (int e = 0; e < n_polys; e++) {
      int id = lay[e].poly;
      size_t o = lay[e].index << (pk[id] - ks);
      cuda_check(gpu::compress_lo(poly_dev(id), pk[id], rsp, P() + o, st()), "compress_lo");
    }
    cuda_check(cudaMemsetAsync(W(), 0, N * sizeof(E4), st()), "memset");
    // group the eq additions by target range
    std::map<std::pair<size_t, int>, std::pair<std::vector<std::vector<E4>>, std::vector<E4>>> groups;
    a = e_one();
    for (auto &oe : order) {
      const SvoClaim &c = claims[oe.first];
      int ksplit = c.k - ks;
      size_t o = lay[oe.second].index << ksplit;
      E4 scale = e_mul(a, eval_eq_xy(c.point.data(), rs.data(), ks));
      auto &g = groups[{o, ksplit}];
      g.first.emplace_back(c.point.begin() + ks, c.point.end());
      g.second.push_back(scale);
      a = e_mul(a, alpha);
    }
    for (auto &v : virt) {
      E4 scale = e_mul(a, eval_eq_xy(v.point.data(), rs.data(), ks));
      auto &g = groups[{0, kc}];
      g.first.emplace_back(v.point.begin() + ks, v.point.end());
      g.second.push_back(scale);
      a = e_mul(a, alpha);
    }
    for (auto &kv : groups) add_eqs(W() + kv.first.first, kv.first.second, kv.second.first, kv.second.second);
    check_sum("new_prover");
  }

  // ---- queries (MerkleTree::query, poseidon_packed.rs:145-233) ----
  // Reserves the leaf + sibling hints of each index in the transcript and
  // starts their gather; the rows land in the deferred pinned area (word
  // offset returned, `per` words per index) and are readable after the next
  // sync; the hint bytes are filled in at the end of the proof.
  size_t query_async(Transcript &ts, const DeviceTree &t, const std::vector<size_t> &idx) {
    int n = (int)idx.size();
    if (n == 0) return 0;
    size_t per = (size_t)t.row_len + 8 * (size_t)t.log_h;
    // the gather writes the hint words straight into the deferred pinned area
    size_t off = defer_alloc(per * n, ts);
    if (n <= gpu::IdxArgs::N) {  // indexes by value: no upload
      static thread_local gpu::IdxArgs a;
      for (int i = 0; i < n; i++) a.idx[i] = (uint32_t)idx[i];
      cuda_check(gpu::gather_openings_val(t.rows, t.row_len, t.nodes, t.log_h, a, n,
                                          defer_ptr(off), st()),
                 "gather");
    } else {
      size_t need = 4 * (size_t)n + 16;
      if (need > gather.bytes()) {
        sync();  // an earlier gather may still be in flight
        gather.reserve(2 * need);
      }
      std::vector<uint32_t> hidx(n);
      for (int i = 0; i < n; i++) hidx[i] = (uint32_t)idx[i];
      uint32_t *didx = gather.as<uint32_t>();
      upload(didx, hidx.data(), 4 * (size_t)n);
      cuda_check(gpu::gather_openings(t.rows, t.row_len, t.nodes, t.log_h, didx, n,
                                      defer_ptr(off), st()),
                 "gather");
    }
    ctx->count_copy(4 * per * n, cudaMemcpyDeviceToHost);
    for (int i = 0; i < n; i++) {
      PendingHint h{ts.hint_reserve(per), off + per * i, per, {}, idx[i], t.log_h, t.row_len};
      memcpy(h.root, t.root, 32);
      pending_hints.push_back(h);
    }
    return off;
  }

  std::vector<size_t> stir_indexes(Transcript &ts, int bits, int n) {  // whir.rs:64-77
    Span span("stir_indexes");  // whir.rs:63
    std::vector<size_t> v(n);
    for (int i = 0; i < n; i++) v[i] = ts.draw_bits(bits);
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    return v;
  }

  // ---- fold (prover.rs:378-397) ----
  // The pow-claim evaluations come from opening rows still in flight
  // (rows_off in the deferred area); they only enter `sum`, which is first
  // needed after the first round's coefficients are read back, so they are
  // evaluated after that sync.
  std::vector<E4> fold(Transcript &ts, const std::vector<std::vector<E4>> &eq_pts,
                       const std::vector<E4> &eq_evals, const std::vector<uint32_t> &vars,
                       size_t rows_off, size_t per, int row_len, const std::vector<E4> &point) {
    Span span("fold");  // sumcheck/prover.rs:377
    alpha = ts.draw_ext();
    flush();
    std::vector<E4> sc;
    E4 a = e_one();
    for (size_t i = 0; i < eq_pts.size(); i++) {
      sc.push_back(a);
      a = e_mul(a, alpha);
    }
    add_eqs(W(), kc, eq_pts, sc);
    std::vector<E4> ps;
    for (size_t i = 0; i < vars.size(); i++) {
      ps.push_back(a);
      a = e_mul(a, alpha);
    }
    add_pows(vars, ps);
    std::vector<E4> out;
    for (int i = 0; i < p.folding; i++) {
      E4 c0, c2;
      coeffs(&c0, &c2);
      if (i == 0) {  // combine_claims' sum update (combine.rs:49-53)
        std::vector<E4> ev(eq_evals);
        for (size_t q = 0; q < vars.size(); q++)
          ev.push_back(eval_ext_small(reinterpret_cast<const E4 *>(defer_ptr(rows_off + per * q)),
                                      p.folding, point.data()));
        sum = e_add(sum, horner(ev.data(), ev.size(), alpha));
      }
      ts.write_ext(c0);
      ts.write_ext(c2);
      E4 r = ts.draw_ext();
      defer_fold(r);
      sum = extrapolate012(c0, e_sub(sum, c0), c2, r);
      out.push_back(r);
      rs.push_back(r);
      check_sum("a fold round");
    }
    (void)row_len;
    return out;
  }

  // ---- fold_with_code (prover.rs:400-561) ----
  std::vector<E4> fold_with_code(Transcript &ts, const std::vector<std::vector<E4>> &eq_pts,
                                 const std::vector<E4> &eq_evals, const std::vector<size_t> &idx) {
    Span span("fold_with_code");  // sumcheck/prover.rs:399
    int d = p.folding;
    alpha = ts.draw_ext();
    int k_data = t0.log_h;
    sum = e_add(sum, horner(eq_evals.data(), eq_evals.size(), alpha));
    flush();
    std::vector<E4> sc;
    E4 a = e_one();
    for (size_t i = 0; i < eq_pts.size(); i++) {
      sc.push_back(a);
      a = e_mul(a, alpha);
    }
    add_eqs(W(), kc, eq_pts, sc);
    int n = (int)idx.size();
    std::vector<E4> scales(n);
    for (int i = 0; i < n; i++) {
      scales[i] = a;
      a = e_mul(a, alpha);
    }
    // The recursion g (prover.rs:437-461) of one query reads, at round r,
    // g(r, .) at two positions; all of them lie on the 2^d rows base + t S
    // (S = 2^(k_data - d), base = idx mod S, t < 2^d), the recursive indexes
    // of prover.rs:483-495.  The device keeps g per query and folds it round
    // by round (gpu::code_round); the round's part of (c0, c2) lands in the
    // same reduction slots as the expression's, so the host reads them with
    // one sync per round as in a plain round.
    if (k_data < d) throw WhirError(-1, "codeword shorter than the folding");
    const int lS = k_data - d;
    const size_t S = (size_t)1 << lS, T = (size_t)1 << d;
    gpu::CodeState cs;
    cs.n = n;
    cs.d = d;
    cs.k_data = k_data;
    cs.omega = two_adic_generator(k_data);
    cs.winv = inv(cs.omega);
    cs.two_inv = inv(from_canonical(2));
    // device layout in codebuf: G | scales | idx | ws | tw | B | wd | row list
    size_t g_bytes = 16 * (size_t)n * T, sc_bytes = 16 * (size_t)n, u_bytes = 4 * (((size_t)n + 3) & ~(size_t)3);
    size_t wd_bytes = 4 * ((T + 3) & ~(size_t)3), rl_bytes = 4 * (size_t)n * T;
    size_t need = g_bytes + sc_bytes + 4 * u_bytes + wd_bytes + rl_bytes + 64;
    if (need > codebuf.bytes()) {
      sync();
      codebuf.reserve(2 * need);
    }
    uint8_t *cb = codebuf.as<uint8_t>();
    cs.G = reinterpret_cast<E4 *>(cb);
    cs.scales = reinterpret_cast<E4 *>(cb + g_bytes);
    uint32_t *didx = reinterpret_cast<uint32_t *>(cb + g_bytes + sc_bytes);
    cs.idx = didx;
    cs.ws = didx + u_bytes / 4;
    cs.tw = cs.ws + u_bytes / 4;
    cs.B = cs.tw + u_bytes / 4;
    uint32_t *dwd = cs.B + u_bytes / 4;
    cs.wd = dwd;
    uint32_t *drows = dwd + wd_bytes / 4;
    {
      std::vector<uint32_t> h((size_t)n * T), hi(n), hw(T);
      for (int i = 0; i < n; i++) {
        hi[i] = (uint32_t)idx[i];
        for (size_t t = 0; t < T; t++) h[(size_t)i * T + t] = (uint32_t)((idx[i] & (S - 1)) + t * S);
      }
      uint32_t wd = kb::pow(cs.winv, S);
      hw[0] = ONE;
      for (size_t t = 1; t < T; t++) hw[t] = mul(hw[t - 1], wd);
      upload(drows, h.data(), 4 * h.size());
      upload(didx, hi.data(), 4 * (size_t)n);
      upload(dwd, hw.data(), 4 * T);
      upload(cs.scales, scales.data(), 16 * (size_t)n);
    }
    gpu::Point rsp;
    rsp.k = (int)rs.size();
    for (size_t i = 0; i < rs.size(); i++) rsp.z[i] = rs[i];
    // G_0: row evaluations at eq(rs), written in place (query-major)
    cuda_check(gpu::row_evals(t0.rows, t0.row_len, drows, (int)((size_t)n * T), rsp, cs.G, st()),
               "row_evals");
    std::vector<E4> rc;  // rs of this call
    for (int round = 0; round < d; round++) {
      E4 c0, c2, sum_add;
      coeffs_begin(&cs, round, round ? rc[round - 1] : e_zero());
      coeffs_end(&c0, &c2, &sum_add);
      if (round == 0) sum = e_add(sum, sum_add);  // prover.rs:426-435
      ts.write_ext(c0);
      ts.write_ext(c2);
      E4 r = ts.draw_ext();
      sum = extrapolate012(c0, e_sub(sum, c0), c2, r);
      rc.push_back(r);
      defer_fold(r);
    }
    cuda_check(gpu::code_finish(cs, rc.back(), st()), "code_finish");
    flush();
    add_pows_dev(cs.ws, cs.scales, n);  // combine_pows_scaled (combine.rs:441-468)
    check_sum("fold_with_code");
    for (auto &r : rc) rs.push_back(r);
    return rc;
  }

  // ---- Whir::open (whir.rs:168-359) ----
  void open(Transcript &ts) {
    pending_hints.clear();
    defer_off = 0;
    int n_ood = n_ood_queries(p.soundness, p.security_level, p.k, p.rate, EXT_BITS);
    {
      Span span("ood claims");  // whir.rs:187
      for (int i = 0; i < n_ood; i++) write_virtual_eval(ts);
    }
    new_prover(ts);
    int n_rounds, final_rounds;
    number_of_rounds(p.folding, p.k, &n_rounds, &final_rounds);
    cur_tree = -1;
    std::vector<E4> round_point;
    for (int round = 0; round < n_rounds; round++) {
      Span round_span("round");  // whir.rs:206
      int kfd, this_rate, prev_rate;
      round_params(round, &kfd, &this_rate, &prev_rate);
      flush();
      int slot = cur_tree < 0 ? 0 : 1 - cur_tree;
      encode_commit(*ctx, reinterpret_cast<const uint32_t *>(P()), kc, this_rate, p.folding, 4,
                    cw[slot].as<uint32_t>(), scratch.as<uint32_t>(), trees[slot].as<uint32_t>(),
                    &tr[slot]);
      ts.write_digest(tr[slot].root);
      int n_o = n_ood_queries(p.soundness, p.security_level, kc, this_rate, EXT_BITS);
      std::vector<std::vector<E4>> pts;
      std::vector<E4> evs;
      Span ood_span("ood claims in round");  // whir.rs:224
      for (int i = 0; i < n_o; i++) {
        std::vector<E4> pt(kc);
        expand(pt.data(), kc, ts.draw_ext());
        E4 e = eval_poly(pt);
        ts.write_ext(e);
        pts.push_back(std::move(pt));
        evs.push_back(e);
      }
      int n_s = n_stir_queries(p.soundness, p.security_level, prev_rate);
      Span stir_span("stir claims");  // whir.rs:250
      std::vector<size_t> idx = stir_indexes(ts, kfd, n_s);
      std::vector<E4> rnew;
      if (round == 0) {
        size_t rows_off = query_async(ts, t0, idx);
        check_stir(idx, kfd, rows_off, (size_t)t0.row_len + 8 * (size_t)t0.log_h, t0.row_len,
                   true, rs, nullptr);
        rnew = fold_with_code(ts, pts, evs, idx);
      } else {
        const DeviceTree &prev = tr[cur_tree];
        size_t rows_off = query_async(ts, prev, idx);
        size_t per = (size_t)prev.row_len + 8 * (size_t)prev.log_h;
        check_stir(idx, kfd, rows_off, per, prev.row_len, false, round_point, nullptr);
        uint32_t omega = two_adic_generator(kfd);
        std::vector<uint32_t> vars(idx.size());
        for (size_t i = 0; i < idx.size(); i++) vars[i] = kb::pow(omega, idx[i]);
        rnew = fold(ts, pts, evs, vars, rows_off, per, prev.row_len, round_point);
      }
      round_point = rnew;
      cur_tree = slot;
    }
    Span final_span("final");  // whir.rs:314
    flush();
    size_t nf = (size_t)1 << kc;
    E4 *hf = (E4 *)ctx->pinned(16 * nf);
    cuda_check(copy_async(*ctx, hf, P(), 16 * nf, cudaMemcpyDeviceToHost), "d2h");
    sync();
    std::vector<E4> fp(hf, hf + nf);
    for (auto &e : fp) ts.write_ext(e);
    int kfd, this_rate, prev_rate;
    round_params(n_rounds, &kfd, &this_rate, &prev_rate);
    int n_s = n_stir_queries(p.soundness, p.security_level, prev_rate);
    std::vector<size_t> idx = stir_indexes(ts, kfd, n_s);
    const DeviceTree &last = cur_tree >= 0 ? tr[cur_tree] : t0;
    size_t rows_off = query_async(ts, last, idx);
    sync();
    check_stir(idx, kfd, rows_off, (size_t)last.row_len + 8 * (size_t)last.log_h, last.row_len,
               cur_tree < 0, cur_tree >= 0 ? round_point : rs, &fp);
    fill_pending_hints(ts);
    if (kc != final_rounds) throw WhirError(-1, "final sumcheck size mismatch");
  }

  // Poly::eval_ext on the current expression poly (SplitEq::eval_ext)
  E4 eval_poly(const std::vector<E4> &pt) {
    int k = kc;
    if (k == 0) {
      E4 *h = (E4 *)ctx->pinned(16);
      cuda_check(copy_async(*ctx, h, P(), 16, cudaMemcpyDeviceToHost), "d2h");
      sync();
      return *h;
    }
    int s_lo = std::min(10, k);
    E4 *lo = eqbuf.as<E4>(), *hi = lo + ((size_t)1 << s_lo);
    make_eq_tables({pt.data()}, k, {e_one()}, s_lo, lo);
    unsigned long long *a = acc.as<unsigned long long>();
    cuda_check(gpu::eval_ext(P(), k, lo, s_lo, hi, a, st(), publish(4)), "eval_ext");
    const unsigned long long *h = published();
    wait_published();
    return reduce_acc(h);
  }
};

void check_params(const Params &p) {
  if (p.folding < 1 || p.folding > 8 || p.k < p.folding || p.k > 26 || p.rate < 0 ||
      p.rate > 8 || p.initial_reduction < 1 || p.soundness < 0 || p.soundness > 2 ||
      p.security_level < 0)
    throw WhirError(-1, "invalid WHIR parameters");
  // every codeword lies on a subgroup of KoalaBear's 2^24 two-adic group
  if (p.k + p.rate - p.folding > 24)
    throw WhirError(-1, "invalid WHIR parameters: codeword above 2^24 rows");
  // the reference computes the round shapes in usize (params.rs:186-202,
  // whir.rs:150-166), where a negative result panics: refuse those sets
  // (e.g. an initial_reduction above rate + folding, or a folding that
  // leaves a negative number of final sumcheck rounds)
  int n_rounds, fin;
  number_of_rounds(p.folding, p.k, &n_rounds, &fin);
  if (fin < 0) throw WhirError(-1, "invalid WHIR parameters: negative final sumcheck rounds");
  for (int r = 0; r <= n_rounds; r++) {
    int kfd, this_rate, prev_rate;
    round_params(p, r, &kfd, &this_rate, &prev_rate);
    if (kfd < 0 || this_rate < 0 || prev_rate < 0)
      throw WhirError(-1, "invalid WHIR parameters: a round's domain or rate is negative");
    if (r < n_rounds && p.k - p.folding * (r + 1) + this_rate - p.folding > 24)
      throw WhirError(-1, "invalid WHIR parameters: codeword above 2^24 rows");
  }
}

Prover::Prover(Context *ctx, const Params &p) : m_(new Impl), ctx_(ctx), p_(p) {
  check_params(p);
  m_->ctx = ctx;
  m_->p = p;
  m_->ks = p.folding;
}

void Prover::set_params(const Params &p) {
  check_params(p);
  p_ = p;
  m_->p = p;
  m_->ks = p.folding;
}

void Prover::reserve() { m_->reserve(); }

size_t Prover::workspace_bytes(const Params &p) {
  check_params(p);
  return workspace_plan(p).total();
}
Prover::~Prover() { delete m_; }

size_t Prover::device_bytes() const {
  size_t s = 0;
  const DeviceBuffer *bufs[] = {&m_->stacked, &m_->cw0,   &m_->tree0,  &m_->scratch,
                                &m_->cw[0],   &m_->cw[1], &m_->trees[0], &m_->trees[1],
                                &m_->sp[0],   &m_->sp[1], &m_->sw[0],  &m_->sw[1],
                                &m_->eqbuf,   &m_->acc,   &m_->small,  &m_->gather,
                                &m_->codebuf};
  for (auto b : bufs) s += b->bytes();
  return s;
}

void Prover::commit(Transcript &ts, const uint32_t *polys, bool on_device,
                    const std::vector<int> &poly_k) {
  Impl &m = *m_;
  m.n_polys = (int)poly_k.size();
  if (m.n_polys == 0) throw WhirError(-1, "no polynomials");
  m.pk = poly_k;
  m.make_layout();
  m.reserve();
  // reductions publish and re-zero their accumulators (Impl::publish); start
  // every proof from zero
  cuda_check(cudaMemsetAsync(m.acc.as<void>(), 0, m.acc.bytes(), ctx_->stream()), "memset");
  m.claims.clear();
  m.virt.clear();
  cudaStream_t st = ctx_->stream();
  size_t total = (size_t)1 << p_.k;
  uint32_t *stk = m.stacked.as<uint32_t>();
  if (m.n_polys > 1) cuda_check(cudaMemsetAsync(stk, 0, 4 * total, st), "memset");
  size_t src_off = 0;
  for (int id = 0; id < m.n_polys; id++) {
    size_t n = (size_t)1 << poly_k[id];
    cuda_check(copy_async(*ctx_, stk + m.poly_off[id], polys + src_off, 4 * n,
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice),
               "poly copy");
    src_off += n;
  }
  encode_commit(*ctx_, stk, p_.k, p_.rate, p_.folding, 1, m.cw0.as<uint32_t>(),
                m.scratch.as<uint32_t>(), m.tree0.as<uint32_t>(), &m.t0);
  ts.write_digest(m.t0.root);
}

E4 Prover::eval(Transcript &ts, int id, const E4 *point) {
  Impl &m = *m_;
  if (id < 0 || id >= m.n_polys) throw WhirError(-1, "unknown polynomial id");
  for (int i = 0; i < m.pk[id]; i++)
    for (int c = 0; c < 4; c++)
      if (point[i].c[c] >= P) throw WhirError(-1, "non-canonical field element");
  SvoClaim c;
  c.poly = id;
  m.svo_claim(c, m.poly_dev(id), m.pk[id], point);
  ts.write_ext(c.eval);
  E4 e = c.eval;
  m.claims.push_back(std::move(c));
  return e;
}

void Prover::open(Transcript &ts) { m_->open(ts); }

void Prover::prove(Transcript &ts, const uint32_t *polys, bool on_device,
                   const std::vector<int> &poly_k, const std::vector<std::vector<int>> &groups) {
  commit(ts, polys, on_device, poly_k);
  for (auto &g : groups) {
    if (g.empty()) throw WhirError(-1, "empty claim group");
    int kg = poly_k.at(g[0]);
    std::vector<E4> pt(kg);
    expand(pt.data(), kg, ts.draw_ext());
    for (int id : g) {
      if (poly_k.at(id) != kg) throw WhirError(-1, "claim group mixes polynomial sizes");
      eval(ts, id, pt.data());
    }
  }
  open(ts);
}

}  // namespace whir
