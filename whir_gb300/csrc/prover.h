// GPU WHIR prover: the host orchestration of Whir::commit / ProverStack /
// Whir::open (crates/whir/src/whir.rs:20-359, crates/whir/src/sumcheck/*.rs)
// with all polynomial-sized data resident on the device.  Per sumcheck round
// only (c0, c2) come back to the host and only the challenge goes down (as a
// kernel argument).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "kb.cuh"
#include "kernels.h"
#include "transcript.h"

namespace whir {

struct Params {
  int k;
  int folding;
  int rate;
  int initial_reduction;
  int soundness;  // 0 UniqueDecoding, 1 JohnsonBound, 2 CapacityBound
  int security_level;
};

// crates/whir/src/params.rs
int n_ood_queries(int soundness, int security, int log_degree, int log_inv_rate, int field_bits);
int n_stir_queries(int soundness, int security, int log_inv_rate);
void number_of_rounds(int folding, int k, int *n_rounds, int *final_rounds);
constexpr int EXT_BITS = 124;  // bits of |BinomialExtensionField<KoalaBear, 4>|

uint32_t two_adic_generator(int bits);  // Montgomery form

// one entry of the stacked layout: poly id, selector bits, aligned index
struct LayEntry {
  int nbits = 0;
  uint8_t bits[32] = {};
  int poly = 0;
  size_t index = 0;
};
std::vector<LayEntry> stack_layout(const std::vector<int> &pk, int k_expect, int folding);

// domain bits, folded-domain bits and rates of WHIR round `round`
void round_params(const Params &p, int round, int *kfd, int *this_rate, int *prev_rate);

// device buffer sizes (bytes) of one prover for params p
struct Workspace {
  size_t stacked, cw0, tree0, scratch, cw, tree, sumcheck, eqbuf, acc, small, gather, code;
  size_t total() const;
};
Workspace workspace_plan(const Params &p);
// device bytes of the buffers that serve every one of these parameter sets
// (per buffer, the largest need)
size_t workspace_union_bytes(const std::vector<Params> &ps);
// upper bound of the proof bytes with n_claims claims
size_t proof_bytes_max(const Params &p, int n_claims);

struct WhirError : std::runtime_error {
  int code;
  WhirError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};
void cuda_check(cudaError_t e, const char *what);

// device allocation owned by one object
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  ~DeviceBuffer();
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  void reserve(size_t bytes);
  template <class T>
  T *as() const { return reinterpret_cast<T *>(ptr_); }
  size_t bytes() const { return bytes_; }

 private:
  void *ptr_ = nullptr;
  size_t bytes_ = 0;
};

// page-locked host memory owned by one object
class PinnedBuffer {
 public:
  PinnedBuffer() = default;
  ~PinnedBuffer() {
    if (p_) cudaFreeHost(p_);
  }
  PinnedBuffer(const PinnedBuffer &) = delete;
  PinnedBuffer &operator=(const PinnedBuffer &) = delete;
  void reserve(size_t bytes) {
    if (bytes <= bytes_) return;
    if (p_) cudaFreeHost(p_);
    p_ = nullptr;
    bytes_ = 0;
    cuda_check(cudaMallocHost(&p_, bytes), "cudaMallocHost");
    bytes_ = bytes;
  }
  uint8_t *data() const { return static_cast<uint8_t *>(p_); }
  size_t bytes() const { return bytes_; }

 private:
  void *p_ = nullptr;
  size_t bytes_ = 0;
};

// refuses parameter sets the reference cannot run (WhirError code -1)
void check_params(const Params &p);

// One device, one stream, the device tables and a pinned staging area.
class Context {
 public:
  explicit Context(int device);
  ~Context();
  int device() const { return device_; }
  cudaStream_t stream() const { return stream_; }
  // Runs the following work on a high-priority stream (the device schedules
  // its blocks first) or back on the normal one; waits for the current
  // stream first.
  void set_high_priority(bool on);
  void *pinned(size_t bytes);  // staging for D2H results and H2D arguments
  void sync();
  // Waiting for the stream: a blocking synchronise (lowest latency, keeps a
  // core busy), or a short poll with yields followed by a sleep on a
  // blocking-sync event, so that many worker threads can share the host cores.
  void set_yield_wait(bool on) { yield_ = on; }
  // A word of pinned host memory that kernels raise to a sequence number
  // after writing their results there (gpu::Publish): waiting on it costs no
  // driver call.  next_seq() hands out the number for the next such launch.
  unsigned int *flag() const { return flag_; }
  unsigned int next_seq() { return seq_ = seq_ + 1 ? seq_ + 1 : 1; }
  void wait_flag(unsigned int seq);
  // per-kernel-class CUDA-event timing on this stream
  // kernel classes timed with events, and K_SYNC: host time blocked in sync()
  enum Klass { K_DFT = 0, K_LEAF = 1, K_TREE = 2, K_SUMCHECK = 3, K_SYNC = 4, K_NCLASS = 5 };
  void prof_enable(bool on) { prof_mask_ = on ? (1u << K_NCLASS) - 1 : 0; }
  // time only the classes whose bit is set (fewer events on the stream)
  void prof_enable_classes(unsigned mask) { prof_mask_ = mask & ((1u << K_NCLASS) - 1); }
  void prof_begin(int klass);
  void prof_end(int klass, double bytes);
  // drains recorded events: total ms, launches and bytes per class
  void prof_read(int klass, double *ms, long *launches, double *bytes);
  // bytes copied host<->device through copy_async since creation
  void count_copy(size_t bytes, int kind);
  unsigned long long h2d_bytes() const { return h2d_bytes_; }
  unsigned long long d2h_bytes() const { return d2h_bytes_; }

 private:
  void wait_stream();
  int device_;
  bool yield_ = false;
  cudaEvent_t block_ev_ = nullptr;
  unsigned int *flag_ = nullptr;
  unsigned int seq_ = 0;
  cudaStream_t stream_ = nullptr;
  cudaStream_t streams_[2] = {nullptr, nullptr};  // normal, high priority
  void *pinned_ = nullptr;
  size_t pinned_bytes_ = 0;
  unsigned prof_mask_ = 0;
  bool prof_on(int klass) const { return (prof_mask_ >> klass) & 1u; }
  struct Ev {
    cudaEvent_t a, b;
    int klass;
    double bytes;
  };
  std::vector<Ev> evs_;
  std::vector<cudaEvent_t> free_events_;
  double acc_ms_[K_NCLASS] = {0, 0, 0, 0, 0};
  long acc_n_[K_NCLASS] = {0, 0, 0, 0, 0};
  double acc_bytes_[K_NCLASS] = {0, 0, 0, 0, 0};
  unsigned long long h2d_bytes_ = 0, d2h_bytes_ = 0;
  int open_klass_ = -1;
  cudaEvent_t open_ev_ = nullptr;
  cudaEvent_t take_event();
};

// cudaMemcpyAsync on the context stream, counted in the context's totals
cudaError_t copy_async(Context &c, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind);

// Merkle data kept on the device (MerkleData, crates/merkle/src/lib.rs:11-17)
struct DeviceTree {
  const uint32_t *rows = nullptr;  // codeword rows (borrowed)
  uint32_t *nodes = nullptr;       // all levels, leaves first
  int log_h = 0;
  int row_len = 0;
  uint32_t root[8];
};

// Reed-Solomon encode + Merkle commit of `src` (2^k rows... see commit_rows)
void encode_commit(Context &ctx, const uint32_t *src, int k, int rate, int folding, int dim,
                   uint32_t *codeword, uint32_t *scratch, uint32_t *nodes, DeviceTree *out);

class Prover {
 public:
  Prover(Context *ctx, const Params &p);
  ~Prover();
  const Params &params() const { return p_; }
  // Whir::commit of the stacked layout of the given polys (ProverStack::layout
  // order, prover.rs:92-124); a single poly is committed as is.
  void commit(Transcript &ts, const uint32_t *polys, bool on_device,
              const std::vector<int> &poly_k);
  // ProverStack::eval (prover.rs:64-90): claim on poly `id` at `point` (k_id
  // extension elements); writes and returns the evaluation.
  kb::E4 eval(Transcript &ts, int id, const kb::E4 *point);
  // Whir::open (whir.rs:168-359)
  void open(Transcript &ts);
  // the whole reference harness (test.rs:218-235) except the final draw:
  // commit, then each claim group draws one expanded point and evaluates it
  // on its polys, then open.
  void prove(Transcript &ts, const uint32_t *polys, bool on_device, const std::vector<int> &poly_k,
             const std::vector<std::vector<int>> &groups);
  size_t device_bytes() const;
  // re-target the prover at new parameters; device buffers are kept and
  // grown on the next commit when they are too small
  void set_params(const Params &p);
  // grow the device buffers to the current parameters' workspace now (they
  // only grow; a proof would otherwise do it on its first use)
  void reserve();
  // device bytes a prover holds after proving with params p
  static size_t workspace_bytes(const Params &p);

 private:
  struct Impl;
  Impl *m_;
  Context *ctx_;
  Params p_;
};

}  // namespace whir
