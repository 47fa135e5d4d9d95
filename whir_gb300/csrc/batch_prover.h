// Lock-step proving of many instances of one shape.  A group of `batch`
// jobs with the same parameters and claim count runs through the prover's
// sequence of passes together: each device pass is one launch over all
// instances (kernels.h, batched launches), and each transcript round trip
// waits once for all of them, after which the instances' host work (their
// own transcripts, SVO algebra, query sampling) runs on a pool of host
// threads.  Every instance's proof bytes are exactly those of Prover on the
// same polynomial: the same arithmetic in the same order per instance, only
// scheduled together (crates/whir/src/whir.rs:20-359, the harness
// crates/whir/src/test.rs:218-235 per instance).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <functional>
#include <vector>

#include "prover.h"

namespace whir {

// A small pool of host threads for per-instance work: run(n, fn, parts)
// calls fn(0) .. fn(n-1) on at most `parts` threads (the calling thread and
// pool helpers), and returns when all are done (rethrowing the first
// exception).
class HostPool {
 public:
  explicit HostPool(int threads);
  ~HostPool();
  HostPool(const HostPool &) = delete;
  HostPool &operator=(const HostPool &) = delete;
  void run(int n, const std::function<void(int)> &fn, int parts);
  int threads() const { return threads_; }

 private:
  struct State;
  State *s_;
  int threads_;
};

class BatchProver {
 public:
  BatchProver(Context *ctx, const Params &p, int host_threads);
  ~BatchProver();
  BatchProver(const BatchProver &) = delete;
  BatchProver &operator=(const BatchProver &) = delete;
  const Params &params() const { return p_; }
  void set_params(const Params &p);
  // The harness on each instance: commit polys[b] (2^k words, host or device
  // memory), then n_claims times draw one expanded point and write the
  // evaluation, then open; commit_only stops after the root.  ts[b] are the
  // instances' transcripts (fresh).  1 <= ts.size() <= max_batch(params).
  // finish (optional) runs once per instance on the host pool after its
  // proof is complete (the caller's read-out of ts[b]).
  void prove(const std::vector<Transcript *> &ts, const std::vector<const uint32_t *> &polys,
             bool on_device, int n_claims, bool commit_only,
             const std::function<void(int)> &finish = nullptr);
  // grow the device buffers for `batch` instances of the current parameters
  void reserve(int batch);
  size_t device_bytes() const;
  // device bytes held after proving `batch` instances with params p
  static size_t workspace_bytes(const Params &p, int batch);
  // the most instances one group of these parameters takes (the batched
  // codewords' rows and widths must fit the DFT's 32-bit indexing)
  static int max_batch(const Params &p);

 private:
  struct Impl;
  Impl *m_;
  Params p_;
};

}  // namespace whir
