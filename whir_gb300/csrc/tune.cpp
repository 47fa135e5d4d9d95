// Autotuner of the tree and DFT launch splits (see tune.h).
#include "tune.h"

#include <stdio.h>

#include <algorithm>
#include <vector>

#include "kernels.h"

namespace whir {

namespace {
// mean time of 3 runs after a warm-up run, on the context's stream
template <class F>
double time_ms(Context &ctx, cudaEvent_t a, cudaEvent_t b, F &&fn) {
  cudaStream_t st = ctx.stream();
  fn();
  cuda_check(cudaEventRecord(a, st), "event");
  for (int r = 0; r < 3; r++) fn();
  cuda_check(cudaEventRecord(b, st), "event");
  cuda_check(cudaEventSynchronize(b), "event");
  float ms = 0;
  cuda_check(cudaEventElapsedTime(&ms, a, b), "event");
  return ms / 3;
}
}  // namespace

void tune_reset() {
  for (int h = 0; h <= 40; h++) gpu::set_tree_tune(h, gpu::TreeTune());
  for (int h = 0; h <= 24; h++) {
    gpu::set_dft_tune(h, 16, gpu::DftTune());
    gpu::set_dft_tune(h, 64, gpu::DftTune());
  }
}

std::string autotune(Context &ctx, int lo, int hi) {
  lo = std::max(lo, 4);
  hi = std::min(hi, 24);
  std::string rep;
  char line[160];
  if (lo > hi) return rep;
  cudaStream_t st = ctx.stream();
  cudaEvent_t a, b;
  cuda_check(cudaEventCreate(&a), "event");
  cuda_check(cudaEventCreate(&b), "event");
  try {
    // trees: the leaf digests' values do not change the time
    DeviceBuffer nodes;
    nodes.reserve(4 * gpu::tree_words(hi));
    cuda_check(cudaMemsetAsync(nodes.as<void>(), 0x5a, nodes.bytes(), st), "memset");
    for (int h = std::max(lo, 8); h <= hi; h++) {
      gpu::TreeTune best, base;
      double best_ms = 1e30, base_ms = 0;
      for (int wl = 12; wl <= 18; wl++)
        for (int sp = -1; sp <= 1; sp++) {
          gpu::TreeTune t;
          t.wide_log = wl;
          t.split = sp;
          if (!gpu::tree_tune_valid(h, t)) continue;
          if (h <= wl && wl != base.wide_log) continue;  // wide_log >= h: the same split
          gpu::set_tree_tune(h, t);
          double ms = time_ms(ctx, a, b, [&] {
            cuda_check(gpu::build_tree(nodes.as<uint32_t>(), h, st), "build_tree");
          });
          if (wl == base.wide_log && sp == base.split) base_ms = ms;
          if (ms < best_ms) {
            best_ms = ms;
            best = t;
          }
        }
      gpu::set_tree_tune(h, best);
      snprintf(line, sizeof line, "tree log_h=%d wide_log=%d split=%d %.4f ms (default %.4f ms)\n",
               h, best.wide_log, best.split, best_ms, base_ms);
      rep += line;
    }
    // two-pass DFTs at the WHIR shapes: base rows of 16 words from a quarter
    // of the rows, extension rows of 64 words from a 32nd
    for (size_t width : {(size_t)16, (size_t)64}) {
      int ratio = width == 16 ? 2 : 5;
      size_t max_words = (size_t)1 << 27;
      for (int h = std::max(lo, 12); h <= hi; h++) {
        size_t words = width << h;
        if (words > max_words) break;
        size_t h_in = (size_t)1 << std::max(0, h - ratio);
        if (gpu::dft_coset_one_pass(h, h_in, width)) continue;  // nothing to choose
        DeviceBuffer in, out, scr;
        in.reserve(4 * h_in * width);
        out.reserve(4 * words);
        scr.reserve(4 * words);
        cuda_check(cudaMemsetAsync(in.as<void>(), 0x11, in.bytes(), st), "memset");
        gpu::DftTune best;
        double best_ms = 1e30, base_ms = 0;
        for (int bias = -2; bias <= 2; bias++) {
          gpu::DftTune t;
          t.l1_bias = bias;
          if (!gpu::dft_tune_valid(h, t)) continue;
          gpu::set_dft_tune(h, width, t);
          double ms = time_ms(ctx, a, b, [&] {
            cuda_check(gpu::dft_batch(in.as<uint32_t>(), h_in, width, h, out.as<uint32_t>(),
                                      scr.as<uint32_t>(), st),
                       "dft_batch");
          });
          if (bias == 0) base_ms = ms;
          if (ms < best_ms) {
            best_ms = ms;
            best = t;
          }
        }
        gpu::set_dft_tune(h, width, best);
        snprintf(line, sizeof line, "dft log_h=%d width=%zu l1_bias=%d %.4f ms (default %.4f ms)\n",
                 h, width, best.l1_bias, best_ms, base_ms);
        rep += line;
        cuda_check(cudaStreamSynchronize(st), "sync");  // before the buffers go
      }
    }
  } catch (...) {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    throw;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return rep;
}

}  // namespace whir
