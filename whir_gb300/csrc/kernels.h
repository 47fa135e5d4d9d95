// Launchers of the sm_103a kernels.  Every pointer is a device pointer unless
// its name ends in _h; every launch goes to the given stream and returns
// without synchronising.  Field words are Montgomery form (see kb.cuh).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "kb.cuh"

namespace whir {
namespace gpu {

// Where a reduction's result goes.  With host set, the last CTA of the
// reducing launch copies acc[0..words) to host (pinned memory the device can
// write), then zeroes those words and the counter, so the next reduction
// starts from zero without a memset and the host reads the result after a
// stream sync without a copy.  Without host, acc keeps the sums.
struct Publish {
  unsigned int *counter = nullptr;
  unsigned long long *host = nullptr;
  int words = 0;
  // optional: after the results, the last CTA stores seq to *flag (pinned
  // host memory), so the host can wait on that word instead of the stream
  unsigned int *flag = nullptr;
  unsigned int seq = 0;
};

// ---- per-size scheduling choices ----
// How a tree or a DFT of a given size is split into launches.  Every choice
// computes the same result; whir::autotune picks them by measurement.
// Tree: levels that make >= 2^wide_log nodes run one thread per node; the
// remaining S levels run as 2^((S + split) / 2) strided subtrees, then one
// CTA to the root.  DFT (two-pass sizes): the first pass transforms columns
// of 2^L1 rows, L1 = (log_h + 1) / 2 + l1_bias.
struct TreeTune {
  int wide_log = 15;
  int split = 0;
};
struct DftTune {
  int l1_bias = 0;
};
TreeTune tree_tune(int log_h);
void set_tree_tune(int log_h, TreeTune t);
DftTune dft_tune(int log_h, size_t width);
void set_dft_tune(int log_h, size_t width, DftTune t);
bool tree_tune_valid(int log_h, TreeTune t);
bool dft_tune_valid(int log_h, DftTune t);
// true when dft_batch runs one pass of coset transforms for this shape
// (16-byte aligned buffers), so the two-pass split does not apply
bool dft_coset_one_pass(int log_h, size_t h_in, size_t width);

// ---- kernel launches issued by this library (all contexts), for reporting ----
unsigned long long launch_count();
void count_launches(unsigned n);

// ---- one-time device set-up (constants, twiddle tables) ----
cudaError_t init_device_tables();

// ---- RS encoding: p3 TwoAdicSubgroupDft::dft_batch (crates/whir/src/whir.rs:34,59) ----
// out[i][c] = sum_{r < h_in} in[r][c] * w^(r i), w = two_adic_generator(log_h),
// rows of `width` words, natural order; rows >= h_in are zero.  `scratch`
// holds 2^log_h * width words when log_h > 11 (two passes), else unused.
cudaError_t dft_batch(const uint32_t *in, size_t h_in, size_t width, int log_h, uint32_t *out,
                      uint32_t *scratch, cudaStream_t st);

// ---- Merkle (crates/merkle/src/poseidon_packed.rs) ----
// leaf digests: PaddingFreeSponge<P24, 24, 16, 8> over each row of row_len words
cudaError_t hash_rows(const uint32_t *rows, size_t n_rows, int row_len, uint32_t *digests,
                      cudaStream_t st);
// all levels above the leaves: level l+1 node i = C(level l node i, node i + n/2)
// nodes: level 0 (2^log_h digests) first, then each level in turn
// host_root (optional, device-writable host memory): the root is also written
// there, and then seq to *flag (when flag is set)
cudaError_t build_tree(uint32_t *nodes, int log_h, cudaStream_t st, uint32_t *host_root = nullptr,
                       unsigned int *flag = nullptr, unsigned int seq = 0);
// per query: the leaf row then log_h sibling digests bottom-up
cudaError_t gather_openings(const uint32_t *rows, int row_len, const uint32_t *nodes, int log_h,
                            const uint32_t *idx, int n, uint32_t *out, cudaStream_t st);
// the same with at most IdxArgs::N indexes passed by value
struct IdxArgs {
  static constexpr int N = 2048;
  uint32_t idx[N];
};
cudaError_t gather_openings_val(const uint32_t *rows, int row_len, const uint32_t *nodes,
                                int log_h, const IdxArgs &a, int n, uint32_t *out,
                                cudaStream_t st);
// Merkle path checks of many openings (MerkleTree::verify,
// crates/merkle/src/poseidon_packed.rs:235-257, path check poseidon.rs:22-41):
// path i's words start at words[d[i].off]: the row (row_len words, hashed as
// a leaf), then log_h sibling digests bottom-up, as an opening lies in a
// proof; its root is roots[8 i .. 8 i + 8).  ok[i] = 1 when the path climbs
// to its root, else 0.  One thread per path; paths sorted by (row_len,
// log_h) keep warps uniform.  log_h <= 40.
struct PathDesc {
  uint64_t off;
  uint64_t index;
  int32_t log_h;
  int32_t row_len;
};
cudaError_t verify_paths(const PathDesc *d, const uint32_t *words, const uint32_t *roots, int n,
                         uint8_t *ok, cudaStream_t st);
KB_HD size_t tree_words(int log_h) { return (((size_t)2 << log_h) - 1) * 8; }
KB_HD size_t level_offset_words(int log_h, int level) {
  return (((size_t)2 << log_h) - ((size_t)2 << (log_h - level))) * 8;
}

// ---- eq tables and sumcheck passes (crates/poly, crates/whir/src/sumcheck) ----
constexpr int MAX_VARS = 32;
struct Point {
  int k;
  kb::E4 z[MAX_VARS];
};
// eq(z) * scale as two split tables: lo over z[0..s), hi over z[s..k) (scale in hi)
// lo/hi hold 2^s and 2^(k-s) E4.
cudaError_t eq_split(const Point &z, int s, kb::E4 scale, kb::E4 *lo, kb::E4 *hi,
                     cudaStream_t st);
// n split tables at once: pts (device) n x k extension elements, scales (device)
// n; table t at out + t * (2^s + 2^(k-s)): lo over pts[t][0..s), hi over the
// rest times scales[t]
cudaError_t eq_tables(const kb::E4 *pts, const kb::E4 *scales, int n, int k, int s, kb::E4 *out,
                      cudaStream_t st);
// eq_tables with at most EqArgs::N points of at most EqArgs::K coordinates
// passed by value (no device copy of the points)
struct EqArgs {
  static constexpr int N = 8, K = 32;
  kb::E4 z[N * K];  // point t at z[t * K]
  kb::E4 scale[N];
};
cudaError_t eq_tables_val(const EqArgs &a, int n, int k, int s, kb::E4 *out, cudaStream_t st);
// full table eq(z) * scale of 2^k entries (k <= 24)
cudaError_t eq_full(const Point &z, kb::E4 scale, kb::E4 *out, kb::E4 *tmp, cudaStream_t st);

// SplitEq::compress_hi (crates/poly/src/eq.rs:290-398) over a base poly:
// acc[j] += sum_h eq(zrest)[h] * P[h * 2^ks + j]; acc is u64[2^ks][4] of
// unreduced canonical sums (reduce mod p on read).  eq tables from eq_split.
cudaError_t compress_hi(const uint32_t *poly, int k, int ks, const kb::E4 *eq_lo, int s_lo,
                        const kb::E4 *eq_hi, unsigned long long *acc, cudaStream_t st,
                        const Publish &pub = Publish());
// SplitEq::compress_lo_into (eq.rs:491-539): out[i] = sum_j eq(rs)[j] * P[i*2^ks + j]
cudaError_t compress_lo(const uint32_t *poly, int k, const Point &rs, kb::E4 *out,
                        cudaStream_t st);
// w[i] += sum_t lo_t[i & (2^s-1)] * hi_t[i >> s] for n_tables split eq tables
// stored back to back (lo0, hi0, lo1, hi1, ...), s = k / 2, each lo 2^s and
// hi 2^(k-s) entries.
cudaError_t add_eq(kb::E4 *w, int k, const kb::E4 *tables, int n_tables, cudaStream_t st);
// w[i] += sum_t scale_t * var_t^i  (pow::combine_pows(_scaled), combine.rs:408-468);
// tab: add_pows_scratch_words(k, n) words for the split power tables
size_t add_pows_scratch_words(int k, int n);
cudaError_t add_pows(kb::E4 *w, int k, const uint32_t *vars, const kb::E4 *scales, int n,
                     uint32_t *tab, cudaStream_t st);
// add_pows with at most PowArgs::N variables and scales passed by value
struct PowArgs {
  static constexpr int N = 256;
  uint32_t vars[N];
  kb::E4 scales[N];
};
cudaError_t add_pows_val(kb::E4 *w, int k, const PowArgs &a, int n, uint32_t *tab,
                         cudaStream_t st);
// one sumcheck round (expr.rs:14-27, poly.rs:131-142): optionally fold both
// arrays by r into (p_out, w_out), then add (c0, c2) of the result into acc
// (u64[8], unreduced canonical) when coeffs != 0.
cudaError_t sumcheck_round(const kb::E4 *p_in, const kb::E4 *w_in, size_t n_in, bool fold,
                           kb::E4 r, kb::E4 *p_out, kb::E4 *w_out, bool coeffs,
                           unsigned long long *acc, cudaStream_t st,
                           const Publish &pub = Publish());
// <eq(z), poly> for an extension poly (SplitEq::eval_ext, eq.rs:179-250) -> acc u64[4]
cudaError_t eval_ext(const kb::E4 *poly, int k, const kb::E4 *eq_lo, int s_lo,
                     const kb::E4 *eq_hi, unsigned long long *acc, cudaStream_t st,
                     const Publish &pub = Publish());
// <a, b> of two extension arrays of n elements -> acc u64[4] (debug checks)
cudaError_t dot_ext(const kb::E4 *a, const kb::E4 *b, size_t n, unsigned long long *acc,
                    cudaStream_t st, const Publish &pub = Publish());
// fold_with_code's per-query state on the device (see code_round_kernel)
struct CodeState {
  const uint32_t *idx;  // n query indexes
  kb::E4 *G;            // n * 2^d values of g
  kb::E4 *scales;       // n
  uint32_t *ws, *tw, *B;  // n each
  const uint32_t *wd;   // 2^d powers of w^-S
  int n, d, k_data;
  uint32_t omega, winv, two_inv;  // w, w^-1 (w = two_adic_generator(k_data)), 1/2
  // several instances' queries in one launch: query i belongs to instance
  // inst[i], whose challenge (r_prev, r_last) is r_b[inst[i]] and whose sums
  // go to acc + inst[i] * acc_stride (all unset for one instance)
  const int *inst = nullptr;
  const kb::E4 *r_b = nullptr;
  size_t acc_stride = 0;
};
// round r: G update with r_prev (r >= 1), then this round's part of (c0, c2)
// added to acc[0..8) (and, at round 0, the sum term to acc[8..12))
cudaError_t code_round(const CodeState &s, int round, kb::E4 r_prev, unsigned long long *acc,
                       cudaStream_t st, const Publish &pub = Publish());
cudaError_t code_finish(const CodeState &s, kb::E4 r_last, cudaStream_t st);
// out[q] = <eq(rs), row(idx[q])> over base rows (fold_with_code evals, prover.rs:497-506)
cudaError_t row_evals(const uint32_t *rows, int row_len, const uint32_t *idx, int n,
                      const Point &rs, kb::E4 *out, cudaStream_t st);

// ---- many instances of one shape in one launch (batched proving) ----
// Instance y of a launch (blockIdx.y) works on its own arrays, found at y
// times a stride from each base, with its own challenges from per-instance
// device arrays; reductions land in acc + y * (words per instance), and the
// last CTA of the whole launch publishes every instance's words at once.
// A batched codeword is the row-major matrix whose row r holds row r of
// every instance in turn (row r of instance y = row r batch + y); its
// Merkle tree is the halves-paired tree over those rows stopped at the level
// of `batch` nodes, which are the instances' roots (with halves pairing the
// instances never meet below that level).
struct HiStrides {
  size_t poly = 0, tab = 0, acc = 0;  // elements between consecutive instances
};
cudaError_t compress_hi_batch(const uint32_t *poly, int k, int ks, const kb::E4 *eq_lo, int s_lo,
                              const kb::E4 *eq_hi, unsigned long long *acc, int batch,
                              const HiStrides &sd, cudaStream_t st,
                              const Publish &pub = Publish());
// rs_b: batch x ks challenges; instance y reads poly + y poly_stride, writes
// out + y 2^(k - ks)
cudaError_t compress_lo_batch(const uint32_t *poly, int k, int ks, const kb::E4 *rs_b, int batch,
                              size_t poly_stride, kb::E4 *out, cudaStream_t st);
// instance y: w + y 2^k and n_tables tables from tables + y n_tables (2^s + 2^(k-s))
cudaError_t add_eq_batch(kb::E4 *w, int k, const kb::E4 *tables, int n_tables, int batch,
                         cudaStream_t st);
// ragged: instance y adds vars[off[y] .. off[y+1]) with their scales into
// w + y 2^k (off: batch + 1 device ints, max_n the largest count)
cudaError_t add_pows_batch(kb::E4 *w, int k, const uint32_t *vars, const kb::E4 *scales,
                           const int *off, int n_total, int max_n, int batch, uint32_t *tab,
                           cudaStream_t st);
// arrays of instance y at y n_in (in) and y n_in / 2 (out), challenge r_b[y]
// (fold), sums at acc + y acc_stride
cudaError_t sumcheck_round_batch(const kb::E4 *p_in, const kb::E4 *w_in, size_t n_in, bool fold,
                                 const kb::E4 *r_b, kb::E4 *p_out, kb::E4 *w_out, bool coeffs,
                                 unsigned long long *acc, size_t acc_stride, int batch,
                                 cudaStream_t st, const Publish &pub = Publish());
// instance y: poly + y 2^k, tables at y tab_stride, sum at acc + 4 y
cudaError_t eval_ext_batch(const kb::E4 *poly, int k, const kb::E4 *eq_lo, int s_lo,
                           const kb::E4 *eq_hi, size_t tab_stride, int batch,
                           unsigned long long *acc, cudaStream_t st,
                           const Publish &pub = Publish());
// instance y: rows idx[off[y] .. off[y+1]) of its part of a batched codeword
// (rows of 2^ks words) at its rs_b[y ks ..]
cudaError_t row_evals_batch(const uint32_t *rows, int row_len, const uint32_t *idx,
                            const int *off, int max_n, int ks, const kb::E4 *rs_b, int batch,
                            kb::E4 *out, cudaStream_t st);
// src: batch matrices of rows x w words back to back; dst: the batched
// matrix (row r = row r of each instance in turn)
cudaError_t interleave_rows(const uint32_t *src, size_t rows, size_t w, int batch, uint32_t *dst,
                            cudaStream_t st);
// the batched tree over batch * 2^log_h leaves up to the instances' roots:
// level l (batch 2^(log_h - l) nodes) at batch * level_offset_words(log_h, l)
cudaError_t build_tree_batch(uint32_t *nodes, int log_h, int batch, cudaStream_t st);
// per query q: instance inst[q], index idx[q] of its codeword; out + q (row_len
// + 8 log_h) gets the row then log_h sibling digests bottom-up
cudaError_t gather_openings_batch(const uint32_t *rows, int row_len, const uint32_t *nodes,
                                  int log_h, int batch, const uint32_t *idx, const int *inst,
                                  int n, uint32_t *out, cudaStream_t st);

}  // namespace gpu
}  // namespace whir
