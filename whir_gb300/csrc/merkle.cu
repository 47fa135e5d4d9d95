// Merkle commitment kernels: leaf hashing (width-24 sponge), tree ascent
// (width-16 truncated-permutation compression, halves pairing) and the
// opening gather.  Tree shape and hashing follow
// crates/merkle/src/poseidon_packed.rs:98-143,269-304,344-384 and
// crates/merkle/src/poseidon.rs:33-74.
#include <algorithm>
#include <atomic>

#include "kernels.h"
#include "launch.cuh"
#include "p2_device.cuh"
#include "poseidon2_host.h"

namespace whir {
namespace gpu {

static cudaError_t upload_p2(int width) {
  const Poseidon2Constants &c = poseidon2_constants(width);
  uint32_t buf[8 * 24 + 23 + 24];
  int n = 0;
  // round constants minus p, for the signed S-box (p2_device.cuh)
  for (int r = 0; r < 8; r++)
    for (int i = 0; i < width; i++) buf[n++] = c.ext_rc[r][i] - kb::P;
  for (int r = 0; r < c.rounds_p; r++) buf[n++] = c.int_rc[r] - kb::P;
  for (int i = 0; i < width; i++) buf[n++] = c.diag[i];
  if (width == 16) return cudaMemcpyToSymbol(c_p2_16, buf, n * 4);
  return cudaMemcpyToSymbol(c_p2_24, buf, n * 4);
}

static std::atomic<unsigned long long> g_launches{0};
unsigned long long launch_count() { return g_launches.load(); }
void count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

cudaError_t init_poseidon2_tables() {
  cudaError_t e = upload_p2(16);
  if (e != cudaSuccess) return e;
  return upload_p2(24);
}

// One row per thread; a row of ROW = 16·c words is c permutations
// (PaddingFreeSponge: overwrite the 16 rate lanes, permute).  Base rows are
// 2^f words and extension rows 4·2^f, so foldings 4..6 use 16..256.
template <int ROW>
__global__ void __launch_bounds__(128) hash_rows_fixed(const uint32_t *__restrict__ rows,
                                                       size_t n_rows,
                                                       uint32_t *__restrict__ digests) {
  pdl_wait();
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_rows) return;
  const uint4 *src = reinterpret_cast<const uint4 *>(rows + i * ROW);
  uint32_t s[24];
#pragma unroll
  for (int j = 16; j < 24; j++) s[j] = 0;
#pragma unroll 1
  for (int chunk = 0; chunk < ROW / 16; chunk++) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      uint4 v = __ldg(src + chunk * 4 + q);
      s[4 * q] = v.x;
      s[4 * q + 1] = v.y;
      s[4 * q + 2] = v.z;
      s[4 * q + 3] = v.w;
    }
    p2_permute<24>(s);
  }
  uint4 *dst = reinterpret_cast<uint4 *>(digests + i * 8);
  dst[0] = make_uint4(s[0], s[1], s[2], s[3]);
  dst[1] = make_uint4(s[4], s[5], s[6], s[7]);
}

// Any row length (small foldings): the trailing partial chunk overwrites only
// its lanes and is permuted; an empty trailing chunk is not.
__global__ void hash_rows_generic(const uint32_t *__restrict__ rows, size_t n_rows, int row_len,
                                  uint32_t *__restrict__ digests) {
  pdl_wait();
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_rows) return;
  const uint32_t *src = rows + i * row_len;
  uint32_t s[24];
#pragma unroll
  for (int j = 0; j < 24; j++) s[j] = 0;
  int pos = 0;
  while (pos < row_len) {
    int take = row_len - pos < 16 ? row_len - pos : 16;
    for (int j = 0; j < take; j++) s[j] = src[pos + j];
    pos += take;
    p2_permute<24>(s);
  }
  for (int j = 0; j < 8; j++) digests[i * 8 + j] = s[j];
}

// One opening per thread: the leaf sponge over the row (16 rate words per
// permutation, a shorter last chunk overwriting only its words), then one
// width-16 compression per level with the sibling on the side the index's
// bit names (halves pairing: at a level of 2m nodes, index i >= m is the
// right child).
__global__ void __launch_bounds__(128) verify_paths_kernel(const PathDesc *__restrict__ d,
                                                           const uint32_t *__restrict__ words,
                                                           const uint32_t *__restrict__ roots,
                                                           int n, uint8_t *__restrict__ ok) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PathDesc pd = d[i];
  const uint32_t *w = words + pd.off;
  uint32_t s[24];
#pragma unroll
  for (int j = 0; j < 24; j++) s[j] = 0;
  for (int pos = 0; pos < pd.row_len; pos += 16) {
    const int take = pd.row_len - pos < 16 ? pd.row_len - pos : 16;
#pragma unroll
    for (int j = 0; j < 16; j++)
      if (j < take) s[j] = w[pos + j];
    p2_permute<24>(s);
  }
  uint32_t acc[8];
#pragma unroll
  for (int j = 0; j < 8; j++) acc[j] = s[j];
  const uint32_t *sib = w + pd.row_len;
  uint64_t idx = pd.index;
  for (int l = 0; l < pd.log_h; l++) {
    const uint64_t mid = 1ull << (pd.log_h - l - 1);
    const bool right = idx >= mid;
    uint32_t t[16];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const uint32_t a = acc[j], b = sib[8 * l + j];
      t[j] = right ? b : a;
      t[8 + j] = right ? a : b;
    }
    p2_permute<16>(t);
#pragma unroll
    for (int j = 0; j < 8; j++) acc[j] = t[j];
    idx &= mid - 1;
  }
  const uint32_t *root = roots + 8 * (size_t)i;
  bool good = true;
#pragma unroll
  for (int j = 0; j < 8; j++) good &= acc[j] == root[j];
  ok[i] = good ? 1 : 0;
}

cudaError_t verify_paths(const PathDesc *d, const uint32_t *words, const uint32_t *roots, int n,
                         uint8_t *ok, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int T = 128;
  launch(verify_paths_kernel, (unsigned)((n + T - 1) / T), T, 0, st, d, words, roots, n, ok);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t hash_rows(const uint32_t *rows, size_t n_rows, int row_len, uint32_t *digests,
                      cudaStream_t st) {
  if (n_rows == 0) return cudaSuccess;
  const int T = 128;
  unsigned grid = (unsigned)((n_rows + T - 1) / T);
  // the fixed-width kernels use 16-byte vector loads and stores
  bool aligned = (((uintptr_t)rows | (uintptr_t)digests) & 15) == 0;
  switch (aligned ? row_len : 0) {
    case 16: launch(hash_rows_fixed<16>, grid, T, 0, st, rows, n_rows, digests); break;
    case 32: launch(hash_rows_fixed<32>, grid, T, 0, st, rows, n_rows, digests); break;
    case 64: launch(hash_rows_fixed<64>, grid, T, 0, st, rows, n_rows, digests); break;
    case 128: launch(hash_rows_fixed<128>, grid, T, 0, st, rows, n_rows, digests); break;
    case 256: launch(hash_rows_fixed<256>, grid, T, 0, st, rows, n_rows, digests); break;
    default: launch(hash_rows_generic, grid, T, 0, st, rows, n_rows, row_len, digests);
  }
  count_launches(1);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) compress_level(const uint32_t *__restrict__ src,
                                                      uint32_t *__restrict__ dst, size_t half) {
  pdl_wait();
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= half) return;
  const uint4 *a = reinterpret_cast<const uint4 *>(src + i * 8);
  const uint4 *b = reinterpret_cast<const uint4 *>(src + (i + half) * 8);
  uint4 a0 = __ldg(a), a1 = __ldg(a + 1), b0 = __ldg(b), b1 = __ldg(b + 1);
  uint32_t s[16] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w,
                    b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
  p2_permute<16>(s);
  uint4 *d = reinterpret_cast<uint4 *>(dst + i * 8);
  d[0] = make_uint4(s[0], s[1], s[2], s[3]);
  d[1] = make_uint4(s[4], s[5], s[6], s[7]);
}

// ---- width-16 permutation on a quad of lanes (latency) ----
// Lane l of an aligned group of 4 holds state words 4l .. 4l+3, which is one
// group of the light MDS: mat4 stays in registers and a column sum is three
// xor shuffles added as a tree (one shuffle latency, not two in a row).  In
// an internal round every lane tracks word 0 (z), so the S-box on it runs
// beside the shuffled sum of the other 15 words instead of before it.  The
// round constants for the next round are loaded one round ahead.  This is
// what a level with few nodes waits for: on GB300 one permutation takes
// 3.1 us here against 4.9 us for two chained xor shuffles per sum with the
// S-box ahead of the internal sum (and 6.3 us on one thread).
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ uint32_t quad_sum(uint32_t v) {
  uint32_t a = __shfl_xor_sync(FULL, v, 1, 4);
  uint32_t b = __shfl_xor_sync(FULL, v, 2, 4);
  uint32_t c = __shfl_xor_sync(FULL, v, 3, 4);
  return kb::add(kb::add(v, a), kb::add(b, c));
}

__device__ __forceinline__ void p2q_mds(uint32_t (&x)[4]) {
  p2_mat4(x[0], x[1], x[2], x[3]);
#pragma unroll
  for (int c = 0; c < 4; c++) x[c] = kb::add(x[c], quad_sum(x[c]));
}

// kc: the 8*16 external and 20 internal constants (stored minus p); dg: this
// lane's 4 diagonal entries (Montgomery form).  Every lane of the warp calls it.
__device__ __forceinline__ void p2q_permute(uint32_t (&x)[4], int l, const uint32_t *kc,
                                            const uint32_t (&dg)[4]) {
  using namespace kb;
  static_assert(P2Shape<16>::RP == 20, "internal rounds");
  static_assert(diag_entry16(0).sign < 0 && diag_entry16(0).num == 2 &&
                    diag_entry16(0).log_den == 0,
                "word 0's diagonal entry");
  p2q_mds(x);
  uint32_t ce[4];
#pragma unroll
  for (int i = 0; i < 4; i++) ce[i] = kc[4 * l + i];
#pragma unroll 1
  for (int r = 0; r < 8; r++) {
    if (r == 4) {
      uint32_t z = __shfl_sync(FULL, x[0], 0, 4);  // word 0 (lane 0's first)
      uint32_t rc = kc[8 * 16];
#pragma unroll 2
      for (int q = 0; q < 20; q++) {
        const uint32_t rcn = kc[8 * 16 + (q + 1 < 20 ? q + 1 : 19)];
        const uint32_t y = sbox((int32_t)(z + rc));
        // this lane's words other than word 0: < 4p < 2^33, folded below 2p
        uint64_t w = (uint64_t)x[1] + x[2] + x[3] + (l ? x[0] : 0u);
        uint32_t f = (uint32_t)(w & 0x7fffffffu) + (uint32_t)(w >> 31) * 0x00ffffffu;
        const uint32_t sum = add(quad_sum(kb::umin(f, f - P)), y);
        const uint32_t x0 = l ? x[0] : y;
        x[0] = add(sum, mul(x0, dg[0]));
#pragma unroll
        for (int i = 1; i < 4; i++) x[i] = add(sum, mul(x[i], dg[i]));
        z = sub(sum, dbl(y));  // word 0's diagonal entry is -2
        rc = rcn;
      }
    }
    uint32_t cn[4];
    const int rn = r + 1 < 8 ? r + 1 : 7;
#pragma unroll
    for (int i = 0; i < 4; i++) cn[i] = kc[rn * 16 + 4 * l + i];
#pragma unroll
    for (int i = 0; i < 4; i++) x[i] = sbox((int32_t)(x[i] + ce[i]));
    p2q_mds(x);
#pragma unroll
    for (int i = 0; i < 4; i++) ce[i] = cn[i];
  }
}

// ---- the narrow levels of a tree ----
// With halves pairing, node i of a level with H nodes is C(i, i + H/2) of the
// level below, and i, i + H/2 agree modulo any G dividing H/2.  So the nodes
// congruent to j mod G form an independent subtree down to the level with G
// nodes: CTA j keeps its share of a level in shared memory and climbs
// log2(H/G) levels with one barrier per level, writing every level it makes
// to the tree in global memory (the openings read them).  A narrow level is
// bound by the latency of one permutation, so this replaces one launch per
// level by two launches per tree (G CTAs up to the level of G nodes, then one
// CTA, G = 1, to the root), and each node is compressed by a quad of lanes.
// Threads: 4 per node of the first level made (at most 1024).
// A batched tree (kernels.h: batch instances' leaves interleaved) is the
// same ascent over batch 2^log_h leaves: level l holds batch 2^(log_h - l)
// nodes at batch * level_offset_words(log_h, l), and G is a multiple of
// batch, so every subtree lies inside one instance.
__global__ void __launch_bounds__(1024) tree_subtrees(uint32_t *__restrict__ nodes, int log_h,
                                                     int l0, int steps, uint32_t *host_root,
                                                     unsigned int *flag, unsigned int seq,
                                                     unsigned batch) {
  pdl_wait();
  extern __shared__ uint4 sm[];  // 2 uint4 per node of this CTA's share
  __shared__ uint32_t kc[8 * 16 + 20];
  for (int i = threadIdx.x; i < 8 * 16 + 20; i += blockDim.x) kc[i] = c_p2_16[i];
  const int l = threadIdx.x & 3, m = threadIdx.x >> 2;
  uint32_t dg[4];
#pragma unroll
  for (int i = 0; i < 4; i++) dg[i] = c_p2_16[8 * 16 + 20 + 4 * l + i];
  const size_t G = gridDim.x, j = blockIdx.x;
  int n = (int)(((size_t)batch << (log_h - l0)) / G);
  const uint4 *src = reinterpret_cast<const uint4 *>(nodes + batch * level_offset_words(log_h, l0));
  for (int q = threadIdx.x; q < 2 * n; q += blockDim.x) sm[q] = src[(j + G * (q >> 1)) * 2 + (q & 1)];
  __syncthreads();
  for (int st = 0; st < steps; st++) {
    const int half = n >> 1;
    const bool warp_live = ((threadIdx.x & ~31) >> 2) < half;  // warp-uniform
    const bool live = m < half;
    uint32_t x[4] = {0, 0, 0, 0};
    if (warp_live) {
      if (live) {
        // lanes 0, 1: the left child's two halves; lanes 2, 3: the right child's
        uint4 v = l < 2 ? sm[2 * m + l] : sm[2 * (m + half) + (l - 2)];
        x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
      }
      p2q_permute(x, l, kc, dg);
      if (live && l < 2) {
        uint4 *dst =
            reinterpret_cast<uint4 *>(nodes + batch * level_offset_words(log_h, l0 + st + 1));
        dst[(j + G * m) * 2 + l] = make_uint4(x[0], x[1], x[2], x[3]);
        if (host_root && G == 1 && half == 1) {  // the root, also to the host
#pragma unroll
          for (int w = 0; w < 4; w++) host_root[4 * l + w] = x[w];
        }
      }
    }
    __syncthreads();  // every read of this level's shared copy is done
    if (live && l < 2) sm[2 * m + l] = make_uint4(x[0], x[1], x[2], x[3]);
    __syncthreads();
    n = half;
  }
  if (flag && host_root && gridDim.x == 1) {  // the root is written: raise the flag
    __threadfence_system();
    __syncthreads();
    if (threadIdx.x == 0) *reinterpret_cast<volatile unsigned int *>(flag) = seq;
  }
}

// Default: levels whose step makes at least 2^15 nodes run one thread per
// node over the whole GPU; the rest (at most 2^16 nodes at the first narrow
// level) go through tree_subtrees.  Per-size overrides in tree_tune().
static std::atomic<int> g_tree_tune[41];  // 0: default, else (wide_log << 4) | (split + 2)

TreeTune tree_tune(int log_h) {
  TreeTune t;
  if (log_h < 0 || log_h > 40) return t;
  int v = g_tree_tune[log_h].load(std::memory_order_relaxed);
  if (v) {
    t.wide_log = v >> 4;
    t.split = (v & 15) - 2;
  }
  return t;
}
bool tree_tune_valid(int log_h, TreeTune t) {
  if (t.wide_log < 10 || t.wide_log > 18 || t.split < -1 || t.split > 1) return false;
  // the narrow part has S <= wide_log levels; both subtree launches hold at
  // most 512 nodes per CTA (1024 threads)
  int S = std::min(log_h, t.wide_log);
  int log_g = std::max(0, std::min(S, (S + t.split) / 2));
  return S - log_g <= 9 && log_g <= 9;
}
void set_tree_tune(int log_h, TreeTune t) {
  if (log_h < 0 || log_h > 40 || !tree_tune_valid(log_h, t)) return;
  g_tree_tune[log_h].store((t.wide_log << 4) | (t.split + 2), std::memory_order_relaxed);
}

static cudaError_t launch_subtrees(uint32_t *nodes, int log_h, int l0, int log_g, cudaStream_t st,
                                   uint32_t *host_root, unsigned int *flag, unsigned int seq) {
  int steps = log_h - l0 - log_g;
  if (steps <= 0) return cudaSuccess;
  int n = 1 << steps;  // nodes per CTA at level l0
  int threads = 2 * n < 32 ? 32 : 2 * n;  // a quad per node made at the first step
  launch(tree_subtrees, 1u << log_g, threads, (size_t)n * 32, st, nodes, log_h, l0, steps,
         host_root, flag, seq, 1u);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t build_tree(uint32_t *nodes, int log_h, cudaStream_t st, uint32_t *host_root,
                       unsigned int *flag, unsigned int seq) {
  const int T = 128;
  TreeTune tune = tree_tune(log_h);
  if (!tree_tune_valid(log_h, tune)) tune = TreeTune();
  int l = 0;
  for (; l < log_h && ((size_t)1 << (log_h - l)) / 2 >= ((size_t)1 << tune.wide_log); l++) {
    size_t half = ((size_t)1 << (log_h - l)) / 2;
    launch(compress_level, (unsigned)((half + T - 1) / T), T, 0, st,
           nodes + level_offset_words(log_h, l), nodes + level_offset_words(log_h, l + 1),
           half);
    count_launches(1);
  }
  // remaining S = log_h - l steps (S <= wide_log): G = 2^((S + split)/2)
  // subtrees, then the top
  int S = log_h - l;
  int log_g = std::max(0, std::min(S, (S + tune.split) / 2));
  // only the last launch (one CTA, G = 1) reaches the root
  cudaError_t e = launch_subtrees(nodes, log_h, l, log_g, st, host_root, flag, seq);
  if (e != cudaSuccess) return e;
  return launch_subtrees(nodes, log_h, log_h - log_g, 0, st, host_root, flag, seq);
}

// ---- batched trees (kernels.h) ----
// Wide levels one thread per node, as build_tree; the remaining S levels up
// to the instances' roots in two subtree launches: batch 2^g CTAs climb
// S - g levels, then batch CTAs climb g (each CTA holds at most 512 nodes).
cudaError_t build_tree_batch(uint32_t *nodes, int log_h, int batch, cudaStream_t st) {
  if (batch < 1 || log_h < 0 || log_h > 30) return cudaErrorInvalidValue;
  const int T = 128;
  const size_t B = (size_t)batch;
  int l = 0;
  for (; l < log_h && (B << (log_h - l)) / 2 >= ((size_t)1 << 15); l++) {
    size_t half = (B << (log_h - l)) / 2;
    launch(compress_level, (unsigned)((half + T - 1) / T), T, 0, st,
           nodes + B * level_offset_words(log_h, l),
           nodes + B * level_offset_words(log_h, l + 1), half);
    count_launches(1);
  }
  const int S = log_h - l;
  if (S == 0) return cudaGetLastError();
  int g = S / 2;
  if (S - g > 9) g = S - 9;
  if (g > 9 || (B << g) > 0x7fffffffu) return cudaErrorInvalidValue;
  const int parts[2][2] = {{l, S - g}, {log_h - g, g}};  // (first level, steps)
  for (int i = 0; i < 2; i++) {
    const int l0 = parts[i][0], steps = parts[i][1];
    if (steps == 0) continue;
    const size_t G = B << (i == 0 ? g : 0);
    const int n = 1 << steps;
    const int threads = 2 * n < 32 ? 32 : 2 * n;
    launch(tree_subtrees, (unsigned)G, threads, (size_t)n * 32, st, nodes, log_h, l0, steps,
           nullptr, nullptr, 0, (unsigned)batch);
    count_launches(1);
  }
  return cudaGetLastError();
}

__global__ void gather_openings_batch_kernel(const uint32_t *__restrict__ rows, int row_len,
                                             const uint32_t *__restrict__ nodes, int log_h,
                                             unsigned batch, const uint32_t *__restrict__ idx,
                                             const int *__restrict__ inst, int n,
                                             uint32_t *__restrict__ out) {
  pdl_wait();
  const int q = blockIdx.x;
  if (q >= n) return;
  const size_t b = (size_t)inst[q], r = idx[q];
  const size_t per = (size_t)row_len + 8 * (size_t)log_h;
  uint32_t *o = out + q * per;
  const uint32_t *row = rows + (r * batch + b) * row_len;
  for (int j = threadIdx.x; j < row_len; j += blockDim.x) o[j] = row[j];
  for (int t = threadIdx.x; t < 8 * log_h; t += blockDim.x) {
    const int l = t / 8, w = t % 8;
    const size_t at = r & (((size_t)1 << (log_h - l)) - 1);  // the instance's node at level l
    const size_t sib = at ^ ((size_t)1 << (log_h - l - 1));
    o[row_len + t] = nodes[batch * level_offset_words(log_h, l) + (sib * batch + b) * 8 + w];
  }
}

cudaError_t gather_openings_batch(const uint32_t *rows, int row_len, const uint32_t *nodes,
                                  int log_h, int batch, const uint32_t *idx, const int *inst,
                                  int n, uint32_t *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (batch < 1) return cudaErrorInvalidValue;
  launch(gather_openings_batch_kernel, n, 128, 0, st, rows, row_len, nodes, log_h, (unsigned)batch,
         idx, inst, n, out);
  count_launches(1);
  return cudaGetLastError();
}

// dst row r = (src row r of instance 0, of instance 1, ...): 16-byte
// pieces when the row width allows, one thread per piece of dst
template <class T>
__global__ void interleave_kernel(const T *__restrict__ src, size_t rows, size_t w, size_t batch,
                                  T *__restrict__ dst) {
  pdl_wait();
  const size_t total = rows * w * batch;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t j = i % w, rb = i / w, b = rb % batch, r = rb / batch;
    dst[i] = src[(b * rows + r) * w + j];
  }
}

cudaError_t interleave_rows(const uint32_t *src, size_t rows, size_t w, int batch, uint32_t *dst,
                            cudaStream_t st) {
  if (batch < 1) return cudaErrorInvalidValue;
  const size_t total = rows * w * (size_t)batch;
  if (total == 0) return cudaSuccess;
  const unsigned T = 256;
  const bool vec = w % 4 == 0 && (((uintptr_t)src | (uintptr_t)dst) & 15) == 0;
  const size_t items = vec ? total / 4 : total;
  const size_t g = (items + T - 1) / T;
  const unsigned grid = (unsigned)(g < 152 * 32 ? g : 152 * 32);
  if (vec)
    launch(interleave_kernel<uint4>, grid, T, 0, st, reinterpret_cast<const uint4 *>(src), rows,
           w / 4, (size_t)batch, reinterpret_cast<uint4 *>(dst));
  else
    launch(interleave_kernel<uint32_t>, grid, T, 0, st, src, rows, w, (size_t)batch, dst);
  count_launches(1);
  return cudaGetLastError();
}

__device__ __forceinline__ void gather_one(const uint32_t *__restrict__ rows, int row_len,
                                           const uint32_t *__restrict__ nodes, int log_h,
                                           size_t index, int q, uint32_t *__restrict__ out) {
  size_t per = (size_t)row_len + 8 * (size_t)log_h;
  uint32_t *o = out + q * per;
  for (int j = threadIdx.x; j < row_len; j += blockDim.x) o[j] = rows[index * row_len + j];
  // sibling at level l is index_l ^ mid_l with mid_l = 2^(log_h - l - 1)
  for (int t = threadIdx.x; t < 8 * log_h; t += blockDim.x) {
    int l = t / 8, w = t % 8;
    size_t mask = ((size_t)1 << (log_h - l)) - 1;  // index at level l is index & mask
    size_t mid = (size_t)1 << (log_h - l - 1);
    size_t sib = (index & mask) ^ mid;
    o[row_len + t] = nodes[level_offset_words(log_h, l) + sib * 8 + w];
  }
}

__global__ void gather_openings_kernel(const uint32_t *__restrict__ rows, int row_len,
                                       const uint32_t *__restrict__ nodes, int log_h,
                                       const uint32_t *__restrict__ idx, int n,
                                       uint32_t *__restrict__ out) {
  pdl_wait();
  int q = blockIdx.x;
  if (q >= n) return;
  gather_one(rows, row_len, nodes, log_h, idx[q], q, out);
}
// the same with the indexes passed by value
__global__ void gather_openings_val_kernel(const uint32_t *__restrict__ rows, int row_len,
                                           const uint32_t *__restrict__ nodes, int log_h,
                                           const __grid_constant__ IdxArgs a, int n,
                                           uint32_t *__restrict__ out) {
  pdl_wait();
  int q = blockIdx.x;
  if (q >= n) return;
  gather_one(rows, row_len, nodes, log_h, a.idx[q], q, out);
}

cudaError_t gather_openings_val(const uint32_t *rows, int row_len, const uint32_t *nodes,
                                int log_h, const IdxArgs &a, int n, uint32_t *out,
                                cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (n > IdxArgs::N) return cudaErrorInvalidValue;
  launch(gather_openings_val_kernel, n, 128, 0, st, rows, row_len, nodes, log_h, a, n, out);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t gather_openings(const uint32_t *rows, int row_len, const uint32_t *nodes, int log_h,
                            const uint32_t *idx, int n, uint32_t *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  launch(gather_openings_kernel, n, 128, 0, st, rows, row_len, nodes, log_h, idx, n, out);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace gpu
}  // namespace whir
