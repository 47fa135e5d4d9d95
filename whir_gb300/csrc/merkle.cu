// Merkle commitment kernels: leaf hashing (width-24 sponge), tree ascent
// (width-16 truncated-permutation compression, halves pairing) and the
// opening gather.  Tree shape and hashing follow
// crates/merkle/src/poseidon_packed.rs:98-143,269-304,344-384 and
// crates/merkle/src/poseidon.rs:33-74.
#include <atomic>

#include "kernels.h"
#include "p2_device.cuh"
#include "poseidon2_host.h"

namespace whir {
namespace gpu {

static cudaError_t upload_p2(int width) {
  const Poseidon2Constants &c = poseidon2_constants(width);
  uint32_t buf[8 * 24 + 23 + 24];
  int n = 0;
  for (int r = 0; r < 8; r++)
    for (int i = 0; i < width; i++) buf[n++] = c.ext_rc[r][i];
  for (int r = 0; r < c.rounds_p; r++) buf[n++] = c.int_rc[r];
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

// One row per thread; rows of 16 words are one permutation, rows of 64 words
// four (PaddingFreeSponge: overwrite the 16 rate lanes, permute).
template <int ROW>
__global__ void __launch_bounds__(128) hash_rows_fixed(const uint32_t *__restrict__ rows,
                                                       size_t n_rows,
                                                       uint32_t *__restrict__ digests) {
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

cudaError_t hash_rows(const uint32_t *rows, size_t n_rows, int row_len, uint32_t *digests,
                      cudaStream_t st) {
  if (n_rows == 0) return cudaSuccess;
  const int T = 128;
  unsigned grid = (unsigned)((n_rows + T - 1) / T);
  // the fixed-width kernels use 16-byte vector loads and stores
  bool aligned = (((uintptr_t)rows | (uintptr_t)digests) & 15) == 0;
  if (aligned && row_len == 16) hash_rows_fixed<16><<<grid, T, 0, st>>>(rows, n_rows, digests);
  else if (aligned && row_len == 64) hash_rows_fixed<64><<<grid, T, 0, st>>>(rows, n_rows, digests);
  else hash_rows_generic<<<grid, T, 0, st>>>(rows, n_rows, row_len, digests);
  count_launches(1);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) compress_level(const uint32_t *__restrict__ src,
                                                      uint32_t *__restrict__ dst, size_t half) {
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

// ---- warp-cooperative width-16 permutation for the small tree levels ----
// A level with few nodes is bound by the latency of one permutation, not by
// throughput.  Here the 16 lanes of a half-warp hold the 16 state words, so
// the S-boxes of a full round run in parallel and the linear layers are a
// few shuffles: mat4 inside each group of 4 lanes, column sums by xor
// shuffles across groups, and the internal layer's sum by a 4-step xor
// reduction.  Two nodes per warp (lanes 0-15 and 16-31).
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ uint32_t p2w_mds(uint32_t x, int l) {
  using namespace kb;
  const int g = l & ~3;  // first lane of this group of 4 (shuffle width 16)
  uint32_t x0 = __shfl_sync(FULL, x, g, 16), x1 = __shfl_sync(FULL, x, g + 1, 16);
  uint32_t x2 = __shfl_sync(FULL, x, g + 2, 16), x3 = __shfl_sync(FULL, x, g + 3, 16);
  uint32_t t01 = add(x0, x1), t23 = add(x2, x3), t0123 = add(t01, t23);
  uint32_t t01123 = add(t0123, x1), t01233 = add(t0123, x3);
  uint32_t y;
  switch (l & 3) {
    case 0: y = add(t01123, t01); break;
    case 1: y = add(t01123, dbl(x2)); break;
    case 2: y = add(t01233, t23); break;
    default: y = add(t01233, dbl(x0)); break;
  }
  uint32_t s = add(y, __shfl_xor_sync(FULL, y, 4, 16));
  s = add(s, __shfl_xor_sync(FULL, s, 8, 16));
  return add(y, s);
}

struct P2WarpConsts {
  uint32_t ext[8];  // this lane's external round constants
  uint32_t diag;    // this lane's internal diagonal entry
};
__device__ __forceinline__ P2WarpConsts p2w_consts(int l) {
  P2WarpConsts k;
#pragma unroll
  for (int r = 0; r < 8; r++) k.ext[r] = c_p2_16[r * 16 + l];
  k.diag = c_p2_16[8 * 16 + 20 + l];
  return k;
}

__device__ __forceinline__ uint32_t p2w_permute(uint32_t x, int l, const P2WarpConsts &k) {
  using namespace kb;
  x = p2w_mds(x, l);
#pragma unroll
  for (int r = 0; r < 4; r++) x = p2w_mds(cube(add(x, k.ext[r])), l);
#pragma unroll 4
  for (int r = 0; r < 20; r++) {
    uint32_t y = cube(add(x, c_p2_16[8 * 16 + r]));
    x = l == 0 ? y : x;
    uint32_t s = add(x, __shfl_xor_sync(FULL, x, 1, 16));
    s = add(s, __shfl_xor_sync(FULL, s, 2, 16));
    s = add(s, __shfl_xor_sync(FULL, s, 4, 16));
    s = add(s, __shfl_xor_sync(FULL, s, 8, 16));
    x = add(s, mul(k.diag, x));
  }
#pragma unroll
  for (int r = 4; r < 8; r++) x = p2w_mds(cube(add(x, k.ext[r])), l);
  return x;
}

// node i of the next level = C(src[i], src[i + half]); half-warp per node
__device__ __forceinline__ void p2w_compress(const uint32_t *src, uint32_t *dst, size_t half,
                                             size_t node, int l, const P2WarpConsts &k) {
  bool live = node < half;
  uint32_t x = 0;
  if (live) x = l < 8 ? src[node * 8 + l] : src[(node + half) * 8 + (l - 8)];
  x = p2w_permute(x, l, k);  // every lane of the warp takes part in the shuffles
  if (live && l < 8) dst[node * 8 + l] = x;
}

__global__ void __launch_bounds__(256) compress_level_warp(const uint32_t *__restrict__ src,
                                                           uint32_t *__restrict__ dst,
                                                           size_t half) {
  const int l = threadIdx.x & 15;
  const P2WarpConsts k = p2w_consts(l);
  size_t node = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 4;
  p2w_compress(src, dst, half, node, l, k);
}

// the last levels of a tree (each at most 2^TOP_LOG nodes) in one CTA
constexpr int TOP_LOG = 9;
__global__ void __launch_bounds__(1024) tree_top(uint32_t *nodes, int log_h, int from_level) {
  const int l = threadIdx.x & 15;
  const P2WarpConsts k = p2w_consts(l);
  const size_t slots = blockDim.x >> 4;
  for (int lev = from_level; lev < log_h; lev++) {
    size_t half = ((size_t)1 << (log_h - lev)) / 2;
    const uint32_t *src = nodes + level_offset_words(log_h, lev);
    uint32_t *dst = nodes + level_offset_words(log_h, lev + 1);
    for (size_t base = 0; base < half; base += slots)
      p2w_compress(src, dst, half, base + (threadIdx.x >> 4), l, k);
    __syncthreads();
  }
}

cudaError_t build_tree(uint32_t *nodes, int log_h, cudaStream_t st) {
  const int T = 128;
  int l = 0;
  // wide levels: one thread per node (throughput)
  for (; l < log_h && ((size_t)1 << (log_h - l)) / 2 >= ((size_t)1 << 15); l++) {
    size_t half = ((size_t)1 << (log_h - l)) / 2;
    compress_level<<<(unsigned)((half + T - 1) / T), T, 0, st>>>(
        nodes + level_offset_words(log_h, l), nodes + level_offset_words(log_h, l + 1), half);
    count_launches(1);
  }
  // middle levels: half a warp per node (latency)
  for (; l < log_h && ((size_t)1 << (log_h - l)) / 2 > ((size_t)1 << TOP_LOG); l++) {
    size_t half = ((size_t)1 << (log_h - l)) / 2;
    size_t threads = half * 16;
    compress_level_warp<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
        nodes + level_offset_words(log_h, l), nodes + level_offset_words(log_h, l + 1), half);
    count_launches(1);
  }
  // top levels: one CTA, one launch
  if (l < log_h) {
    tree_top<<<1, 1024, 0, st>>>(nodes, log_h, l);
    count_launches(1);
  }
  return cudaGetLastError();
}

__global__ void gather_openings_kernel(const uint32_t *__restrict__ rows, int row_len,
                                       const uint32_t *__restrict__ nodes, int log_h,
                                       const uint32_t *__restrict__ idx, int n,
                                       uint32_t *__restrict__ out) {
  int q = blockIdx.x;
  if (q >= n) return;
  size_t index = idx[q];
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

cudaError_t gather_openings(const uint32_t *rows, int row_len, const uint32_t *nodes, int log_h,
                            const uint32_t *idx, int n, uint32_t *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  gather_openings_kernel<<<n, 128, 0, st>>>(rows, row_len, nodes, log_h, idx, n, out);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace gpu
}  // namespace whir
