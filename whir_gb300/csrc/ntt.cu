// Batched column DFT over KoalaBear for the Reed-Solomon encoding
// (p3 TwoAdicSubgroupDft::dft_batch / dft_algebra_batch called at
// crates/whir/src/whir.rs:34,59).
//
// A row-major matrix of `width` columns is transformed down each column.
// Sizes up to 2^11 run in one pass: a CTA stages one column slice of the
// whole column in shared memory and runs radix-2 stages there.  Larger sizes
// use the four-step split M = M1 * M2:
//   pass 1: for each n2, a size-M1 DFT of x[M2 n1 + n2] (stride M2 rows),
//           times w_M^(n2 k1), stored at row M2 k1 + n2;
//   pass 2: for each k1, a size-M2 DFT of the contiguous rows M2 k1 + n2,
//           stored at row k1 + M1 k2.
// Each pass reads and writes the matrix once with full 32-byte sectors (a
// CTA owns 8 columns = 32 bytes of every row it touches).  Zero padding is
// never materialised: rows >= h_in are read as zero in pass 1.
#include "kernels.h"

namespace whir {
namespace gpu {

// powers of the 2^24-th root of unity: w^e = lo[e & 4095] * hi[e >> 12]
__device__ uint32_t g_tw_lo[4096];
__device__ uint32_t g_tw_hi[4096];

static const uint32_t ROOT24 = 0x6ac49f88u;  // two_adic_generator(24), canonical

cudaError_t init_poseidon2_tables();

cudaError_t init_device_tables() {
  static uint32_t lo[4096], hi[4096];
  uint32_t w = kb::from_canonical(ROOT24);
  uint32_t w4096 = kb::pow(w, 4096);
  lo[0] = hi[0] = kb::ONE;
  for (int i = 1; i < 4096; i++) {
    lo[i] = kb::mul(lo[i - 1], w);
    hi[i] = kb::mul(hi[i - 1], w4096);
  }
  cudaError_t e = cudaMemcpyToSymbol(g_tw_lo, lo, sizeof lo);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_tw_hi, hi, sizeof hi);
  if (e == cudaSuccess) e = init_poseidon2_tables();
  return e;
}

__device__ __forceinline__ uint32_t root_pow(uint32_t e24) {  // w_24^e, e < 2^24
  return kb::mul(g_tw_lo[e24 & 4095], g_tw_hi[e24 >> 12]);
}

__device__ __forceinline__ uint32_t brev(uint32_t i, int bits) {
  return bits ? (__brev(i) >> (32 - bits)) : 0;
}

constexpr int MAX_TILE_LOG = 12;

// o = blockIdx.x selects the sub-transform; in_row = o*a_in + i*b_in,
// out_row = o*a_out + k*b_out.  tw_log > 0 multiplies output k by
// w_{2^tw_log}^(o*k) (the four-step twiddle).
template <int C>
__global__ void __launch_bounds__(512) dft_tile(const uint32_t *__restrict__ in,
                                                uint32_t *__restrict__ out, int S, size_t width,
                                                size_t rows_valid, size_t a_in, size_t b_in,
                                                size_t a_out, size_t b_out, int tw_log) {
  extern __shared__ uint32_t sm[];
  const int n = 1 << S;
  uint32_t *tile = sm;
  uint32_t *tw = sm + n * C;
  const size_t o = blockIdx.x;
  const size_t col0 = (size_t)blockIdx.y * C;
  const int tid = threadIdx.x, nt = blockDim.x;

  for (int j = tid; j < n / 2; j += nt) tw[j] = root_pow((uint32_t)j << (24 - S));
  for (int e = tid; e < n * C; e += nt) {
    int i = e / C, c = e % C;
    size_t row = o * a_in + (size_t)i * b_in;
    uint32_t v = row < rows_valid ? __ldg(in + row * width + col0 + c) : 0u;
    tile[brev(i, S) * C + c] = v;
  }
  __syncthreads();
  for (int s = 1; s <= S; s++) {
    const int half = 1 << (s - 1);
    for (int b = tid; b < (n / 2) * C; b += nt) {
      int c = b % C, j = b / C;
      int pos = j & (half - 1);
      int i0 = ((j >> (s - 1)) << s) + pos, i1 = i0 + half;
      uint32_t u = tile[i0 * C + c];
      uint32_t v = kb::mul(tile[i1 * C + c], tw[pos << (S - s)]);
      tile[i0 * C + c] = kb::add(u, v);
      tile[i1 * C + c] = kb::sub(u, v);
    }
    __syncthreads();
  }
  for (int e = tid; e < n * C; e += nt) {
    int k = e / C, c = e % C;
    uint32_t v = tile[k * C + c];
    if (tw_log) {
      uint64_t ex = ((uint64_t)o * (uint64_t)k) & ((1ull << tw_log) - 1);
      v = kb::mul(v, root_pow((uint32_t)(ex << (24 - tw_log))));
    }
    out[(o * a_out + (size_t)k * b_out) * width + col0 + c] = v;
  }
}

template <int C>
static cudaError_t launch_tile(const uint32_t *in, uint32_t *out, int S, size_t width,
                               size_t rows_valid, size_t n_outer, size_t a_in, size_t b_in,
                               size_t a_out, size_t b_out, int tw_log, cudaStream_t st) {
  size_t smem = ((size_t)(1 << S) * C + (1 << S) / 2 + 1) * 4;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(dft_tile<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         ((1 << MAX_TILE_LOG) * C + (1 << MAX_TILE_LOG) / 2 + 1) * 4);
    attr_set = true;
  }
  int threads = (1 << S) * C / 2;
  threads = threads < 32 ? 32 : (threads > 512 ? 512 : threads);
  dim3 grid((unsigned)n_outer, (unsigned)(width / C));
  dft_tile<C><<<grid, threads, smem, st>>>(in, out, S, width, rows_valid, a_in, b_in, a_out,
                                           b_out, tw_log);
  count_launches(1);
  return cudaGetLastError();
}

static cudaError_t tile_any(const uint32_t *in, uint32_t *out, int S, size_t width,
                            size_t rows_valid, size_t n_outer, size_t a_in, size_t b_in,
                            size_t a_out, size_t b_out, int tw_log, cudaStream_t st) {
  if (width % 8 == 0)
    return launch_tile<8>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                          tw_log, st);
  if (width % 4 == 0)
    return launch_tile<4>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                          tw_log, st);
  if (width % 2 == 0)
    return launch_tile<2>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                          tw_log, st);
  return launch_tile<1>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                        tw_log, st);
}

cudaError_t dft_batch(const uint32_t *in, size_t h_in, size_t width, int log_h, uint32_t *out,
                      uint32_t *scratch, cudaStream_t st) {
  if (log_h < 0 || log_h > 24 || width == 0) return cudaErrorInvalidValue;
  size_t h = (size_t)1 << log_h;
  if (h_in > h) return cudaErrorInvalidValue;
  if (log_h <= 11)
    return tile_any(in, out, log_h, width, h_in, 1, 0, 1, 0, 1, 0, st);
  int L1 = (log_h + 1) / 2, L2 = log_h - L1;
  if (L1 > MAX_TILE_LOG) return cudaErrorInvalidValue;
  size_t M1 = (size_t)1 << L1, M2 = (size_t)1 << L2;
  cudaError_t e = tile_any(in, scratch, L1, width, h_in, M2, 1, M2, 1, M2, log_h, st);
  if (e != cudaSuccess) return e;
  return tile_any(scratch, out, L2, width, h, M1, M2, 1, 1, M1, 0, st);
}

}  // namespace gpu
}  // namespace whir
