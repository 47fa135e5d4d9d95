// Batched column DFT over KoalaBear for the Reed-Solomon encoding
// (p3 TwoAdicSubgroupDft::dft_batch / dft_algebra_batch called at
// crates/whir/src/whir.rs:34,59).
//
// A row-major matrix of `width` columns is transformed down each column.
// Sizes up to 2^11 run in one pass: a CTA stages one column slice of the
// whole column in shared memory and runs a decimation-in-frequency transform
// there, three radix-2 stages per step in registers.  When the nonzero input
// has at most 2^12 rows (every WHIR round after the first, whose rate grows),
// the codeword is a set of independent coset transforms of that input and
// also takes one pass.  Otherwise sizes
// use the four-step split M = M1 * M2:
//   pass 1: for each n2, a size-M1 DFT of x[M2 n1 + n2] (stride M2 rows),
//           times w_M^(n2 k1), stored at row M2 k1 + n2;
//   pass 2: for each k1, a size-M2 DFT of the contiguous rows M2 k1 + n2,
//           stored at row k1 + M1 k2.
// Each pass reads and writes the matrix once with full 32-byte sectors (a
// CTA owns 8 columns = 32 bytes of every row it touches).  Zero padding is
// never materialised: rows >= h_in are read as zero in pass 1.
#include <atomic>
#include <type_traits>
#include <mutex>

#include "kernels.h"
#include "launch.cuh"

#include <type_traits>

namespace whir {
namespace gpu {

// powers of the 2^24-th root of unity: w^e = lo[e & 4095] * hi[e >> 12]
__device__ uint32_t g_tw_lo[4096];
__device__ uint32_t g_tw_hi[4096];
// DIF twiddles: g_dif[h + pos] = w_{2h}^pos for h = 1, 2, .., 2048 and pos < h
// (the entry depends on the index alone, so one table serves every size)
__device__ uint32_t g_dif[4096];
// the same twiddles for Shoup products: {plain value w, floor(w 2^32 / p)}
__device__ uint2 g_dif2[4096];

static const uint32_t ROOT24 = 0x6ac49f88u;  // two_adic_generator(24), canonical

cudaError_t init_poseidon2_tables();

static cudaError_t upload_device_tables() {
  static uint32_t lo[4096], hi[4096];
  uint32_t w = kb::from_canonical(ROOT24);
  uint32_t w4096 = kb::pow(w, 4096);
  lo[0] = hi[0] = kb::ONE;
  for (int i = 1; i < 4096; i++) {
    lo[i] = kb::mul(lo[i - 1], w);
    hi[i] = kb::mul(hi[i - 1], w4096);
  }
  static uint32_t dif[4096];
  dif[0] = 0;
  for (int x = 1; x < 4096; x++) {
    int lh = 31 - __builtin_clz((unsigned)x);
    uint32_t pos = (uint32_t)(x - (1 << lh));
    uint32_t e = pos << (24 - 1 - lh);  // w_{2^(lh+1)}^pos = w_24^(pos 2^(23-lh))
    dif[x] = kb::mul(lo[e & 4095], hi[e >> 12]);
  }
  cudaError_t e = cudaMemcpyToSymbol(g_tw_lo, lo, sizeof lo);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_tw_hi, hi, sizeof hi);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_dif, dif, sizeof dif);
  static uint2 dif2[4096];
  for (int x = 0; x < 4096; x++) {
    uint32_t w = kb::to_canonical(dif[x]);
    dif2[x] = make_uint2(w, (uint32_t)(((uint64_t)w << 32) / kb::P));
  }
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_dif2, dif2, sizeof dif2);
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

// Index maps of the vectorised tile beyond the linear ones: sub-transform o
// reads input row (o & in_mask) * a_in + i * b_in, its pre-twiddle exponent
// is (o >> pre_shift) * i, and its post-twiddle exponent is
// (o & post_mask) * ((o >> post_shift) + (k << post_kshift)).  The identity
// map (all-ones masks, shifts 0, 31, 0) gives o * i and o * k.
struct TileIdx {
  uint32_t in_mask = 0xffffffffu;
  int pre_shift = 0;
  uint32_t post_mask = 0xffffffffu;
  int post_shift = 31;
  int post_kshift = 0;
};

// Shared-memory tile index of (row, column): rows are permuted inside each
// aligned group of 4 by XOR with bits 3..4 of the row, so that the 4 rows a
// warp touches at once (consecutive rows, or rows 8 apart in the last radix
// steps) fall in different 8-bank groups.
template <int C>
__device__ __forceinline__ int sidx(int row, int c) {
  return (row ^ ((row >> 3) & 3)) * C + c;
}

// One decimation-in-frequency step of R radix-2 stages done in registers:
// the first stage has half-size H = 2^lh (blocks of 2H, never straddling two
// sub-transforms), each task owns the 2^R elements j + t*q (q = H / 2^(R-1))
// of one block and one column.
// Butterfly at half h, position pos: (a, b) -> (a + b, (a - b) * w_{2h}^pos),
// with w_{2h}^pos stored at twl[h + pos] (one contiguous table per level, so
// consecutive positions read consecutive banks).
template <int C, int R>
__device__ __forceinline__ void dif_step(uint32_t *tile, const uint32_t *twl, int S_rows, int lh) {
  constexpr int T = 1 << R;
  const int lq = lh - (R - 1);
  const int q = 1 << lq, H = 1 << lh;
  const int tasks = (1 << (S_rows - R)) * C;  // all 2^S_rows tile rows, 2^R per task
  for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
    const int c = task % C, rest = task / C;
    const int j = rest & (q - 1), blk = rest >> lq;
    const int base = blk * 2 * H + j;
    uint32_t v[T];
#pragma unroll
    for (int t = 0; t < T; t++) v[t] = tile[sidx<C>(base + t * q, c)];
#pragma unroll
    for (int st = 0; st < R; st++) {
      const int span = T >> (st + 1);
      const int hh = H >> st;
      if (hh == 1) {  // the last stage of the transform: every twiddle is 1
#pragma unroll
        for (int t = 0; t < T; t += 2) {
          uint32_t a = v[t], b = v[t + 1];
          v[t] = kb::add(a, b);
          v[t + 1] = kb::sub(a, b);
        }
        continue;
      }
#pragma unroll
      for (int t = 0; t < T; t++) {
        if (t & span) continue;
        const int pos = j + (t & (span - 1)) * q;
        uint32_t a = v[t], b = v[t + span];
        v[t] = kb::add(a, b);
        // a - b + p < 2^32 needs no reduction before a Montgomery product
        // with a canonical twiddle (the product stays below p 2^32)
        v[t + span] = kb::mul(a - b + kb::P, twl[hh + pos]);
      }
    }
#pragma unroll
    for (int t = 0; t < T; t++) tile[sidx<C>(base + t * q, c)] = v[t];
  }
}

// blockIdx.x selects the column slice (fastest, so the CTAs sharing a row's
// 32-byte sectors run together and the row is fetched from DRAM once);
// blockIdx.y selects 2^lg consecutive sub-transforms o, each of size 2^S,
// held back to back in the tile.  in_row = o*a_in + i*b_in and out_row =
// o*a_out + k*b_out.  pre_log > 0 multiplies input i by w_{2^pre_log}^(o*i)
// (coset transforms of a zero-padded input); tw_log > 0 multiplies output k
// by w_{2^tw_log}^(o*k) (the four-step twiddle).  The DIF leaves X[k] at
// position bitrev(k) of its sub-transform.  Index arithmetic is 32-bit: the
// launcher only uses this kernel when every word offset fits.
template <int C>
__global__ void __launch_bounds__(256) dft_tile(const uint32_t *__restrict__ in,
                                                uint32_t *__restrict__ out, int S, int lg,
                                                uint32_t width, uint32_t rows_valid,
                                                uint32_t a_in, uint32_t b_in, uint32_t a_out,
                                                uint32_t b_out, int pre_log, int tw_log) {
  pdl_wait();
  extern __shared__ uint32_t sm[];
  const int n = 1 << S, rows = n << lg;
  uint32_t *tile = sm;
  // aux holds, in turn: the per-row input twiddles, the DIF twiddles
  // (aux[h + pos] = w_{2h}^pos for h = 1, 2, .., n/2), the per-row output twiddles
  uint32_t *aux = sm + rows * C;
  const uint32_t o0 = blockIdx.y << lg;
  const uint32_t col0 = blockIdx.x * C;
  const int tid = threadIdx.x, nt = blockDim.x;

  if (pre_log) {
    const uint32_t m = (1u << pre_log) - 1u;
    for (int r = tid; r < rows; r += nt) {
      uint32_t o = o0 + (uint32_t)(r >> S), i = (uint32_t)(r & (n - 1));
      aux[r] = root_pow(((o * i) & m) << (24 - pre_log));
    }
    __syncthreads();
  }
  for (int e = tid; e < rows * C; e += nt) {
    int r = e / C, c = e % C;
    uint32_t o = o0 + (uint32_t)(r >> S), i = (uint32_t)(r & (n - 1));
    uint32_t row = o * a_in + i * b_in;
    uint32_t v = row < rows_valid ? __ldg(in + row * width + col0 + c) : 0u;
    if (pre_log) v = kb::mul(v, aux[r]);
    tile[sidx<C>(r, c)] = v;
  }
  __syncthreads();
  for (int x = tid + 1; x < n; x += nt) {
    int lh = 31 - __clz(x);
    uint32_t pos = (uint32_t)(x - (1 << lh));
    aux[x] = root_pow(pos << (24 - 1 - lh));  // w_{2^(lh+1)}^pos
  }
  __syncthreads();
  int left = S, lh = S - 1;
  while (left >= 3) {
    dif_step<C, 3>(tile, aux, S + lg, lh);
    __syncthreads();
    left -= 3;
    lh -= 3;
  }
  if (left == 2) {
    dif_step<C, 2>(tile, aux, S + lg, lh);
    __syncthreads();
  } else if (left == 1) {
    dif_step<C, 1>(tile, aux, S + lg, lh);
    __syncthreads();
  }
  if (tw_log) {
    const uint32_t m = (1u << tw_log) - 1u;
    for (int r = tid; r < rows; r += nt) {
      uint32_t o = o0 + (uint32_t)(r >> S), k = brev((uint32_t)(r & (n - 1)), S);
      aux[r] = root_pow(((o * k) & m) << (24 - tw_log));
    }
    __syncthreads();
  }
  for (int e = tid; e < rows * C; e += nt) {
    int r = e / C, c = e % C;
    uint32_t v = tile[sidx<C>(r, c)];
    uint32_t o = o0 + (uint32_t)(r >> S);
    uint32_t k = brev((uint32_t)(r & (n - 1)), S);
    if (tw_log) v = kb::mul(v, aux[r]);
    out[(o * a_out + k * b_out) * width + col0 + c] = v;
  }
}

// ---- vectorised tile: 4 columns per task ----
// The same transform as dft_tile, for column slices of C = 4 or 8 words held
// as uint4: a task moves and butterflies 4 columns at once, so shared-memory
// instructions, index arithmetic and twiddle loads are shared by 4 columns.
// Rows are permuted inside aligned groups of 32 / C rows (one group spans
// the 32 banks) by XOR with bits 3.. of the row, which keeps the 8 lanes of
// a 128-byte phase on distinct banks for row strides 1, 8 and 2^k >= 8.
template <int C>
__device__ __forceinline__ int vrow(int row) {
  return row ^ ((row >> 3) & (32 / C - 1));
}
__device__ __forceinline__ uint4 add4(uint4 a, uint4 b) {
  return make_uint4(kb::add(a.x, b.x), kb::add(a.y, b.y), kb::add(a.z, b.z), kb::add(a.w, b.w));
}
__device__ __forceinline__ uint4 sub4(uint4 a, uint4 b) {
  return make_uint4(kb::sub(a.x, b.x), kb::sub(a.y, b.y), kb::sub(a.z, b.z), kb::sub(a.w, b.w));
}
// (a - b) * w for a canonical twiddle w (a - b + p < 2^32 needs no reduction)
__device__ __forceinline__ uint4 submul4(uint4 a, uint4 b, uint32_t w) {
  return make_uint4(kb::mul(a.x - b.x + kb::P, w), kb::mul(a.y - b.y + kb::P, w),
                    kb::mul(a.z - b.z + kb::P, w), kb::mul(a.w - b.w + kb::P, w));
}
__device__ __forceinline__ uint4 mul4(uint4 a, uint32_t w) {
  return make_uint4(kb::mul(a.x, w), kb::mul(a.y, w), kb::mul(a.z, w), kb::mul(a.w, w));
}

// Twiddle sources for the vectorised steps.  TwMont: Montgomery words (a
// shared table); TwShoup: the plain value w and floor(w 2^32 / p) (a global
// table), so (a - b) w mod p is one high and two low products and one
// correction (Shoup's method); both give the same field element.
struct TwMont {
  const uint32_t *t;
  __device__ __forceinline__ uint4 submul(uint4 a, uint4 b, int i) const {
    return submul4(a, b, t[i]);
  }
};
__device__ __forceinline__ uint32_t shoup_mul(uint32_t d, uint2 w) {  // d < 2^32
  uint32_t q = __umulhi(d, w.y);
  uint32_t r = d * w.x - q * kb::P;  // in [0, 2p)
  return kb::umin(r, r - kb::P);
}
struct TwShoup {
  const uint2 *t;
  __device__ __forceinline__ uint4 submul(uint4 a, uint4 b, int i) const {
    return submul_w(a, b, t[i]);
  }
  static __device__ __forceinline__ uint4 submul_w(uint4 a, uint4 b, uint2 w) {
    return make_uint4(shoup_mul(a.x - b.x + kb::P, w), shoup_mul(a.y - b.y + kb::P, w),
                      shoup_mul(a.z - b.z + kb::P, w), shoup_mul(a.w - b.w + kb::P, w));
  }
};

// The 7 twiddles of a radix-8 task with block offset j, in the order
// dif_step_v reads them (entry hh + j + tl q with hh = H >> st): stage 0's
// four in slots 0..3, stage 1's two in 4..5, stage 2's one in 6.
struct Tw8 {
  uint2 w[7];
  __device__ __forceinline__ void load(const uint2 *t, int H, int j, int q) {
#pragma unroll
    for (int tl = 0; tl < 4; tl++) w[tl] = t[H + j + tl * q];
#pragma unroll
    for (int tl = 0; tl < 2; tl++) w[4 + tl] = t[(H >> 1) + j + tl * q];
    w[6] = t[(H >> 2) + j];
  }
};

// R radix-2 DIF stages in registers (see dif_step).  LAST: the final step of
// the transform, where the block stride q is 1, the first half-size is
// 2^(R-1) and position 0 of every stage has twiddle 1.
template <int C, int R, bool LAST, class TW>
__device__ __forceinline__ void dif_step_v(uint4 *tile, const TW &tw, int rows_log, int lh) {
  constexpr int T = 1 << R, V = C / 4, LV = V == 2 ? 1 : 0;
  const int lq = LAST ? 0 : lh - (R - 1);
  const int q = 1 << lq;
  const int H = LAST ? (1 << (R - 1)) : (1 << lh);
  const int tasks = (1 << (rows_log - R)) << LV;
  if constexpr (R == 3 && !LAST && std::is_same<TW, TwShoup>::value) {
    // every task of a thread has the same block offset j when the block's
    // task stride is a multiple of q: its 7 twiddles are loaded once
    if (((blockDim.x >> LV) & (q - 1)) == 0) {
      Tw8 w8;
      w8.load(tw.t, H, (threadIdx.x >> LV) & (q - 1), q);
      for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
        const int c = task & (V - 1), rest = task >> LV;
        const int j = rest & (q - 1), blk = rest >> lq;
        const int base = blk * 2 * H + j;
        uint4 v[T];
#pragma unroll
        for (int t = 0; t < T; t++) v[t] = tile[vrow<C>(base + t * q) * V + c];
#pragma unroll
        for (int st = 0; st < R; st++) {
          const int span = T >> (st + 1);
#pragma unroll
          for (int t = 0; t < T; t++) {
            if (t & span) continue;
            const int tl = t & (span - 1);
            uint4 a = v[t], b = v[t + span];
            v[t] = add4(a, b);
            v[t + span] = TwShoup::submul_w(a, b, w8.w[(st == 0 ? 0 : st == 1 ? 4 : 6) + tl]);
          }
        }
#pragma unroll
        for (int t = 0; t < T; t++) tile[vrow<C>(base + t * q) * V + c] = v[t];
      }
      return;
    }
  }
  for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
    const int c = task & (V - 1), rest = task >> LV;
    const int j = rest & (q - 1), blk = rest >> lq;
    const int base = blk * 2 * H + j;
    uint4 v[T];
#pragma unroll
    for (int t = 0; t < T; t++) v[t] = tile[vrow<C>(base + t * q) * V + c];
#pragma unroll
    for (int st = 0; st < R; st++) {
      const int span = T >> (st + 1);
      const int hh = H >> st;
#pragma unroll
      for (int t = 0; t < T; t++) {
        if (t & span) continue;
        const int tl = t & (span - 1);
        uint4 a = v[t], b = v[t + span];
        v[t] = add4(a, b);
        if (LAST && tl == 0) v[t + span] = sub4(a, b);  // w^0 = 1
        else v[t + span] = tw.submul(a, b, hh + j + tl * q);
      }
    }
#pragma unroll
    for (int t = 0; t < T; t++) tile[vrow<C>(base + t * q) * V + c] = v[t];
  }
}

template <int C, int R>
__device__ __forceinline__ void dif_run_v(uint4 *tile, const uint32_t *twl, int rows_log, int lh) {
  TwMont tw{twl};
  if (lh == R - 1) dif_step_v<C, R, true>(tile, tw, rows_log, lh);
  else dif_step_v<C, R, false>(tile, tw, rows_log, lh);
  __syncthreads();
}

// Arguments as dft_tile; C in {4, 8}; the rows of `in` and `out` start on
// 16-byte boundaries (width % 4 == 0, aligned base pointers).
template <int C>
__global__ void __launch_bounds__(256) dft_tile_v(const uint32_t *__restrict__ in,
                                                  uint32_t *__restrict__ out, int S, int lg,
                                                  uint32_t width, uint32_t rows_valid,
                                                  uint32_t a_in, uint32_t b_in, uint32_t a_out,
                                                  uint32_t b_out, int pre_log, int tw_log) {
  pdl_wait();
  constexpr int V = C / 4, LV = V == 2 ? 1 : 0;
  extern __shared__ uint4 smv[];
  const int n = 1 << S, rows = n << lg;
  uint4 *tile = smv;
  uint32_t *aux = reinterpret_cast<uint32_t *>(smv + rows * V);
  const uint32_t o0 = blockIdx.y << lg;
  const uint32_t v0 = blockIdx.x * V;  // first uint4 of the slice in a row
  const uint32_t wv = width / 4;       // uint4 per matrix row
  const uint4 *in4 = reinterpret_cast<const uint4 *>(in);
  uint4 *out4 = reinterpret_cast<uint4 *>(out);
  const int tid = threadIdx.x, nt = blockDim.x;

  if (pre_log) {
    const uint32_t m = (1u << pre_log) - 1u;
    for (int r = tid; r < rows; r += nt) {
      uint32_t o = o0 + (uint32_t)(r >> S), i = (uint32_t)(r & (n - 1));
      aux[r] = root_pow(((o * i) & m) << (24 - pre_log));
    }
    __syncthreads();
  }
  for (int e = tid; e < rows * V; e += nt) {
    int r = e >> LV, c = e & (V - 1);
    uint32_t o = o0 + (uint32_t)(r >> S), i = (uint32_t)(r & (n - 1));
    uint32_t row = o * a_in + i * b_in;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (row < rows_valid) v = __ldg(in4 + row * wv + v0 + c);
    if (pre_log) v = mul4(v, aux[r]);
    tile[vrow<C>(r) * V + c] = v;
  }
  __syncthreads();
  for (int x = tid + 1; x < n; x += nt) {
    int lh = 31 - __clz(x);
    uint32_t pos = (uint32_t)(x - (1 << lh));
    aux[x] = root_pow(pos << (24 - 1 - lh));  // w_{2^(lh+1)}^pos
  }
  __syncthreads();
  // S % 3 stages first (large block strides), then radix-8 steps; the last
  // step has block stride 1
  const int rows_log = S + lg;
  int lh = S - 1;
  if (S % 3 == 1) { dif_run_v<C, 1>(tile, aux, rows_log, lh); lh -= 1; }
  else if (S % 3 == 2) { dif_run_v<C, 2>(tile, aux, rows_log, lh); lh -= 2; }
  while (lh >= 2) {
    dif_run_v<C, 3>(tile, aux, rows_log, lh);
    lh -= 3;
  }
  if (tw_log) {
    const uint32_t m = (1u << tw_log) - 1u;
    for (int r = tid; r < rows; r += nt) {
      uint32_t o = o0 + (uint32_t)(r >> S), k = brev((uint32_t)(r & (n - 1)), S);
      aux[r] = root_pow(((o * k) & m) << (24 - tw_log));
    }
    __syncthreads();
  }
  for (int e = tid; e < rows * V; e += nt) {
    int r = e >> LV, c = e & (V - 1);
    uint4 v = tile[vrow<C>(r) * V + c];
    uint32_t o = o0 + (uint32_t)(r >> S);
    uint32_t k = brev((uint32_t)(r & (n - 1)), S);
    if (tw_log) v = mul4(v, aux[r]);
    out4[(o * a_out + k * b_out) * wv + v0 + c] = v;
  }
}

// ---- vectorised tile with the first and last radix steps on global memory ----
// The same transform as dft_tile_v, but the first radix step reads its rows
// straight from global memory (zero padding and the coset pre-twiddle on the
// fly) and the last step writes its rows straight to their bit-reversed
// output rows (four-step post-twiddle on the fly): two shared-memory passes
// and two barriers fewer per tile.  Needs S >= 4 (at least two steps).
template <int C, int R, class TW>
__device__ __forceinline__ void dif_first_v(uint4 *tile, const TW &tw, int rows_log, int S,
                                            const uint4 *__restrict__ in4, uint32_t o0,
                                            uint32_t wv, uint32_t v0, uint32_t rows_valid,
                                            uint32_t a_in, uint32_t b_in, int pre_log,
                                            const TileIdx &ix) {
  constexpr int T = 1 << R, V = C / 4, LV = V == 2 ? 1 : 0;
  const int lh = S - 1, lq = lh - (R - 1);
  const int q = 1 << lq, H = 1 << lh, n = 1 << S;
  const uint32_t pmask = (1u << pre_log) - 1u;
  const int tasks = (1 << (rows_log - R)) << LV;
  for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
    const int c = task & (V - 1), rest = task >> LV;
    const int j = rest & (q - 1), blk = rest >> lq;
    const int base = blk * 2 * H + j;
    uint4 v[T];
    // the task's rows lie in one sub-transform (T q = 2^S rows), so their
    // coset pre-twiddles w^(o' i) with i = i0 + t q form a geometric
    // sequence: two table lookups, then one product per row
    uint32_t ptw = 0, pstep = 0;
    if (pre_log) {
      const uint32_t o = o0 + (uint32_t)(base >> S), i0 = (uint32_t)(base & (n - 1));
      const uint32_t oo = o >> ix.pre_shift;
      ptw = root_pow(((oo * i0) & pmask) << (24 - pre_log));
      pstep = root_pow(((oo * (uint32_t)q) & pmask) << (24 - pre_log));
    }
#pragma unroll
    for (int t = 0; t < T; t++) {
      const int r = base + t * q;
      const uint32_t o = o0 + (uint32_t)(r >> S), i = (uint32_t)(r & (n - 1));
      const uint32_t row = (o & ix.in_mask) * a_in + i * b_in;
      v[t] = make_uint4(0, 0, 0, 0);
      if (row < rows_valid) {
        // rows read once bypass the L1 (it keeps the twiddles); coset
        // transforms (pre_log > 0) read every input row once per coset, so
        // theirs stay cached
        if (pre_log) {
          v[t] = __ldg(in4 + row * wv + v0 + c);
          v[t] = mul4(v[t], ptw);
        } else {
          v[t] = __ldcg(in4 + row * wv + v0 + c);
        }
      }
      if (pre_log && t + 1 < T) ptw = kb::mul(ptw, pstep);
    }
#pragma unroll
    for (int st = 0; st < R; st++) {
      const int span = T >> (st + 1);
      const int hh = H >> st;
#pragma unroll
      for (int t = 0; t < T; t++) {
        if (t & span) continue;
        const int tl = t & (span - 1);
        uint4 a = v[t], b = v[t + span];
        v[t] = add4(a, b);
        v[t + span] = tw.submul(a, b, hh + j + tl * q);
      }
    }
#pragma unroll
    for (int t = 0; t < T; t++) tile[vrow<C>(base + t * q) * V + c] = v[t];
  }
}

// the final radix-8 step (block stride 1, first half-size 4), written to the
// output rows
template <int C, class TW>
__device__ __forceinline__ void dif_last_v(const uint4 *tile, const TW &tw, int rows_log,
                                           int S, uint4 *__restrict__ out4, uint32_t o0,
                                           uint32_t wv, uint32_t v0, uint32_t a_out,
                                           uint32_t b_out, int tw_log, const TileIdx &ix) {
  constexpr int R = 3, T = 8, V = C / 4, LV = V == 2 ? 1 : 0;
  const int n = 1 << S;
  const uint32_t tmask = (1u << tw_log) - 1u;
  const int tasks = (1 << (rows_log - R)) << LV;
  // the step's only twiddles (entries 3, 5, 6, 7), loaded once per thread
  uint2 wl[8];
  wl[3] = tw.t[3];
  wl[5] = tw.t[5];
  wl[6] = tw.t[6];
  wl[7] = tw.t[7];
  for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
    const int c = task & (V - 1), blk = task >> LV;
    const int base = blk * T;
    uint4 v[T];
#pragma unroll
    for (int t = 0; t < T; t++) v[t] = tile[vrow<C>(base + t) * V + c];
#pragma unroll
    for (int st = 0; st < R; st++) {
      const int span = T >> (st + 1);
      const int hh = 4 >> st;
#pragma unroll
      for (int t = 0; t < T; t++) {
        if (t & span) continue;
        const int tl = t & (span - 1);
        uint4 a = v[t], b = v[t + span];
        v[t] = add4(a, b);
        if (tl == 0) v[t + span] = sub4(a, b);  // w^0 = 1
        else v[t + span] = TwShoup::submul_w(a, b, wl[hh + tl]);
      }
    }
#pragma unroll
    for (int t = 0; t < T; t++) {
      const int r = base + t;
      const uint32_t o = o0 + (uint32_t)(r >> S);
      const uint32_t k = brev((uint32_t)(r & (n - 1)), S);
      uint4 x = v[t];
      if (tw_log) {
        const uint32_t e = (o & ix.post_mask) * ((o >> ix.post_shift) + (k << ix.post_kshift));
        x = mul4(x, root_pow((e & tmask) << (24 - tw_log)));
      }
      out4[(o * a_out + k * b_out) * wv + v0 + c] = x;
    }
  }
}

// MINB: CTAs per SM the registers must allow; tiles of more than 48 KB fit
// three per SM by shared memory, so they take up to 80 registers a thread
template <int C, int MINB>
__global__ void __launch_bounds__(256, MINB) dft_tile_v2(const uint32_t *__restrict__ in,
                                                   uint32_t *__restrict__ out, int S, int lg,
                                                   uint32_t width, uint32_t rows_valid,
                                                   uint32_t a_in, uint32_t b_in, uint32_t a_out,
                                                   uint32_t b_out, int pre_log, int tw_log,
                                                   const TileIdx ix) {
  pdl_wait();
  constexpr int V = C / 4;
  extern __shared__ uint4 smv[];
  uint4 *tile = smv;
  const TwShoup aux{g_dif2};  // DIF twiddles (global, read through the L1)
  const uint32_t o0 = blockIdx.y << lg;
  const uint32_t v0 = blockIdx.x * V;
  const uint32_t wv = width / 4;
  const uint4 *in4 = reinterpret_cast<const uint4 *>(in);
  uint4 *out4 = reinterpret_cast<uint4 *>(out);
  const int rows_log = S + lg;
  const int r0 = S % 3 == 0 ? 3 : S % 3;
  if (r0 == 1)
    dif_first_v<C, 1>(tile, aux, rows_log, S, in4, o0, wv, v0, rows_valid, a_in, b_in, pre_log,
                         ix);
  else if (r0 == 2)
    dif_first_v<C, 2>(tile, aux, rows_log, S, in4, o0, wv, v0, rows_valid, a_in, b_in, pre_log,
                         ix);
  else
    dif_first_v<C, 3>(tile, aux, rows_log, S, in4, o0, wv, v0, rows_valid, a_in, b_in, pre_log,
                         ix);
  __syncthreads();
  for (int lh = S - 1 - r0; lh >= 5; lh -= 3) {
    dif_step_v<C, 3, false>(tile, aux, rows_log, lh);
    __syncthreads();
  }
  dif_last_v<C>(tile, aux, rows_log, S, out4, o0, wv, v0, a_out, b_out, tw_log, ix);
}

template <int C>
static cudaError_t launch_tile_v(const uint32_t *in, uint32_t *out, int S, size_t width,
                                 size_t rows_valid, size_t n_outer, size_t a_in, size_t b_in,
                                 size_t a_out, size_t b_out, int pre_log, int tw_log,
                                 cudaStream_t st, const TileIdx &ix = TileIdx()) {
  // pack small sub-transforms so that a CTA holds at least 2^10 rows
  int lg = 0;
  while (S + lg < 10 && ((size_t)2 << lg) <= n_outer) lg++;
  size_t rows = (size_t)1 << (S + lg);
  size_t smem = (rows * C + rows) * 4;
  int threads = (int)(rows * (C / 4) / 8);
  threads = threads < 32 ? 32 : (threads > 256 ? 256 : threads);
  dim3 grid((unsigned)(width / C), (unsigned)(n_outer >> lg));
  if (S >= 4 && rows * C * 4 > (48u << 10))
    launch(dft_tile_v2<C, 3>, grid, threads, rows * C * 4, st, in, out, S, lg, (uint32_t)width,
           (uint32_t)rows_valid, (uint32_t)a_in, (uint32_t)b_in, (uint32_t)a_out,
           (uint32_t)b_out, pre_log, tw_log, ix);
  else if (S >= 4)
    launch(dft_tile_v2<C, 4>, grid, threads, rows * C * 4, st, in, out, S, lg, (uint32_t)width,
           (uint32_t)rows_valid, (uint32_t)a_in, (uint32_t)b_in, (uint32_t)a_out,
           (uint32_t)b_out, pre_log, tw_log, ix);
  else
    launch(dft_tile_v<C>, grid, threads, smem, st, in, out, S, lg, (uint32_t)width,
           (uint32_t)rows_valid, (uint32_t)a_in, (uint32_t)b_in, (uint32_t)a_out,
           (uint32_t)b_out, pre_log, tw_log);
  count_launches(1);
  return cudaGetLastError();
}

template <int C>
static cudaError_t launch_tile(const uint32_t *in, uint32_t *out, int S, size_t width,
                               size_t rows_valid, size_t n_outer, size_t a_in, size_t b_in,
                               size_t a_out, size_t b_out, int pre_log, int tw_log,
                               cudaStream_t st) {
  // pack small sub-transforms so that a CTA holds at least 2^11 rows
  int lg = 0;
  while (S + lg < 11 && ((size_t)2 << lg) <= n_outer) lg++;
  size_t rows = (size_t)1 << (S + lg);
  size_t smem = (rows * C + rows) * 4;  // tile + aux (rows >= 2^S)
  int threads = (int)(rows * C / 8);
  threads = threads < 32 ? 32 : (threads > 256 ? 256 : threads);
  dim3 grid((unsigned)(width / C), (unsigned)(n_outer >> lg));
  launch(dft_tile<C>, grid, threads, smem, st, in, out, S, lg, (uint32_t)width,
         (uint32_t)rows_valid, (uint32_t)a_in, (uint32_t)b_in, (uint32_t)a_out, (uint32_t)b_out,
         pre_log, tw_log);
  count_launches(1);
  return cudaGetLastError();
}

static cudaError_t tile_any(const uint32_t *in, uint32_t *out, int S, size_t width,
                            size_t rows_valid, size_t n_outer, size_t a_in, size_t b_in,
                            size_t a_out, size_t b_out, int pre_log, int tw_log, cudaStream_t st) {
  const bool aligned = (((uintptr_t)in | (uintptr_t)out) & 15) == 0;
  if (aligned && width % 8 == 0)
    return launch_tile_v<8>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                            pre_log, tw_log, st);
  if (aligned && width % 4 == 0)
    return launch_tile_v<4>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                            pre_log, tw_log, st);
  if (width % 8 == 0)
    return launch_tile<8>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                          pre_log, tw_log, st);
  if (width % 4 == 0)
    return launch_tile<4>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                          pre_log, tw_log, st);
  if (width % 2 == 0)
    return launch_tile<2>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                          pre_log, tw_log, st);
  return launch_tile<1>(in, out, S, width, rows_valid, n_outer, a_in, b_in, a_out, b_out,
                        pre_log, tw_log, st);
}

static int ceil_log2(size_t x) {
  int l = 0;
  while (((size_t)1 << l) < x) l++;
  return l;
}
bool dft_coset_one_pass(int log_h, size_t h_in, size_t width) {
  if (log_h <= 11) return false;
  const int L0 = ceil_log2(h_in);
  return log_h - L0 <= 15 && (L0 <= 11 || (L0 == 12 && width % 4 == 0));
}

// per-size overrides of the two-pass split (0: default), by log_h and width class
static std::atomic<int> g_dft_tune[25][2];
static int width_class(size_t width) { return width > 16 ? 1 : 0; }
DftTune dft_tune(int log_h, size_t width) {
  DftTune t;
  if (log_h < 0 || log_h > 24) return t;
  int v = g_dft_tune[log_h][width_class(width)].load(std::memory_order_relaxed);
  if (v) t.l1_bias = v - 8;
  return t;
}
bool dft_tune_valid(int log_h, DftTune t) {
  int L1 = (log_h + 1) / 2 + t.l1_bias, L2 = log_h - L1;
  return t.l1_bias >= -2 && t.l1_bias <= 2 && L1 >= 4 && L2 >= 4 && L1 <= 11 && L2 <= 11;
}
void set_dft_tune(int log_h, size_t width, DftTune t) {
  if (log_h < 0 || log_h > 24 || !dft_tune_valid(log_h, t)) return;
  g_dft_tune[log_h][width_class(width)].store(t.l1_bias + 8, std::memory_order_relaxed);
}

cudaError_t dft_batch(const uint32_t *in, size_t h_in, size_t width, int log_h, uint32_t *out,
                      uint32_t *scratch, cudaStream_t st) {
  if (log_h < 0 || log_h > 24 || width == 0) return cudaErrorInvalidValue;
  size_t h = (size_t)1 << log_h;
  if (h_in > h) return cudaErrorInvalidValue;
  // the kernel indexes words with 32-bit arithmetic
  if (width >= (1u << 16) || (h * width) >= ((size_t)1 << 32)) return cudaErrorInvalidValue;
  if (log_h <= 11)
    return tile_any(in, out, log_h, width, h_in, 1, 0, 1, 0, 1, 0, 0, st);
  const int L0 = ceil_log2(h_in);
  if (L0 <= 11 && log_h - L0 <= 15) {
    // coset form: with N0 = 2^L0 >= h_in and M1 = 2^(log_h - L0),
    // out[k1 + M1 k2] = sum_{n < N0} (x[n] w^(n k1)) w_{N0}^(n k2): M1 transforms
    // of size N0 of the pre-twiddled input, one pass, no scratch
    size_t M1 = h >> L0;
    return tile_any(in, out, L0, width, h_in, M1, 0, 1, 1, M1, log_h, 0, st);
  }
  if (L0 == 12 && log_h - L0 <= 15 && width % 4 == 0 &&
      (((uintptr_t)in | (uintptr_t)out) & 15) == 0) {
    // the same coset form on 2^12-row tiles of 4 columns (64 KB of shared
    // memory, three CTAs per SM; 8 columns would leave one)
    size_t M1 = h >> L0;
    return launch_tile_v<4>(in, out, L0, width, h_in, M1, 0, 1, 1, M1, log_h, 0, st);
  }
  DftTune tune = dft_tune(log_h, width);
  if (!dft_tune_valid(log_h, tune)) tune = DftTune();
  int L1 = (log_h + 1) / 2 + tune.l1_bias, L2 = log_h - L1;
  if (L1 > MAX_TILE_LOG || L2 > MAX_TILE_LOG) return cudaErrorInvalidValue;
  size_t M1 = (size_t)1 << L1, M2 = (size_t)1 << L2;
  cudaError_t e;
  // Pass 1 of a zero-padded input: column n2 has nonzero entries only at
  // n1 < N' = 2^S' with S' = L0 - L2, so with k = k1 + rho k2 (rho = M1 / N')
  // its size-M1 DFT is rho DFTs of size N' of x[M2 n1 + n2] w_{M1}^(n1 k1),
  // the zero butterfly stages skipped.  Sub-transform o = n2 + M2 k1 reads
  // rows (o & (M2-1)) + M2 n1, writes row o + M2 rho k2 = n2 + M2 k, and
  // applies the four-step twiddle w_M^(n2 k).  Used from rho = 8 up: at
  // rho = 4 the pre-twiddle costs about what the two skipped stages save
  // (measured on GB300).
  const int lr = log_h - L0, S1 = L1 - lr;
  const bool aligned = (((uintptr_t)in | (uintptr_t)scratch) & 15) == 0;
  if (lr >= 3 && S1 >= 4 && aligned && width % 4 == 0) {
    TileIdx ix;
    ix.in_mask = (uint32_t)(M2 - 1);
    ix.pre_shift = L2;
    ix.post_mask = (uint32_t)(M2 - 1);
    ix.post_shift = L2;
    ix.post_kshift = lr;
    const size_t n_outer = M2 << lr;
    if (width % 8 == 0)
      e = launch_tile_v<8>(in, scratch, S1, width, h_in, n_outer, 1, M2, 1, n_outer, L1, log_h,
                           st, ix);
    else
      e = launch_tile_v<4>(in, scratch, S1, width, h_in, n_outer, 1, M2, 1, n_outer, L1, log_h,
                           st, ix);
  } else {
    e = tile_any(in, scratch, L1, width, h_in, M2, 1, M2, 1, M2, 0, log_h, st);
  }
  if (e != cudaSuccess) return e;
  return tile_any(scratch, out, L2, width, h, M1, M2, 1, 1, M1, 0, 0, st);
}

static size_t tile_smem_max(int C) { return ((size_t)(1 << MAX_TILE_LOG) * C + (1 << MAX_TILE_LOG)) * 4; }

// Once per process and device; contexts on several host threads may call it.
cudaError_t init_device_tables() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return cudaSuccess;
  e = upload_device_tables();
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(8));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(4));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(2));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(1));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile_v<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(8));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile_v<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(4));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile_v2<8, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(8));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile_v2<4, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(4));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile_v2<8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(8));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(dft_tile_v2<4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem_max(4));
  if (e == cudaSuccess) done[dev] = true;
  return e;
}

}  // namespace gpu
}  // namespace whir
