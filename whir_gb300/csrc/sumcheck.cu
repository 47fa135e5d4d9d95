// eq tables, SVO compression, expression build, constraint combination and
// sumcheck round kernels (crates/poly/src/{point,eq,poly}.rs,
// crates/whir/src/sumcheck/{svo,expr,combine,prover}.rs).
//
// Reductions are exact: every thread sums canonical words mod p, then CTA
// partials are added as plain integers into 64-bit accumulators with
// atomicAdd (the sum of canonical words stays far below 2^64), and the host
// reduces the accumulator mod p.  Any summation order therefore gives the
// same field element, which is why the results match the CPU restatement
// bit for bit.
#include "kernels.h"
#include "launch.cuh"

namespace whir {
namespace gpu {

using kb::E4;

__device__ __forceinline__ void acc_add(unsigned long long *a, const E4 &v) {
#pragma unroll
  for (int c = 0; c < 4; c++) atomicAdd(a + c, (unsigned long long)v.c[c]);
}

// Extension elements through 16-byte accesses when the arrays are 16-byte
// aligned (VEC; E4 itself only promises 4), word by word otherwise.
template <bool VEC>
__device__ __forceinline__ E4 ld_e4(const E4 *p) {
  if constexpr (VEC) {
    const uint4 v = *reinterpret_cast<const uint4 *>(p);
    return E4{{v.x, v.y, v.z, v.w}};
  } else {
    return *p;
  }
}
template <bool VEC>
__device__ __forceinline__ void st_e4(E4 *p, const E4 &a) {
  if constexpr (VEC) *reinterpret_cast<uint4 *>(p) = make_uint4(a.c[0], a.c[1], a.c[2], a.c[3]);
  else *p = a;
}
__host__ __forceinline__ bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }


// Publish (kernels.h): after this CTA's atomics into acc, the last CTA of
// the launch copies the sums out and zeroes them.  Every thread of the CTA
// calls it.  acc is the accumulator base of the whole launch (every instance
// of a batched launch, blockIdx.y, publishes from the same base).
__device__ __forceinline__ void publish_if_last(unsigned long long *acc, const Publish &pub) {
  if (!pub.host) return;
  const unsigned ncta = gridDim.x * gridDim.y;
  if (ncta == 1) {
    // the only CTA is the last: its atomics on acc precede the exchanges
    // below in the same memory location's order, no ticket or fence needed
    __syncthreads();
  } else {
    __shared__ bool last;
    __threadfence();  // this CTA's atomics are visible before its ticket
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(pub.counter, 1u) == ncta - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
  }
  for (int i = threadIdx.x; i < pub.words; i += blockDim.x) pub.host[i] = atomicExch(acc + i, 0ull);
  if (threadIdx.x == 0 && ncta > 1) atomicExch(pub.counter, 0u);
  if (pub.flag) {
    __threadfence_system();  // the results reach host memory before the flag
    __syncthreads();
    if (threadIdx.x == 0) *reinterpret_cast<volatile unsigned int *>(pub.flag) = pub.seq;
  }
}

// eq table entries over z[off .. off+nv) times scale: entry b selects z_i
// when bit i of b is set, 1 - z_i otherwise (Point::eq, point.rs:110-126).
__global__ void eq_entries(Point z, int off, int nv, E4 scale, E4 *out) {
  pdl_wait();
  size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= ((size_t)1 << nv)) return;
  E4 acc = scale;
  for (int i = 0; i < nv; i++) {
    E4 zi = z.z[off + i];
    acc = kb::e_mul(acc, ((b >> i) & 1) ? zi : kb::e_sub(kb::e_one(), zi));
  }
  out[b] = acc;
}

// n_tables split eq tables in one launch: table t = (lo: 2^s entries over
// pts[t][0..s), hi: 2^(k-s) entries over pts[t][s..k) times scales[t]),
// stored back to back as add_eq expects.
__global__ void eq_tables_kernel(const E4 *__restrict__ pts, const E4 *__restrict__ scales, int k,
                                 int s, E4 *__restrict__ out) {
  pdl_wait();
  const int t = blockIdx.y;
  const size_t nlo = (size_t)1 << s, per = nlo + ((size_t)1 << (k - s));
  size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= per) return;
  const E4 *z = pts + (size_t)t * k;
  E4 acc;
  int off, nv;
  size_t b;
  if (x < nlo) {
    acc = kb::e_one(); off = 0; nv = s; b = x;
  } else {
    acc = scales[t]; off = s; nv = k - s; b = x - nlo;
  }
  for (int i = 0; i < nv; i++) {
    E4 zi = z[off + i];
    acc = kb::e_mul(acc, ((b >> i) & 1) ? zi : kb::e_sub(kb::e_one(), zi));
  }
  out[(size_t)t * per + x] = acc;
}

cudaError_t eq_tables(const E4 *pts, const E4 *scales, int n, int k, int s, E4 *out,
                      cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (s < 0 || s > k || n > 65535) return cudaErrorInvalidValue;
  size_t per = ((size_t)1 << s) + ((size_t)1 << (k - s));
  dim3 grid((unsigned)((per + 127) / 128), (unsigned)n);
  launch(eq_tables_kernel, grid, 128, 0, st, pts, scales, k, s, out);
  count_launches(1);
  return cudaGetLastError();
}

// the same tables with the points passed by value in the kernel parameters
// (no upload on the stream)
__global__ void eq_tables_val_kernel(const __grid_constant__ EqArgs a, int k, int s,
                                     E4 *__restrict__ out) {
  pdl_wait();
  const int t = blockIdx.y;
  const size_t nlo = (size_t)1 << s, per = nlo + ((size_t)1 << (k - s));
  size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= per) return;
  const E4 *z = a.z + t * EqArgs::K;
  E4 acc;
  int off, nv;
  size_t b;
  if (x < nlo) {
    acc = kb::e_one(); off = 0; nv = s; b = x;
  } else {
    acc = a.scale[t]; off = s; nv = k - s; b = x - nlo;
  }
  for (int i = 0; i < nv; i++) {
    E4 zi = z[off + i];
    acc = kb::e_mul(acc, ((b >> i) & 1) ? zi : kb::e_sub(kb::e_one(), zi));
  }
  out[(size_t)t * per + x] = acc;
}

cudaError_t eq_tables_val(const EqArgs &a, int n, int k, int s, E4 *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (n > EqArgs::N || k > EqArgs::K || s < 0 || s > k) return cudaErrorInvalidValue;
  size_t per = ((size_t)1 << s) + ((size_t)1 << (k - s));
  dim3 grid((unsigned)((per + 127) / 128), (unsigned)n);
  launch(eq_tables_val_kernel, grid, 128, 0, st, a, k, s, out);
  count_launches(1);
  return cudaGetLastError();
}

static cudaError_t eq_part(const Point &z, int off, int nv, E4 scale, E4 *out, cudaStream_t st) {
  size_t n = (size_t)1 << nv;
  unsigned T = 256, G = (unsigned)((n + T - 1) / T);
  launch(eq_entries, G, T, 0, st, z, off, nv, scale, out);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t eq_split(const Point &z, int s, E4 scale, E4 *lo, E4 *hi, cudaStream_t st) {
  if (s < 0 || s > z.k) return cudaErrorInvalidValue;
  cudaError_t e = eq_part(z, 0, s, kb::e_one(), lo, st);
  if (e != cudaSuccess) return e;
  return eq_part(z, s, z.k - s, scale, hi, st);
}

__global__ void eq_join(const E4 *lo, const E4 *hi, int s, size_t n, E4 *out) {
  pdl_wait();
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = kb::e_mul(lo[i & (((size_t)1 << s) - 1)], hi[i >> s]);
}

cudaError_t eq_full(const Point &z, E4 scale, E4 *out, E4 *tmp, cudaStream_t st) {
  int s = z.k / 2;
  E4 *lo = tmp, *hi = tmp + ((size_t)1 << s);
  cudaError_t e = eq_split(z, s, scale, lo, hi, st);
  if (e != cudaSuccess) return e;
  size_t n = (size_t)1 << z.k;
  launch(eq_join, (unsigned)((n + 255) / 256), 256, 0, st, lo, hi, s, n, out);
  count_launches(1);
  return cudaGetLastError();
}

// compress_hi: rows of W = 2^ks words; row h = h_lo + 2^s_lo * h_hi.  A CTA
// walks whole h_hi blocks (2^s_lo contiguous rows); thread t always sees
// column j = t mod W, so it keeps one inner sum (over h_lo, weighted by
// eq_lo) and folds it into its outer sum with eq_hi[h_hi] once per block.
// Four CTAs per SM, each walking several blocks, so that the fixed cost of a
// CTA (the eq_lo copy, the reduction of its sums) is paid a few hundred
// times per launch, not once per block.
constexpr int CH_T = 256;
__device__ __forceinline__ void ch_accumulate4(E4 &inner, const E4 *lo, int ks, size_t e,
                                               const uint32_t (&x)[4]) {
  // four products of canonical words per 64-bit sum (4 p^2 < 2p 2^32), one
  // Montgomery reduction per four: the sum of Montgomery words' products
  // reduces to the Montgomery word of the sum of products
  unsigned long long s4[4] = {0, 0, 0, 0};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const E4 l = lo[(e + q * CH_T) >> ks];
#pragma unroll
    for (int c = 0; c < 4; c++) s4[c] += (unsigned long long)l.c[c] * x[q];
  }
  E4 part4;
#pragma unroll
  for (int c = 0; c < 4; c++) part4.c[c] = kb::reduce_wide(s4[c]);
  inner = kb::e_add(inner, part4);
}
__global__ void __launch_bounds__(CH_T, 4) compress_hi_kernel(const uint32_t *__restrict__ poly,
                                                              int k, int ks,
                                                              const E4 *__restrict__ eq_lo,
                                                              int s_lo,
                                                              const E4 *__restrict__ eq_hi,
                                                              unsigned long long *acc,
                                                              Publish pub, HiStrides sd) {
  pdl_wait();
  extern __shared__ unsigned char smraw[];
  poly += blockIdx.y * sd.poly;
  eq_lo += blockIdx.y * sd.tab;
  eq_hi += blockIdx.y * sd.tab;
  unsigned long long *const acc_y = acc + blockIdx.y * sd.acc;
  E4 *lo = reinterpret_cast<E4 *>(smraw);
  unsigned long long *part = reinterpret_cast<unsigned long long *>(lo + ((size_t)1 << s_lo));
  const int W = 1 << ks;
  const int tid = threadIdx.x;
  for (int i = tid; i < (1 << s_lo); i += CH_T) lo[i] = eq_lo[i];
  for (int i = tid; i < W * 4; i += CH_T) part[i] = 0;
  __syncthreads();
  const size_t block_words = (size_t)W << s_lo;
  const size_t n_hi = (size_t)1 << (k - ks - s_lo);
  E4 outer = kb::e_zero();
  for (size_t hh = blockIdx.x; hh < n_hi; hh += gridDim.x) {
    const uint32_t *base = poly + hh * block_words;
    E4 inner = kb::e_zero();
    size_t e = tid;
    // sixteen streaming loads in flight per thread
    for (; e + 15 * CH_T < block_words; e += 16 * CH_T) {
      uint32_t x[4][4];
#pragma unroll
      for (int g = 0; g < 4; g++)
#pragma unroll
        for (int q = 0; q < 4; q++) x[g][q] = __ldcs(base + e + (4 * g + q) * CH_T);
#pragma unroll
      for (int g = 0; g < 4; g++) ch_accumulate4(inner, lo, ks, e + 4 * g * CH_T, x[g]);
    }
    for (; e + 3 * CH_T < block_words; e += 4 * CH_T) {
      uint32_t x[4];
#pragma unroll
      for (int q = 0; q < 4; q++) x[q] = __ldcs(base + e + q * CH_T);
      ch_accumulate4(inner, lo, ks, e, x);
    }
    for (; e < block_words; e += CH_T)
      inner = kb::e_add(inner, kb::e_scale(lo[e >> ks], __ldg(base + e)));
    outer = kb::e_add(outer, kb::e_mul(inner, eq_hi[hh]));
  }
  // lanes of a warp that share a column add their sums by shuffles first
  // (modular adds of canonical words), so the shared atomics below see one
  // value per column and warp
  const int lane = tid & 31;
  for (int off = W; off < 32; off <<= 1)
#pragma unroll
    for (int c = 0; c < 4; c++)
      outer.c[c] = kb::add(outer.c[c], __shfl_xor_sync(0xffffffffu, outer.c[c], off));
  if (W >= 32 || lane < W) {
    const int j = tid & (W - 1);
#pragma unroll
    for (int c = 0; c < 4; c++) atomicAdd(part + j * 4 + c, (unsigned long long)outer.c[c]);
  }
  __syncthreads();
  for (int i = tid; i < W * 4; i += CH_T) atomicAdd(acc_y + i, part[i]);
  publish_if_last(acc, pub);
}

// The same pass when a block is exactly 16 words per thread (W 2^s_lo =
// 16 CH_T, the SVO shape): the next block's words and eq_hi entry are
// loaded before this block's products (two blocks in registers, three CTAs
// per SM), and the 64-bit sums fold every three products (2^32 = 2^32 - 2p
// mod p keeps them below 2^58) with one reduction per block.
constexpr uint32_t CH_FOLD = (uint32_t)((1ull << 32) % kb::P);
__device__ __forceinline__ unsigned long long ch_fold(unsigned long long x) {
  return (unsigned long long)(uint32_t)(x >> 32) * CH_FOLD + (uint32_t)x;  // < 2^57 + 2^32
}
__global__ void __launch_bounds__(CH_T, 3) compress_hi_pipe_kernel(
    const uint32_t *__restrict__ poly, int k, int ks, const E4 *__restrict__ eq_lo, int s_lo,
    const E4 *__restrict__ eq_hi, unsigned long long *acc, Publish pub, HiStrides sd) {
  pdl_wait();
  extern __shared__ unsigned char smraw[];
  poly += blockIdx.y * sd.poly;
  eq_lo += blockIdx.y * sd.tab;
  eq_hi += blockIdx.y * sd.tab;
  unsigned long long *const acc_y = acc + blockIdx.y * sd.acc;
  E4 *lo = reinterpret_cast<E4 *>(smraw);
  unsigned long long *part = reinterpret_cast<unsigned long long *>(lo + ((size_t)1 << s_lo));
  const int W = 1 << ks;
  const int tid = threadIdx.x;
  for (int i = tid; i < (1 << s_lo); i += CH_T) lo[i] = eq_lo[i];
  for (int i = tid; i < W * 4; i += CH_T) part[i] = 0;
  __syncthreads();
  const uint32_t step_rows = CH_T >> ks;
  const size_t n_hi = (size_t)1 << (k - ks - s_lo);
  const E4 *lrow = lo + (tid >> ks);
  E4 outer = kb::e_zero();
  size_t hh = blockIdx.x;
  uint32_t xa[16];
  E4 ha = kb::e_zero();
  if (hh < n_hi) {
    const uint32_t *b = poly + hh * (size_t)(16 * CH_T) + tid;
#pragma unroll
    for (int q = 0; q < 16; q++) xa[q] = __ldcs(b + q * CH_T);
    ha = eq_hi[hh];
  }
  for (; hh < n_hi; hh += gridDim.x) {
    uint32_t xb[16];
    E4 hb = kb::e_zero();
    const size_t nx = hh + gridDim.x;
    if (nx < n_hi) {
      const uint32_t *b = poly + nx * (size_t)(16 * CH_T) + tid;
#pragma unroll
      for (int q = 0; q < 16; q++) xb[q] = __ldcs(b + q * CH_T);
      hb = eq_hi[nx];
    }
    unsigned long long a4[4] = {0, 0, 0, 0};
#pragma unroll
    for (int q = 0; q < 16; q++) {
      const E4 l = lrow[q * step_rows];
#pragma unroll
      for (int c = 0; c < 4; c++) a4[c] += (unsigned long long)l.c[c] * xa[q];
      if (q % 3 == 2) {
#pragma unroll
        for (int c = 0; c < 4; c++) a4[c] = ch_fold(a4[c]);
      }
    }
    E4 inner;
#pragma unroll
    for (int c = 0; c < 4; c++) inner.c[c] = kb::reduce_wide(ch_fold(a4[c]));
    outer = kb::e_add(outer, kb::e_mul(inner, ha));
#pragma unroll
    for (int q = 0; q < 16; q++) xa[q] = xb[q];
    ha = hb;
  }
  const int lane = tid & 31;
  for (int off = W; off < 32; off <<= 1)
#pragma unroll
    for (int c = 0; c < 4; c++)
      outer.c[c] = kb::add(outer.c[c], __shfl_xor_sync(0xffffffffu, outer.c[c], off));
  if (W >= 32 || lane < W) {
    const int j = tid & (W - 1);
#pragma unroll
    for (int c = 0; c < 4; c++) atomicAdd(part + j * 4 + c, (unsigned long long)outer.c[c]);
  }
  __syncthreads();
  for (int i = tid; i < W * 4; i += CH_T) atomicAdd(acc_y + i, part[i]);
  publish_if_last(acc, pub);
}

cudaError_t compress_hi(const uint32_t *poly, int k, int ks, const E4 *eq_lo, int s_lo,
                        const E4 *eq_hi, unsigned long long *acc, cudaStream_t st,
                        const Publish &pub) {
  return compress_hi_batch(poly, k, ks, eq_lo, s_lo, eq_hi, acc, 1, HiStrides(), st, pub);
}

cudaError_t compress_hi_batch(const uint32_t *poly, int k, int ks, const E4 *eq_lo, int s_lo,
                              const E4 *eq_hi, unsigned long long *acc, int batch,
                              const HiStrides &sd, cudaStream_t st, const Publish &pub) {
  if ((1 << ks) > CH_T || k < ks + s_lo || batch < 1 || batch > 65535)
    return cudaErrorInvalidValue;
  size_t n_hi = (size_t)1 << (k - ks - s_lo);
  // about four (three) CTAs per SM over all instances
  const size_t per4 = ((size_t)152 * 4 + batch - 1) / batch, per3 = ((size_t)152 * 3 + batch - 1) / batch;
  dim3 grid((unsigned)(n_hi < per4 ? n_hi : per4), (unsigned)batch);
  size_t smem = ((size_t)1 << s_lo) * sizeof(E4) + ((size_t)4 << ks) * 8;
  if (((size_t)1 << (ks + s_lo)) == 16 * (size_t)CH_T) {
    grid.x = (unsigned)(n_hi < per3 ? n_hi : per3);
    launch(compress_hi_pipe_kernel, grid, CH_T, smem, st, poly, k, ks, eq_lo, s_lo, eq_hi, acc,
           pub, sd);
  } else {
    launch(compress_hi_kernel, grid, CH_T, smem, st, poly, k, ks, eq_lo, s_lo, eq_hi, acc, pub, sd);
  }
  count_launches(1);
  return cudaGetLastError();
}

// compress_lo: out[i] = sum_j eq(rs)[j] * P[i * 2^ks + j].  Batched:
// instance y = blockIdx.y reads poly + y poly_stride with its own rs
// (rs_b[y ks ..], ks extension elements) and writes out + y n_out.
template <bool VEC>
__global__ void compress_lo_kernel(const uint32_t *__restrict__ poly, int ks, size_t n_out,
                                   Point rs, const E4 *__restrict__ rs_b, size_t poly_stride,
                                   E4 *__restrict__ out) {
  pdl_wait();
  __shared__ E4 eq[256];
  const int W = 1 << ks;
  poly += blockIdx.y * poly_stride;
  out += blockIdx.y * n_out;
  for (int b = threadIdx.x; b < W; b += blockDim.x) {
    E4 acc = kb::e_one();
    for (int i = 0; i < ks; i++) {
      const E4 zi = rs_b ? rs_b[(size_t)blockIdx.y * ks + i] : rs.z[i];
      acc = kb::e_mul(acc, ((b >> i) & 1) ? zi : kb::e_sub(kb::e_one(), zi));
    }
    eq[b] = acc;
  }
  __syncthreads();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_out;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t *row = poly + i * W;
    E4 acc = kb::e_zero();
    if (VEC) {  // rows of a multiple of 4 words, 16-byte aligned
      for (int j = 0; j < W; j += 4) {
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(row + j));
        acc = kb::e_add(acc, kb::e_scale(eq[j], v.x));
        acc = kb::e_add(acc, kb::e_scale(eq[j + 1], v.y));
        acc = kb::e_add(acc, kb::e_scale(eq[j + 2], v.z));
        acc = kb::e_add(acc, kb::e_scale(eq[j + 3], v.w));
      }
    } else {
      for (int j = 0; j < W; j++) acc = kb::e_add(acc, kb::e_scale(eq[j], __ldg(row + j)));
    }
    st_e4<VEC>(out + i, acc);
  }
}

static cudaError_t compress_lo_launch(const uint32_t *poly, int k, int ks, const Point &rs,
                                      const E4 *rs_b, int batch, size_t poly_stride, E4 *out,
                                      cudaStream_t st) {
  if (ks > 8 || ks > k || batch < 1 || batch > 65535) return cudaErrorInvalidValue;
  size_t n_out = (size_t)1 << (k - ks);
  unsigned T = 256;
  size_t g = (n_out + T - 1) / T, cap = ((size_t)152 * 16 + batch - 1) / batch;
  dim3 grid((unsigned)(g < cap ? g : cap), (unsigned)batch);
  const bool vec = ks >= 2 && aligned16(poly) && aligned16(out) &&
                   (batch == 1 || poly_stride % 4 == 0);
  if (vec)
    launch(compress_lo_kernel<true>, grid, T, 0, st, poly, ks, n_out, rs, rs_b, poly_stride, out);
  else
    launch(compress_lo_kernel<false>, grid, T, 0, st, poly, ks, n_out, rs, rs_b, poly_stride, out);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t compress_lo(const uint32_t *poly, int k, const Point &rs, E4 *out, cudaStream_t st) {
  return compress_lo_launch(poly, k, rs.k, rs, nullptr, 1, 0, out, st);
}

cudaError_t compress_lo_batch(const uint32_t *poly, int k, int ks, const E4 *rs_b, int batch,
                              size_t poly_stride, E4 *out, cudaStream_t st) {
  Point none;
  none.k = ks;
  return compress_lo_launch(poly, k, ks, none, rs_b, batch, poly_stride, out, st);
}

// w[i] += sum_t lo_t[i & mask] * hi_t[i >> s].  Batched: instance y =
// blockIdx.y adds its n_tables tables (stored after those of instances < y)
// into w + y n.
template <bool VEC>
__global__ void add_eq_kernel(E4 *w, size_t n, int s, size_t n_lo, size_t n_hi,
                              const E4 *__restrict__ tables, int n_tables) {
  pdl_wait();
  w += blockIdx.y * n;
  tables += blockIdx.y * (size_t)n_tables * (n_lo + n_hi);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    E4 acc = ld_e4<VEC>(w + i);
    for (int t = 0; t < n_tables; t++) {
      const E4 *lo = tables + t * (n_lo + n_hi), *hi = lo + n_lo;
      acc = kb::e_add(acc, kb::e_mul(ld_e4<VEC>(lo + (i & (n_lo - 1))), ld_e4<VEC>(hi + (i >> s))));
    }
    st_e4<VEC>(w + i, acc);
  }
}

cudaError_t add_eq_batch(E4 *w, int k, const E4 *tables, int n_tables, int batch,
                         cudaStream_t st) {
  if (n_tables == 0) return cudaSuccess;
  if (batch < 1 || batch > 65535) return cudaErrorInvalidValue;
  int s = k / 2;
  size_t n = (size_t)1 << k;
  unsigned T = 256;
  size_t g = (n + T - 1) / T, cap = ((size_t)152 * 16 + batch - 1) / batch;
  dim3 grid((unsigned)(g < cap ? g : cap), (unsigned)batch);
  if (aligned16(w) && aligned16(tables))
    launch(add_eq_kernel<true>, grid, T, 0, st, w, n, s, (size_t)1 << s, (size_t)1 << (k - s),
           tables, n_tables);
  else
    launch(add_eq_kernel<false>, grid, T, 0, st, w, n, s, (size_t)1 << s, (size_t)1 << (k - s),
           tables, n_tables);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t add_eq(E4 *w, int k, const E4 *tables, int n_tables, cudaStream_t st) {
  return add_eq_batch(w, k, tables, n_tables, 1, st);
}

// var_t^i = lo_t[i mod 2^s] * hi_t[i >> s]: per var, 2^s low powers then
// 2^(k-s) powers of var^(2^s), built by one thread per entry.
__global__ void pow_tables_kernel(const uint32_t *__restrict__ vars, int n, int s, int k,
                                  uint32_t *__restrict__ tab) {
  pdl_wait();
  const size_t nlo = (size_t)1 << s, per = nlo + ((size_t)1 << (k - s));
  size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= (size_t)n * per) return;
  size_t t = x / per, j = x % per;
  uint64_t e = j < nlo ? j : (uint64_t)(j - nlo) << s;
  tab[x] = kb::pow(vars[t], e);
}

// w[i] += sum_t scale_t * var_t^i, one thread per i
// w[i] += sum_t scale_t * lo_t[i mod 2^s] * hi_t[i >> s] (per-point power
// tables from pow_tables).  When 2^s >= the CTA size every thread of a CTA
// shares hi_t, so the CTA first forms S_t = scale_t * hi_t in shared memory
// and each thread then adds S_t * lo_t: four 64-bit products per point,
// folded every three points (2^32 = 2^32 - 2p mod p keeps the sum below
// 2^58) and reduced once.  Otherwise every thread forms the products itself.
constexpr int AP_T = 256;
constexpr uint32_t FOLD_2_32 = (uint32_t)((1ull << 32) % kb::P);
__device__ __forceinline__ unsigned long long fold_2_32(unsigned long long x) {
  return (unsigned long long)(uint32_t)(x >> 32) * FOLD_2_32 + (uint32_t)x;  // < 2^57 + 2^32
}
template <bool VEC, class SCALE>
__device__ __forceinline__ void add_pows_body(E4 *__restrict__ w, size_t n_out, int s, int n,
                                              const uint32_t *__restrict__ tab,
                                              const SCALE &scale) {
  extern __shared__ E4 sh[];
  const size_t nlo = (size_t)1 << s, per = nlo + (n_out >> s);
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (nlo >= blockDim.x) {  // one hi index per CTA
    const size_t ih = nlo + (((size_t)blockIdx.x * blockDim.x) >> s);
    for (int t = threadIdx.x; t < n; t += blockDim.x)
      sh[t] = kb::e_scale(scale(t), __ldg(tab + (size_t)t * per + ih));
    __syncthreads();
    if (i >= n_out) return;
    const uint32_t *tb = tab + (i & (nlo - 1));
    unsigned long long a[4] = {0, 0, 0, 0};
    int t = 0;
    for (; t + 2 < n; t += 3) {
      uint32_t x[3];
#pragma unroll
      for (int u = 0; u < 3; u++) x[u] = __ldg(tb + (size_t)(t + u) * per);
#pragma unroll
      for (int u = 0; u < 3; u++) {
        const E4 sc = sh[t + u];
#pragma unroll
        for (int c = 0; c < 4; c++) a[c] += (unsigned long long)sc.c[c] * x[u];
      }
#pragma unroll
      for (int c = 0; c < 4; c++) a[c] = fold_2_32(a[c]);
    }
    for (; t < n; t++) {
      const uint32_t x = __ldg(tb + (size_t)t * per);
      const E4 sc = sh[t];
#pragma unroll
      for (int c = 0; c < 4; c++) a[c] = fold_2_32(a[c] + (unsigned long long)sc.c[c] * x);
    }
    E4 add;
#pragma unroll
    for (int c = 0; c < 4; c++) add.c[c] = kb::reduce_wide(a[c]);
    st_e4<VEC>(w + i, kb::e_add(ld_e4<VEC>(w + i), add));
    return;
  }
  if (i >= n_out) return;
  const size_t il = i & (nlo - 1), ih = nlo + (i >> s);
  E4 acc = ld_e4<VEC>(w + i);
  for (int t = 0; t < n; t++) {
    const uint32_t *tb = tab + (size_t)t * per;
    uint32_t pw = kb::mul(__ldg(tb + il), __ldg(tb + ih));
    acc = kb::e_add(acc, kb::e_scale(scale(t), pw));
  }
  st_e4<VEC>(w + i, acc);
}
struct ScalePtr {
  const E4 *p;
  __device__ __forceinline__ E4 operator()(int t) const { return p[t]; }
};
struct ScaleVal {
  const PowArgs *a;
  __device__ __forceinline__ E4 operator()(int t) const { return a->scales[t]; }
};
template <bool VEC>
__global__ void add_pows_kernel(E4 *__restrict__ w, size_t n_out, int s, int n,
                                const uint32_t *__restrict__ tab, const E4 *__restrict__ scales) {
  pdl_wait();
  add_pows_body<VEC>(w, n_out, s, n, tab, ScalePtr{scales});
}

// the same two passes with the variables and scales passed by value
__global__ void pow_tables_val_kernel(const __grid_constant__ PowArgs a, int n, int s, int k,
                                      uint32_t *__restrict__ tab) {
  pdl_wait();
  const size_t nlo = (size_t)1 << s, per = nlo + ((size_t)1 << (k - s));
  size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= (size_t)n * per) return;
  size_t t = x / per, j = x % per;
  uint64_t e = j < nlo ? j : (uint64_t)(j - nlo) << s;
  tab[x] = kb::pow(a.vars[t], e);
}
template <bool VEC>
__global__ void add_pows_val_kernel(E4 *__restrict__ w, size_t n_out, int s, int n,
                                    const uint32_t *__restrict__ tab,
                                    const __grid_constant__ PowArgs a) {
  pdl_wait();
  add_pows_body<VEC>(w, n_out, s, n, tab, ScaleVal{&a});
}

// shared memory of add_pows_body: the S_t of one CTA (none without them)
static size_t add_pows_smem(int k, int n) {
  int s = k / 2;
  return ((size_t)1 << s) >= (size_t)AP_T ? (size_t)n * sizeof(E4) : 0;
}

cudaError_t add_pows_val(E4 *w, int k, const PowArgs &a, int n, uint32_t *tab, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (n > PowArgs::N || add_pows_smem(k, n) > 48 * 1024) return cudaErrorInvalidValue;
  int s = k / 2;
  size_t words = add_pows_scratch_words(k, n);
  launch(pow_tables_val_kernel, (unsigned)((words + 255) / 256), 256, 0, st, a, n, s, k, tab);
  count_launches(1);
  size_t N = (size_t)1 << k;
  const unsigned g = (unsigned)((N + AP_T - 1) / AP_T);
  if (aligned16(w))
    launch(add_pows_val_kernel<true>, g, AP_T, add_pows_smem(k, n), st, w, N, s, n, tab, a);
  else
    launch(add_pows_val_kernel<false>, g, AP_T, add_pows_smem(k, n), st, w, N, s, n, tab, a);
  count_launches(1);
  return cudaGetLastError();
}

size_t add_pows_scratch_words(int k, int n) {
  int s = k / 2;
  return (size_t)n * (((size_t)1 << s) + ((size_t)1 << (k - s)));
}

cudaError_t add_pows(E4 *w, int k, const uint32_t *vars, const E4 *scales, int n, uint32_t *tab,
                     cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const size_t smem = add_pows_smem(k, n);
  if (smem > 48 * 1024) return cudaErrorInvalidValue;  // more than 3072 points
  int s = k / 2;
  size_t words = add_pows_scratch_words(k, n);
  launch(pow_tables_kernel, (unsigned)((words + 255) / 256), 256, 0, st, vars, n, s, k, tab);
  count_launches(1);
  size_t N = (size_t)1 << k;
  const unsigned g = (unsigned)((N + AP_T - 1) / AP_T);
  if (aligned16(w))
    launch(add_pows_kernel<true>, g, AP_T, smem, st, w, N, s, n, tab, scales);
  else
    launch(add_pows_kernel<false>, g, AP_T, smem, st, w, N, s, n, tab, scales);
  count_launches(1);
  return cudaGetLastError();
}

// Batched and ragged: instance y = blockIdx.y adds the variables
// off[y] .. off[y+1] of the flat arrays (their power tables at the same
// positions of tab) into w + y 2^k.
template <bool VEC>
__global__ void add_pows_batch_kernel(E4 *__restrict__ w, size_t n_out, int s,
                                      const int *__restrict__ off,
                                      const uint32_t *__restrict__ tab,
                                      const E4 *__restrict__ scales) {
  pdl_wait();
  const int y = blockIdx.y, o = off[y], n = off[y + 1] - o;
  const size_t per = ((size_t)1 << s) + (n_out >> s);
  add_pows_body<VEC>(w + (size_t)y * n_out, n_out, s, n, tab + (size_t)o * per,
                     ScalePtr{scales + o});
}

cudaError_t add_pows_batch(E4 *w, int k, const uint32_t *vars, const E4 *scales, const int *off,
                           int n_total, int max_n, int batch, uint32_t *tab, cudaStream_t st) {
  if (n_total == 0) return cudaSuccess;
  const size_t smem = add_pows_smem(k, max_n);
  if (smem > 48 * 1024 || batch < 1 || batch > 65535) return cudaErrorInvalidValue;
  int s = k / 2;
  size_t words = add_pows_scratch_words(k, n_total);
  launch(pow_tables_kernel, (unsigned)((words + 255) / 256), 256, 0, st, vars, n_total, s, k, tab);
  count_launches(1);
  size_t N = (size_t)1 << k;
  dim3 grid((unsigned)((N + AP_T - 1) / AP_T), (unsigned)batch);
  if (aligned16(w))
    launch(add_pows_batch_kernel<true>, grid, AP_T, smem, st, w, N, s, off, tab, scales);
  else
    launch(add_pows_batch_kernel<false>, grid, AP_T, smem, st, w, N, s, off, tab, scales);
  count_launches(1);
  return cudaGetLastError();
}

// block-wide sum of E4 values into 64-bit accumulators at acc; acc_base is
// the launch's accumulator base for publishing (acc itself when unbatched)
template <int NV>
__device__ __forceinline__ void block_acc(const E4 (&v)[NV], unsigned long long *acc,
                                          unsigned long long *acc_base, const Publish &pub) {
  __shared__ unsigned long long part[NV * 4];
  for (int i = threadIdx.x; i < NV * 4; i += blockDim.x) part[i] = 0;
  __syncthreads();
  // warp pre-sum mod p, then one shared atomic per warp and word
#pragma unroll
  for (int q = 0; q < NV; q++)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      uint32_t x = v[q].c[c];
#pragma unroll
      for (int off = 16; off; off >>= 1) x = kb::add(x, __shfl_down_sync(0xffffffffu, x, off));
      if ((threadIdx.x & 31) == 0) atomicAdd(part + q * 4 + c, (unsigned long long)x);
    }
  __syncthreads();
  for (int i = threadIdx.x; i < NV * 4; i += blockDim.x) atomicAdd(acc + i, part[i]);
  publish_if_last(acc_base, pub);
}

// One round: new[i] = a[2i] + r (a[2i+1] - a[2i]) for poly and weights (when
// folding), then c0 += w[2m] p[2m], c2 += (2 w[2m+1] - w[2m]) (2 p[2m+1] - p[2m]).
// Batched: instance y = blockIdx.y has its arrays at y n_in (inputs) and
// y n_in / 2 (outputs), its challenge at r_b[y] and its sums at
// acc + y acc_stride.
template <bool VEC>
__global__ void __launch_bounds__(256) round_kernel(const E4 *__restrict__ p_in,
                                                    const E4 *__restrict__ w_in, size_t n_in,
                                                    int fold, E4 r, E4 *__restrict__ p_out,
                                                    E4 *__restrict__ w_out, int coeffs,
                                                    unsigned long long *acc, Publish pub,
                                                    const E4 *__restrict__ r_b,
                                                    size_t acc_stride) {
  pdl_wait();
  p_in += blockIdx.y * n_in;
  w_in += blockIdx.y * n_in;
  if (fold) {
    p_out += blockIdx.y * (n_in / 2);
    w_out += blockIdx.y * (n_in / 2);
    if (r_b) r = r_b[blockIdx.y];
  }
  unsigned long long *const acc_y = acc + blockIdx.y * acc_stride;
  size_t n = fold ? n_in / 2 : n_in;
  size_t pairs = (n + 1) / 2;
  E4 sums[2] = {kb::e_zero(), kb::e_zero()};
  for (size_t m = (size_t)blockIdx.x * blockDim.x + threadIdx.x; m < pairs;
       m += (size_t)gridDim.x * blockDim.x) {
    E4 p0, p1 = kb::e_zero(), w0, w1 = kb::e_zero();
    if (fold) {
      const E4 *pp = p_in + 4 * m, *ww = w_in + 4 * m;
      const bool two = 2 * m + 1 < n;
      const E4 a0 = ld_e4<VEC>(pp), a1 = ld_e4<VEC>(pp + 1);
      const E4 b0 = ld_e4<VEC>(ww), b1 = ld_e4<VEC>(ww + 1);
      E4 a2 = kb::e_zero(), a3 = kb::e_zero(), b2 = kb::e_zero(), b3 = kb::e_zero();
      if (two) {
        a2 = ld_e4<VEC>(pp + 2); a3 = ld_e4<VEC>(pp + 3);
        b2 = ld_e4<VEC>(ww + 2); b3 = ld_e4<VEC>(ww + 3);
      }
      p0 = kb::e_add(a0, kb::e_mul(r, kb::e_sub(a1, a0)));
      w0 = kb::e_add(b0, kb::e_mul(r, kb::e_sub(b1, b0)));
      st_e4<VEC>(p_out + 2 * m, p0);
      st_e4<VEC>(w_out + 2 * m, w0);
      if (two) {
        p1 = kb::e_add(a2, kb::e_mul(r, kb::e_sub(a3, a2)));
        w1 = kb::e_add(b2, kb::e_mul(r, kb::e_sub(b3, b2)));
        st_e4<VEC>(p_out + 2 * m + 1, p1);
        st_e4<VEC>(w_out + 2 * m + 1, w1);
      }
    } else {
      p0 = ld_e4<VEC>(p_in + 2 * m); w0 = ld_e4<VEC>(w_in + 2 * m);
      if (2 * m + 1 < n) { p1 = ld_e4<VEC>(p_in + 2 * m + 1); w1 = ld_e4<VEC>(w_in + 2 * m + 1); }
    }
    if (coeffs && 2 * m + 1 < n) {
      sums[0] = kb::e_add(sums[0], kb::e_mul(w0, p0));
      E4 dw = kb::e_sub(kb::e_dbl(w1), w0), dp = kb::e_sub(kb::e_dbl(p1), p0);
      sums[1] = kb::e_add(sums[1], kb::e_mul(dw, dp));
    }
  }
  if (coeffs) block_acc<2>(sums, acc_y, acc, pub);
}

static cudaError_t round_launch(const E4 *p_in, const E4 *w_in, size_t n_in, bool fold, E4 r,
                                const E4 *r_b, E4 *p_out, E4 *w_out, bool coeffs,
                                unsigned long long *acc, size_t acc_stride, int batch,
                                cudaStream_t st, const Publish &pub) {
  if (batch < 1 || batch > 65535) return cudaErrorInvalidValue;
  size_t n = fold ? n_in / 2 : n_in;
  size_t pairs = (n + 1) / 2;
  unsigned T = 256;
  size_t g = (pairs + T - 1) / T, cap = ((size_t)152 * 4 + batch - 1) / batch;
  dim3 grid((unsigned)(g < cap ? (g ? g : 1) : cap), (unsigned)batch);
  const bool vec = aligned16(p_in) && aligned16(w_in) &&
                   (!fold || (aligned16(p_out) && aligned16(w_out)));
  if (vec)
    launch(round_kernel<true>, grid, T, 0, st, p_in, w_in, n_in, fold ? 1 : 0, r, p_out, w_out,
           coeffs ? 1 : 0, acc, coeffs ? pub : Publish(), r_b, acc_stride);
  else
    launch(round_kernel<false>, grid, T, 0, st, p_in, w_in, n_in, fold ? 1 : 0, r, p_out, w_out,
           coeffs ? 1 : 0, acc, coeffs ? pub : Publish(), r_b, acc_stride);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t sumcheck_round(const E4 *p_in, const E4 *w_in, size_t n_in, bool fold, E4 r,
                           E4 *p_out, E4 *w_out, bool coeffs, unsigned long long *acc,
                           cudaStream_t st, const Publish &pub) {
  return round_launch(p_in, w_in, n_in, fold, r, nullptr, p_out, w_out, coeffs, acc, 0, 1, st,
                      pub);
}

cudaError_t sumcheck_round_batch(const E4 *p_in, const E4 *w_in, size_t n_in, bool fold,
                                 const E4 *r_b, E4 *p_out, E4 *w_out, bool coeffs,
                                 unsigned long long *acc, size_t acc_stride, int batch,
                                 cudaStream_t st, const Publish &pub) {
  if (fold && !r_b) return cudaErrorInvalidValue;
  return round_launch(p_in, w_in, n_in, fold, kb::e_zero(), r_b, p_out, w_out, coeffs, acc,
                      acc_stride, batch, st, pub);
}

// <eq(z), poly>: CTA walks hi blocks of 2^s_lo contiguous entries.
// Batched: instance y = blockIdx.y reads poly + y 2^k, its tables at
// y tab_stride from eq_lo and eq_hi, and sums into acc + 4 y.
template <bool VEC>
__global__ void __launch_bounds__(256) eval_ext_kernel(const E4 *__restrict__ poly, int k,
                                                       const E4 *__restrict__ eq_lo, int s_lo,
                                                       const E4 *__restrict__ eq_hi,
                                                       unsigned long long *acc, Publish pub,
                                                       size_t tab_stride) {
  pdl_wait();
  size_t n_lo = (size_t)1 << s_lo, n_hi = (size_t)1 << (k - s_lo);
  poly += blockIdx.y * ((size_t)1 << k);
  eq_lo += blockIdx.y * tab_stride;
  eq_hi += blockIdx.y * tab_stride;
  E4 outer = kb::e_zero();
  for (size_t hh = blockIdx.x; hh < n_hi; hh += gridDim.x) {
    E4 inner = kb::e_zero();
    for (size_t l = threadIdx.x; l < n_lo; l += blockDim.x)
      inner = kb::e_add(inner, kb::e_mul(ld_e4<VEC>(eq_lo + l), ld_e4<VEC>(poly + hh * n_lo + l)));
    outer = kb::e_add(outer, kb::e_mul(inner, ld_e4<VEC>(eq_hi + hh)));
  }
  E4 v[1] = {outer};
  block_acc<1>(v, acc + 4 * (size_t)blockIdx.y, acc, pub);
}

cudaError_t eval_ext_batch(const E4 *poly, int k, const E4 *eq_lo, int s_lo, const E4 *eq_hi,
                           size_t tab_stride, int batch, unsigned long long *acc,
                           cudaStream_t st, const Publish &pub) {
  if (batch < 1 || batch > 65535 || s_lo > k) return cudaErrorInvalidValue;
  size_t n_hi = (size_t)1 << (k - s_lo), cap = ((size_t)152 * 8 + batch - 1) / batch;
  dim3 grid((unsigned)(n_hi < cap ? n_hi : cap), (unsigned)batch);
  if (aligned16(poly) && aligned16(eq_lo) && aligned16(eq_hi))
    launch(eval_ext_kernel<true>, grid, 256, 0, st, poly, k, eq_lo, s_lo, eq_hi, acc, pub,
           tab_stride);
  else
    launch(eval_ext_kernel<false>, grid, 256, 0, st, poly, k, eq_lo, s_lo, eq_hi, acc, pub,
           tab_stride);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t eval_ext(const E4 *poly, int k, const E4 *eq_lo, int s_lo, const E4 *eq_hi,
                     unsigned long long *acc, cudaStream_t st, const Publish &pub) {
  return eval_ext_batch(poly, k, eq_lo, s_lo, eq_hi, 0, 1, acc, st, pub);
}

// <poly, weights> = sum_i poly[i] weights[i] (Expression::prod, the debug
// invariant of crates/whir/src/sumcheck/expr.rs:68) -> acc u64[4]
template <bool VEC>
__global__ void __launch_bounds__(256) dot_ext_kernel(const E4 *__restrict__ a,
                                                     const E4 *__restrict__ b, size_t n,
                                                     unsigned long long *acc, Publish pub) {
  pdl_wait();
  E4 s = kb::e_zero();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    s = kb::e_add(s, kb::e_mul(ld_e4<VEC>(a + i), ld_e4<VEC>(b + i)));
  E4 v[1] = {s};
  block_acc<1>(v, acc, acc, pub);
}

cudaError_t dot_ext(const E4 *a, const E4 *b, size_t n, unsigned long long *acc, cudaStream_t st,
                    const Publish &pub) {
  size_t g = (n + 255) / 256;
  unsigned grid = (unsigned)(g < 152 * 4 ? (g ? g : 1) : 152 * 4);
  if (aligned16(a) && aligned16(b))
    launch(dot_ext_kernel<true>, grid, 256, 0, st, a, b, n, acc, pub);
  else
    launch(dot_ext_kernel<false>, grid, 256, 0, st, a, b, n, acc, pub);
  count_launches(1);
  return cudaGetLastError();
}

// Batched: instance y = blockIdx.y evaluates rows idx[off[y] .. off[y+1])
// of its own codeword, which is interleaved with the others' (row r of
// instance y is row r batch + y of rows), at its own rs (rs_b[y ks ..]).
__global__ void row_evals_kernel(const uint32_t *__restrict__ rows, int row_len,
                                 const uint32_t *__restrict__ idx, int n, Point rs,
                                 const int *__restrict__ off, const E4 *__restrict__ rs_b,
                                 int batch, E4 *out) {
  pdl_wait();
  __shared__ E4 eq[256];
  const int y = blockIdx.y;
  for (int b = threadIdx.x; b < row_len; b += blockDim.x) {
    E4 a = kb::e_one();
    for (int i = 0; i < rs.k; i++) {
      const E4 zi = rs_b ? rs_b[(size_t)y * rs.k + i] : rs.z[i];
      a = kb::e_mul(a, ((b >> i) & 1) ? zi : kb::e_sub(kb::e_one(), zi));
    }
    eq[b] = a;
  }
  __syncthreads();
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int q0 = off ? off[y] : 0, nq = off ? off[y + 1] - q0 : n;
  if (q >= nq) return;
  q += q0;
  const uint32_t *row = rows + ((size_t)idx[q] * batch + y) * row_len;
  E4 a = kb::e_zero();
  for (int j = 0; j < row_len; j++) a = kb::e_add(a, kb::e_scale(eq[j], row[j]));
  out[q] = a;
}

cudaError_t row_evals(const uint32_t *rows, int row_len, const uint32_t *idx, int n,
                      const Point &rs, E4 *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (row_len > 256 || (1 << rs.k) != row_len) return cudaErrorInvalidValue;
  launch(row_evals_kernel, (n + 127) / 128, 128, 0, st, rows, row_len, idx, n, rs, nullptr,
         nullptr, 1, out);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t row_evals_batch(const uint32_t *rows, int row_len, const uint32_t *idx,
                            const int *off, int max_n, int ks, const E4 *rs_b, int batch,
                            E4 *out, cudaStream_t st) {
  if (max_n == 0) return cudaSuccess;
  if (row_len > 256 || (1 << ks) != row_len || batch < 1 || batch > 65535)
    return cudaErrorInvalidValue;
  Point rs;
  rs.k = ks;
  dim3 grid((unsigned)((max_n + 127) / 128), (unsigned)batch);
  launch(row_evals_kernel, grid, 128, 0, st, rows, row_len, idx, 0, rs, off, rs_b, batch, out);
  count_launches(1);
  return cudaGetLastError();
}

// ---- fold_with_code's code part (crates/whir/src/sumcheck/prover.rs:400-561) ----
// Query i keeps G[i T .. i T + 2^(d-r)) = g(r, base_i + t S) (S = 2^(k_data -
// d), base_i = idx_i mod S, T = 2^d): round 0 holds the row evaluations at
// eq(rs); round r >= 1 folds G with r_(r-1) (prover.rs:437-461), the
// twiddle of position t being B_i wd^(t 2^(r-1)) with B_i = w^-(base_i
// 2^(r-1)) and wd = w^-S.  Each query adds its part of (c0, c2)
// (prover.rs:503-536) to acc[0..8) and, at round 0, scales_i g(0, idx_i) to
// acc[8..12), as canonical words; the host reduces them with the round pass.
__device__ __forceinline__ void acc_add_e4(unsigned long long *acc, const E4 &v) {
#pragma unroll
  for (int c = 0; c < 4; c++) atomicAdd(acc + c, (unsigned long long)v.c[c]);
}

__device__ __forceinline__ void code_round_query(CodeState s, int round, E4 r_prev,
                                                 unsigned long long *acc) {
  using namespace kb;
  const int i = blockIdx.x;
  const int lS = s.k_data - s.d;
  const int T = 1 << s.d;
  const uint32_t idx = s.idx[i];
  const uint32_t base = idx & ((1u << lS) - 1u), tb = idx >> lS;
  E4 *G = s.G + (size_t)i * T;
  __shared__ uint32_t pw[3];
  if (round == 0) {
    // w^idx, w^-(idx mod 2^(k_data-1)), w^-base: one exponentiation per lane
    if (threadIdx.x < 3) {
      uint32_t b = threadIdx.x == 0 ? s.omega : s.winv;
      uint32_t e = threadIdx.x == 0 ? idx
                   : threadIdx.x == 1 ? (idx & ((1u << (s.k_data - 1)) - 1u))
                                      : base;
      pw[threadIdx.x] = kb::pow(b, e);
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    E4 sc = s.scales[i];
    s.ws[i] = pw[0];
    s.tw[i] = pw[1];
    s.B[i] = pw[2];
    acc_add_e4(acc + 8, e_mul(sc, G[tb]));
  } else {
    const int half = T >> round;
    const uint32_t B = s.B[i];
    for (int t = threadIdx.x; t < half; t += blockDim.x) {
      uint32_t tw = mul(B, s.wd[(t << (round - 1)) & (T - 1)]);
      E4 glo = G[t], ghi = G[t + half];
      E4 even = e_scale(e_add(glo, ghi), s.two_inv);
      E4 odd = e_scale(e_sub(glo, ghi), mul(s.two_inv, tw));
      G[t] = e_add(even, e_mul(r_prev, e_sub(odd, even)));
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    // the updates after round r-1 (prover.rs:542-553)
    uint32_t ws = s.ws[i], tw = s.tw[i];
    E4 f = e_add(e_one(), e_mul(r_prev, e_add(e_neg(e_one()), e_from(ws))));
    s.scales[i] = e_mul(s.scales[i], f);
    ws = mul(ws, ws);
    tw = mul(tw, tw);
    if ((idx >> (s.k_data - round - 1)) & 1u) tw = neg(tw);
    s.ws[i] = ws;
    s.tw[i] = tw;
    s.B[i] = mul(B, B);
  }
  const E4 sc = s.scales[i];
  const uint32_t ws = s.ws[i], tw = s.tw[i];
  const int hlf = (T >> round) / 2;
  const uint32_t tl = tb & (uint32_t)(hlf - 1);
  E4 glo = G[tl], ghi = G[tl + hlf];
  E4 even = e_scale(e_add(glo, ghi), s.two_inv);
  E4 odd = e_scale(e_scale(e_sub(glo, ghi), s.two_inv), tw);
  acc_add_e4(acc, e_mul(sc, even));
  uint32_t wt = sub(dbl(ws), ONE);
  acc_add_e4(acc + 4, e_scale(e_mul(sc, e_sub(e_dbl(odd), even)), wt));
}

__global__ void __launch_bounds__(32) code_round_kernel(CodeState s, int round, E4 r_prev,
                                                        unsigned long long *acc, Publish pub) {
  pdl_wait();
  const int b = s.inst ? s.inst[blockIdx.x] : 0;
  if (s.r_b && round > 0) r_prev = s.r_b[b];
  code_round_query(s, round, r_prev, acc + (size_t)b * s.acc_stride);
  publish_if_last(acc, pub);
}

// the updates after the last round, before combine_pows_scaled (combine.rs:441-468)
__global__ void code_finish_kernel(CodeState s, E4 r_last) {
  pdl_wait();
  using namespace kb;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.n) return;
  if (s.r_b) r_last = s.r_b[s.inst[i]];
  uint32_t ws = s.ws[i];
  E4 f = e_add(e_one(), e_mul(r_last, e_add(e_neg(e_one()), e_from(ws))));
  s.scales[i] = e_mul(s.scales[i], f);
  s.ws[i] = mul(ws, ws);
}

cudaError_t code_round(const CodeState &s, int round, E4 r_prev, unsigned long long *acc,
                       cudaStream_t st, const Publish &pub) {
  if (s.n == 0) return cudaSuccess;
  if (s.d < 1 || s.d > 8 || s.k_data < s.d || s.k_data > 30 || round < 0 || round >= s.d)
    return cudaErrorInvalidValue;
  launch(code_round_kernel, s.n, 32, 0, st, s, round, r_prev, acc, pub);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t code_finish(const CodeState &s, E4 r_last, cudaStream_t st) {
  if (s.n == 0) return cudaSuccess;
  launch(code_finish_kernel, (s.n + 127) / 128, 128, 0, st, s, r_last);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace gpu
}  // namespace whir
