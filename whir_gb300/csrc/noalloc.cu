// whir_compress_hi_noalloc: the SVO claim compression (compress_hi) without
// any memory allocation, for callers that cannot allocate device memory.
//
// Who needs it: a host whose device memory is entirely handed out up front
// by its own pool (a proving service with a fixed per-GPU budget, or another
// framework's caching allocator that owns the device) cannot let a library
// call cudaMalloc behind its back, and latency-sensitive callers must avoid
// cudaMalloc/cudaFree in the middle of a proof because those calls can
// synchronize the whole device and stall every other stream.  The regular
// whir_compress_hi grows per-context scratch buffers with cudaMalloc; this
// variant instead uses one fixed 40 KiB array in device global memory that
// every GPU loading the library holds until the process exits.
//
// Scratch layout (g_noalloc_scratch): split eq tables lo (2^10 extension
// elements) and hi (2^10), then the 64-bit accumulators (4 words for each of
// at most 2^8 outputs).  The tables are rewritten by every call; the
// accumulators are cleared by every call before use.  All calls share the
// array, so calls must be serialised: issued to one stream from one host
// thread, or under the caller's own lock.  Calls that overlap on the GPU
// (different streams) race, and so do calls that two host threads queue on
// the same stream at the same time (their launches interleave, and both read
// the combined accumulators).
//
// The device address of the array is looked up once per device
// (cudaGetSymbolAddress with that device current) by the first call made on
// that device; make that first call before any stream capture begins.  The
// address is kept for the life of the process: a cudaDeviceReset reloads the
// module and may move the array, so do not call this entry point after
// resetting the device in the same process.
#include <mutex>

#include "../../include/whir_gb300.h"
#include "kernels.h"

void whir_record_error(const char *msg);  // capi.cpp: text for whir_last_error()

namespace {

constexpr int NA_MAX_FIXED = 20;  // variables fixed to the point (kz)
constexpr int NA_MAX_KEPT = 8;    // variables left free (k - kz): at most 256 outputs
constexpr int NA_LO_LOG = 10;
constexpr size_t NA_LO_BYTES = sizeof(kb::E4) << NA_LO_LOG;
constexpr size_t NA_HI_BYTES = sizeof(kb::E4) << (NA_MAX_FIXED - NA_LO_LOG);
constexpr size_t NA_ACC_WORDS = (size_t)4 << NA_MAX_KEPT;
constexpr size_t NA_BYTES = NA_LO_BYTES + NA_HI_BYTES + 8 * NA_ACC_WORDS;  // 40 KiB
}  // namespace

// the fixed scratch; host code must use its device address, never this name
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

namespace {
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
void *g_na_addr[NA_MAX_DEVICES];

int fail(int code, const char *msg) {
  whir_record_error(msg);
  return code;
}

}  // namespace

extern "C" int whir_compress_hi_noalloc(void *cuda_stream, const uint32_t *poly, int k,
                                        const uint32_t *point, int kz, uint32_t *out) {
  if (!poly || !out || (kz > 0 && !point))
    return fail(WHIR_ERR_ARG, "whir_compress_hi_noalloc: null argument");
  if (kz < 0 || kz > k)
    return fail(WHIR_ERR_ARG, "whir_compress_hi_noalloc: need 0 <= kz <= k");
  if (kz > NA_MAX_FIXED || k - kz > NA_MAX_KEPT)
    return fail(WHIR_ERR_ARG,
                "whir_compress_hi_noalloc: at most 20 fixed variables (kz) and 8 kept "
                "variables (k - kz) fit its fixed 40 KiB scratch; use whir_compress_hi");
  whir::gpu::Point z;
  z.k = kz;
  for (int i = 0; i < kz; i++)
    for (int c = 0; c < 4; c++) {
      uint32_t v = point[4 * i + c];
      if (v >= kb::P) return fail(WHIR_ERR_ARG, "whir_compress_hi_noalloc: non-canonical point");
      z.z[i].c[c] = v;
    }

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES)
    return fail(WHIR_ERR_CUDA, "whir_compress_hi_noalloc: no usable current device");
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev]) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
        return fail(WHIR_ERR_CUDA, "whir_compress_hi_noalloc: cudaGetSymbolAddress failed");
      g_na_addr[dev] = p;
    }
    base = static_cast<unsigned char *>(g_na_addr[dev]);
  }
  kb::E4 *lo = reinterpret_cast<kb::E4 *>(base);
  kb::E4 *hi = reinterpret_cast<kb::E4 *>(base + NA_LO_BYTES);
  unsigned long long *acc = reinterpret_cast<unsigned long long *>(base + NA_LO_BYTES + NA_HI_BYTES);

  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  const int ks = k - kz;
  const int s_lo = kz < NA_LO_LOG ? kz : NA_LO_LOG;
  const size_t words = (size_t)4 << ks;
  if (whir::gpu::eq_split(z, s_lo, kb::e_one(), lo, hi, st) != cudaSuccess)
    return fail(WHIR_ERR_CUDA, "whir_compress_hi_noalloc: eq table launch failed");
  if (cudaMemsetAsync(acc, 0, 8 * words, st) != cudaSuccess)
    return fail(WHIR_ERR_CUDA, "whir_compress_hi_noalloc: clearing the accumulators failed");
  if (whir::gpu::compress_hi(poly, k, ks, lo, s_lo, hi, acc, st) != cudaSuccess)
    return fail(WHIR_ERR_CUDA, "whir_compress_hi_noalloc: compress_hi launch failed");
  unsigned long long h[NA_ACC_WORDS];
  if (cudaMemcpyAsync(h, acc, 8 * words, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail(WHIR_ERR_CUDA, "whir_compress_hi_noalloc: reading the result failed");
  for (size_t i = 0; i < words; i++) out[i] = (uint32_t)(h[i] % kb::P);
  return WHIR_OK;
}
