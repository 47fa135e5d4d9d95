// Kernel launches with programmatic dependent launch (sm_90 and later).
//
// A launch made with launch() may be processed by the device while the
// kernel before it in the stream is still finishing, instead of after a full
// stream serialisation: on GB300 a chain of dependent kernels of about 10 us
// each took 10.8 us per kernel this way against 12.3 us with plain launches
// (the gap between them shrinks from about 2.3 us to under 1 us).  In
// exchange every kernel of this library begins with pdl_wait(), which returns
// once the preceding grid in the stream has completed and its memory writes
// are visible; nothing of the kernel runs before it, so each kernel sees
// exactly what it would after a plain launch.  (griddepcontrol.wait returns
// at once in a kernel that was launched without the attribute.)
#pragma once
#include <cuda_runtime.h>

#include <utility>

namespace whir {
namespace gpu {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// kernel<<<grid, block, smem, stream>>>(args...) with the attribute set; the
// arguments are converted to the kernel's parameter types as <<<>>> does.
// Errors are also left for cudaGetLastError().
template <class... P, class... A>
inline cudaError_t launch(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem,
                          cudaStream_t st, A &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

}  // namespace gpu
}  // namespace whir
