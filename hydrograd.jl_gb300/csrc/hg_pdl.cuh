// Programmatic dependent launch (sm_90 and later).  A kernel launched with the
// programmatic-serialization attribute may be scheduled while the kernel
// before it in the stream is still running -- once every CTA of that kernel
// has executed griddepcontrol.launch_dependents or exited -- so its launch
// latency hides under the other's tail.  Before it touches anything the
// kernels before it read or write, it executes griddepcontrol.wait, which
// returns when they have completed and their memory is visible.  Launched
// without the attribute, the wait returns at once.
//
// Kernels of a chain call pdl_enter() first: wait, then release the next.  A
// kernel whose wait comes later (it shares nothing with the kernel before it)
// must only follow a kernel that has itself waited before releasing it.
#pragma once

#include <cuda_runtime.h>

#include <utility>

namespace hg {

__device__ __forceinline__ void pdl_release_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait_prerequisites() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_enter() {
  pdl_wait_prerequisites();
  pdl_release_dependents();
}

// Launch k<<<grid, block, smem, st>>>(args...), as a programmatic dependent
// of the kernel before it in st when pdl is set.
template <class... KArgs, class... Args>
cudaError_t launch_k(bool pdl, void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

}  // namespace hg
