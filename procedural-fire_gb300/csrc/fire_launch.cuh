// Programmatic dependent launch (PDL) for the chains of dependent kernels in the step graph.
//
// Every kernel of the step calls pdl_wait() before it reads anything its predecessor wrote, then
// pdl_trigger(), so the next kernel's CTAs may be launched as soon as all CTAs of this grid have started:
// the dependent launch overlaps this grid's last wave instead of waiting for it to drain.  Launches go
// through launch_pdl(), which sets cudaLaunchAttributeProgrammaticStreamSerialization; stream capture
// records the programmatic edge in the graph.  After a non-kernel predecessor (a copy, an event record,
// a conditional node) the attribute has no effect and the dependency is an ordinary one.
#pragma once
#include <cuda_runtime.h>
#include <utility>

namespace fire {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args&&... args) {
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
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace fire
