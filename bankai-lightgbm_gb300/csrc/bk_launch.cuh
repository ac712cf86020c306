// Kernel launches of the grow loop with programmatic dependent launch: each grow-loop kernel is
// launched with programmatic stream serialization, so it is scheduled while the kernel before it
// finishes. It runs its independent prologue (shared-memory setup, static metadata), then waits in
// griddep_wait() until the previous grid has completed and its writes are visible. The histogram,
// search and single-pass partition kernels call griddep_launch() right after that wait, so the
// next kernel's CTAs are resident and through their own prologue by the time this one completes
// (every grid of the chain is small enough to be resident beside the one before it); the stable
// partition's kernels call it when only their last-CTA bookkeeping is left. Without the launch
// attribute (or when the previous stream operation is not a kernel) both are no-ops.
#pragma once
#include <cuda_runtime.h>

namespace bk {

__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// cudaLaunchKernelEx with (pdl != 0) the programmatic-stream-serialization attribute.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_kernel(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, int pdl,
                                 Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = pdl ? attr : nullptr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

}  // namespace bk
