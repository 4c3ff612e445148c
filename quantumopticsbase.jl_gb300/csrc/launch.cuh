// launch.cuh -- programmatic dependent launch (PDL) for the kernels of one
// operator application: the gathers, and the split -> tensor-core GEMM ->
// reduce chain of the ComplexF32 dense path.
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include "qob_internal.h"

namespace qob {

// A kernel launched with the programmatic stream-serialization attribute may
// start while the previous kernel of the stream finishes; it waits here,
// before its first access to memory, until that kernel has completed and its
// writes are visible, and lets the next such launch start in turn.  Without
// the attribute both are no-ops.  The next launch's blocks are scheduled only
// once every block of this grid has passed this point (or exited), so they
// never take resources that this grid's blocks still wait for.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// A launch with the programmatic stream-serialization attribute when pdl is set
// (the kernel calls pdl_enter before its first access to memory), else an
// ordinary one.
template <typename... KArgs, typename... Args>
void launch_kernel(bool pdl, void (*kernel)(KArgs...), dim3 grid, unsigned threads, size_t smem, cudaStream_t s,
                   Args&&... args) {
  if (!pdl) {
    kernel<<<grid, threads, smem, s>>>(std::forward<Args>(args)...);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  QOB_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

}  // namespace qob
