// Programmatic dependent launch helpers (used by the exact-adjoint step's
// chain of short launches; measured slower on the FP64 two-kernel step).
#pragma once

#include <cuda_runtime.h>

namespace psv {
namespace kern {

// Programmatic dependent launch: consecutive launches on a stream overlap
// their start with the previous kernel's tail; pdl_wait() returns once the
// previous kernel has completed and its writes are visible (a no-op when
// launched without the attribute).
__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename K, typename... Args>
cudaError_t launch_pdl(K kernel, dim3 grid, dim3 block, cudaStream_t s, Args... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = grid;
  lc.blockDim = block;
  lc.dynamicSmemBytes = 0;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, kernel, args...);
}

}  // namespace kern
}  // namespace psv
