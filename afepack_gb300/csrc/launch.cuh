// Kernel launches with programmatic dependent launch (PDL).
//
// The V-cycle and the CG loop are long chains of small dependent kernels.
// Launched with cudaLaunchAttributeProgrammaticStreamSerialization, kernel
// N+1 is scheduled while kernel N drains; every kernel of the chain starts
// with pdl_wait() (griddepcontrol.wait), which returns once its predecessor
// has completed and flushed its memory, so the data dependences are kept.
// On a launch without the attribute pdl_wait() returns at once.
// AFP_NO_PDL=1 in the environment turns the attribute off (A/B timing).
#pragma once

#include <cuda_runtime.h>

#include <cstdlib>
#include <utility>

namespace afp {

inline bool pdl_enabled() {
  static const bool on = std::getenv("AFP_NO_PDL") == nullptr;
  return on;
}

template <class... KArgs, class... Args>
inline cudaError_t launch_pdl(cudaStream_t stream, dim3 grid, dim3 block, size_t smem, void (*kernel)(KArgs...),
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  if (pdl_enabled()) {
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Wait for the predecessor grid, then let the successor grid get scheduled.
__device__ __forceinline__ void pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

}  // namespace afp
