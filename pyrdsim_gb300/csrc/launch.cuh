// launch.cuh -- kernel launches of the step engine (host code).
#pragma once

#include <cuda_runtime.h>

namespace rd {

// Kernel launch with programmatic stream serialization: the kernel may be
// scheduled while the previous kernel of the stream still runs (its launch
// and table staging overlap that kernel's tail); every kernel waits
// (griddepcontrol.wait) before it reads what earlier work writes.
template <class... P, class... A>
void launch(void (*k)(P...), dim3 grid, dim3 block, cudaStream_t st, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, static_cast<P>(args)...);
}

}  // namespace rd
