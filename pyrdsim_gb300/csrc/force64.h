// force64.h -- launches of the float64 drift kernels (force64.cu), the
// "plain method" in the reference's own precision.
#pragma once

#include <cuda_runtime.h>

#include "device.cuh"

namespace rd {

// k_force_d<D, tpp> over `grid` CTAs of the step kernels' size.
cudaError_t launch_force64(int D, int tpp, unsigned grid, cudaStream_t st, const Args& a);
// k_em_d<D>: the stand-alone float64 Euler-Maruyama update.
cudaError_t launch_em64(int D, unsigned grid, cudaStream_t st, const Args& a, const int* sid);

}  // namespace rd
