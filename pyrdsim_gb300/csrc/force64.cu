// force64.cu -- translation unit of the float64 drift kernels (force64.cuh),
// compiled apart from engine.cu so that the two build in parallel.
#include "force64.h"

#include "force64.cuh"
#include "launch.cuh"

namespace rd {

template <int D>
static void launch_force64_d(int tpp, unsigned grid, cudaStream_t st, const Args& a) {
  if (tpp == 1) launch(k_force_d<D, 1>, grid, LBLOCK, st, a);
  else if (tpp == 2) launch(k_force_d<D, 2>, grid, LBLOCK, st, a);
  else if (tpp == 8) launch(k_force_d<D, 8>, grid, LBLOCK, st, a);
  else launch(k_force_d<D, 4>, grid, LBLOCK, st, a);
}

cudaError_t launch_force64(int D, int tpp, unsigned grid, cudaStream_t st, const Args& a) {
  if (D == 2) launch_force64_d<2>(tpp, grid, st, a);
  else if (D == 3) launch_force64_d<3>(tpp, grid, st, a);
  else launch_force64_d<1>(tpp, grid, st, a);
  return cudaGetLastError();
}

cudaError_t launch_em64(int D, unsigned grid, cudaStream_t st, const Args& a, const int* sid) {
  if (D == 2) launch(k_em_d<2>, grid, 256, st, a, sid);
  else if (D == 3) launch(k_em_d<3>, grid, 256, st, a, sid);
  else launch(k_em_d<1>, grid, 256, st, a, sid);
  return cudaGetLastError();
}

}  // namespace rd
