// Kernels of the compressible two-population model (sl_thermal.cuh) and
// their host launchers.
#include <cuda_runtime.h>

#include "launch.h"
#include "sl_thermal.cuh"

namespace natgpu {

cudaError_t launch_thermal_step(const ThermalStep& P, bool collide, cudaStream_t st) {
  const int warps = P.nseg * P.ny;
  const int grid = (warps + TH_WARPS - 1) / TH_WARPS;
  void* args[] = {const_cast<ThermalStep*>(&P)};
  const void* fn = collide ? (const void*)k_thermal_step<true> : (const void*)k_thermal_step<false>;
  return cudaLaunchKernel(fn, dim3(grid), dim3(32 * TH_WARPS), args, 0, st);
}

cudaError_t launch_thermal_collide(const ThermalPoint& P, int grid, cudaStream_t st) {
  void* args[] = {const_cast<ThermalPoint*>(&P)};
  return cudaLaunchKernel((const void*)k_thermal_collide, dim3(grid), dim3(256), args, 0, st);
}

cudaError_t launch_thermal_init(const ThermalPoint& P, int grid, cudaStream_t st) {
  void* args[] = {const_cast<ThermalPoint*>(&P)};
  return cudaLaunchKernel((const void*)k_thermal_init, dim3(grid), dim3(256), args, 0, st);
}

}  // namespace natgpu
