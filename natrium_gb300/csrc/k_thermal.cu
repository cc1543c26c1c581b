// Kernels of the compressible two-population model (sl_thermal.cuh) and
// their host launchers: FP64 and FP32-deviation instantiations.
#include <cuda_runtime.h>

#include "launch.h"
#include "thermal_step.h"

namespace natgpu {

template <class Real>
static cudaError_t step_t(const ThermalStepT<Real>& P, bool collide, cudaStream_t st, int form) {
  // order 2 (the compressible benchmark's) has its own instantiations with
  // compile-time window loops (k_thermal_p2.cu)
  if (P.tb.p == 2) return launch_thermal_step_p2(P, collide, st, form);
  if constexpr (sizeof(Real) == 4) {
    if (form == 1) return thermal_step_form<Real, 1, 0>(P, collide, st);
    if (form == 2) return thermal_step_form<Real, 2, 0>(P, collide, st);
  }
  return thermal_step_form<Real, 0, 0>(P, collide, st);
}

cudaError_t launch_thermal_step(const ThermalStepT<double>& P, bool collide, cudaStream_t st, int form) {
  return step_t(P, collide, st, form);
}
cudaError_t launch_thermal_step(const ThermalStepT<float>& P, bool collide, cudaStream_t st, int form) {
  return step_t(P, collide, st, form);
}

template <class Real>
static cudaError_t collide_t(const ThermalPointT<Real>& P, int grid, cudaStream_t st) {
  void* args[] = {const_cast<ThermalPointT<Real>*>(&P)};
  return cudaLaunchKernel((const void*)k_thermal_collide<Real>, dim3(grid), dim3(256), args, 0, st);
}

cudaError_t launch_thermal_collide(const ThermalPointT<double>& P, int grid, cudaStream_t st) {
  return collide_t(P, grid, st);
}
cudaError_t launch_thermal_collide(const ThermalPointT<float>& P, int grid, cudaStream_t st) {
  return collide_t(P, grid, st);
}

cudaError_t launch_thermal_init(const ThermalPointT<double>& P, void* f, void* g, bool fp32, int grid,
                                cudaStream_t st) {
  if (fp32) {
    k_thermal_init<float><<<grid, 256, 0, st>>>(P, static_cast<float*>(f), static_cast<float*>(g));
  } else {
    k_thermal_init<double><<<grid, 256, 0, st>>>(P, static_cast<double*>(f), static_cast<double*>(g));
  }
  return cudaGetLastError();
}

template <class Real>
static cudaError_t wall_nodes_t(const ThermalStepT<Real>& P, int nbn, const int* node, const int* ptr,
                                const int* col, const Real* w, const double* cst, bool collide, cudaStream_t st) {
  const int nrows = nbn * (TH_Q - 1);
  k_thermal_rows<Real><<<(nrows + 255) / 256, 256, 0, st>>>(P, nrows, node, ptr, col, w, cst);
  if (collide) k_thermal_collide_nodes<Real><<<(nbn + 127) / 128, 128, 0, st>>>(P, nbn, node);
  return cudaGetLastError();
}

cudaError_t launch_thermal_wall_nodes(const ThermalStepT<double>& P, int nbn, const int* node, const int* ptr,
                                      const int* col, const double* w, const double* cst, bool collide,
                                      cudaStream_t st) {
  return wall_nodes_t(P, nbn, node, ptr, col, w, cst, collide, st);
}
cudaError_t launch_thermal_wall_nodes(const ThermalStepT<float>& P, int nbn, const int* node, const int* ptr,
                                      const int* col, const float* w, const double* cst, bool collide,
                                      cudaStream_t st) {
  return wall_nodes_t(P, nbn, node, ptr, col, w, cst, collide, st);
}

}  // namespace natgpu
