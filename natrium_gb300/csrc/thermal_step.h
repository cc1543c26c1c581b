// Launch of the fused two-population step (sl_thermal.cuh) in a given form
// and order instantiation; shared by k_thermal.cu (any order) and
// k_thermal_p2.cu (order 2).
#pragma once
#include <cuda_runtime.h>

#include "sl_thermal.cuh"

namespace natgpu {

// form: 0 register form (TH_WARPS warps per CTA), 1 / 2 shared-memory forms
// (TH_WARPS_SS warps per CTA, FP32 only), 3 the register form with staged
// rows (FP32, order 2 only; sl_thermal.cuh); PC: the order as a compile-time
// constant, 0 for any
template <class Real, int FORM, int PC>
cudaError_t thermal_step_form(const ThermalStepT<Real>& P, bool collide, cudaStream_t st) {
  constexpr int W = th_warps<FORM>();
  const int warps = P.nseg * P.ny;
  const int grid = (warps + W - 1) / W;
  void* args[] = {const_cast<ThermalStepT<Real>*>(&P)};
  const void* fn = collide ? (const void*)k_thermal_step<Real, true, W, FORM, PC>
                           : (const void*)k_thermal_step<Real, false, W, FORM, PC>;
  if (!P.wall_bits) return cudaLaunchKernel(fn, dim3(grid), dim3(32 * W), args, 0, st);
  // after k_thermal_rows: programmatic dependent launch, the lattice streams
  // while the rows run; the wall lanes wait for them (griddepcontrol.wait)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(32 * W);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, fn, args);
}

cudaError_t launch_thermal_step_p2(const ThermalStepT<double>& P, bool collide, cudaStream_t st, int form);
cudaError_t launch_thermal_step_p2(const ThermalStepT<float>& P, bool collide, cudaStream_t st, int form);

}  // namespace natgpu
