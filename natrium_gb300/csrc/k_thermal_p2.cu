// Fused two-population step (sl_thermal.cuh) instantiated for order 2: the
// window loops run over three slots at compile time.
#include "launch.h"
#include "thermal_step.h"

namespace natgpu {

template <class Real>
static cudaError_t step_p2(const ThermalStepT<Real>& P, bool collide, cudaStream_t st, int form) {
  if constexpr (sizeof(Real) == 4) {
    if (form == 1) return thermal_step_form<Real, 1, 2>(P, collide, st);
    if (form == 2) return thermal_step_form<Real, 2, 2>(P, collide, st);
    if (form == 3) return thermal_step_form<Real, 3, 2>(P, collide, st);
  }
  return thermal_step_form<Real, 0, 2>(P, collide, st);
}

cudaError_t launch_thermal_step_p2(const ThermalStepT<double>& P, bool collide, cudaStream_t st, int form) {
  return step_p2(P, collide, st, form);
}
cudaError_t launch_thermal_step_p2(const ThermalStepT<float>& P, bool collide, cudaStream_t st, int form) {
  return step_p2(P, collide, st, form);
}

}  // namespace natgpu
