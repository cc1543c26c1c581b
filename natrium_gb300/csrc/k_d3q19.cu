// Kernel instantiations for D3Q19 (compiled as its own translation unit).
#include "launch.h"
#include "sl_step.cuh"

namespace natgpu {

template <class Real>
static KernelSet pick_d3q19(int coll) {
  using S = SD3Q19;
  switch (coll) {
    case L_COLL_NONE:
      return {(const void*)&k_sl_step<S, Real, COLL_NONE, STEP_NPT>, nullptr, nullptr};
    case L_COLL_BGK:
      return {(const void*)&k_sl_step<S, Real, COLL_BGK, STEP_NPT>,
              (const void*)&k_collide<S, Real, COLL_BGK>, (const void*)&k_wall_nodes<S, Real, COLL_BGK>,
              (const void*)&k_sl_step<S, Real, COLL_BGK, STEP_NPT, true>,
              (const void*)&k_collide<S, Real, COLL_BGK, true>, (const void*)&k_wall_nodes<S, Real, COLL_BGK, true>};
    default:
      return {nullptr, nullptr, nullptr};
  }
}

KernelSet kernels_d3q19(int coll, int prec) {
  return prec == 0 ? pick_d3q19<double>(coll) : pick_d3q19<float>(coll);
}

}  // namespace natgpu
