// Kernel instantiations for D3Q27 (compiled as its own translation unit).
#include "launch.h"
#include "sl_step.cuh"

namespace natgpu {

template <class Real>
static KernelSet pick_d3q27(int coll) {
  using S = SD3Q27;
  switch (coll) {
    case L_COLL_NONE:
      return {(const void*)&k_sl_step<S, Real, COLL_NONE, STEP_NPT>, nullptr, nullptr};
    case L_COLL_BGK:
      return {(const void*)&k_sl_step<S, Real, COLL_BGK, STEP_NPT>,
              (const void*)&k_collide<S, Real, COLL_BGK>, (const void*)&k_wall_nodes<S, Real, COLL_BGK>,
              (const void*)&k_sl_step<S, Real, COLL_BGK, STEP_NPT, true>,
              (const void*)&k_collide<S, Real, COLL_BGK, true>, (const void*)&k_wall_nodes<S, Real, COLL_BGK, true>};
    case L_COLL_KBC:
      return {(const void*)&k_sl_step<S, Real, COLL_KBC, STEP_NPT>,
              (const void*)&k_collide<S, Real, COLL_KBC>, (const void*)&k_wall_nodes<S, Real, COLL_KBC>};
    default:
      return {nullptr, nullptr, nullptr};
  }
}

KernelSet kernels_d3q27(int coll, int prec) {
  return prec == 0 ? pick_d3q27<double>(coll) : pick_d3q27<float>(coll);
}

}  // namespace natgpu
