// Kernel instantiations for D2Q9 (compiled as its own translation unit).
#include "launch.h"
#include "sl_step.cuh"

namespace natgpu {

template <class Real>
static KernelSet pick_d2q9(int coll) {
  using S = SD2Q9;
  switch (coll) {
    case L_COLL_NONE:
      return {(const void*)&k_sl_step<S, Real, COLL_NONE, STEP_NPT>, nullptr, nullptr};
    case L_COLL_BGK:
      return {(const void*)&k_sl_step<S, Real, COLL_BGK, STEP_NPT>,
              (const void*)&k_collide<S, Real, COLL_BGK>, (const void*)&k_wall_nodes<S, Real, COLL_BGK>,
              (const void*)&k_sl_step<S, Real, COLL_BGK, STEP_NPT, true>,
              (const void*)&k_collide<S, Real, COLL_BGK, true>, (const void*)&k_wall_nodes<S, Real, COLL_BGK, true>};
    case L_COLL_BGK_INC:
      return {(const void*)&k_sl_step<S, Real, COLL_BGK_INC, STEP_NPT>,
              (const void*)&k_collide<S, Real, COLL_BGK_INC>, (const void*)&k_wall_nodes<S, Real, COLL_BGK_INC>};
    case L_COLL_KBC:
      return {(const void*)&k_sl_step<S, Real, COLL_KBC, STEP_NPT>,
              (const void*)&k_collide<S, Real, COLL_KBC>, (const void*)&k_wall_nodes<S, Real, COLL_KBC>};
    default:
      return {nullptr, nullptr, nullptr};
  }
}

KernelSet kernels_d2q9(int coll, int prec) {
  return prec == 0 ? pick_d2q9<double>(coll) : pick_d2q9<float>(coll);
}

}  // namespace natgpu
