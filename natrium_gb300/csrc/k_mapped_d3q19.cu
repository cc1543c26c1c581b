// Departure-point kernels of mapped (MappingQ1) meshes for D3Q19, orders 1-6
// (compiled as its own translation unit).
#include "launch.h"
#include "sl_mapped.cuh"

namespace natgpu {

template <class Real>
static const void* pick(int coll, int p) {
  if (coll == L_COLL_BGK_FORCE) return mapped_for_order<SD3Q19, Real, COLL_BGK, true>(p);
  switch (coll) {
    case L_COLL_NONE: return mapped_for_order<SD3Q19, Real, COLL_NONE>(p);
    case L_COLL_BGK: return mapped_for_order<SD3Q19, Real, COLL_BGK>(p);
  }
  return nullptr;
}

const void* mapped_kernel_d3q19(int coll, int prec, int p) { return prec == 0 ? pick<double>(coll, p) : pick<float>(coll, p); }

}  // namespace natgpu
