// Cell-row kernel instantiations: D3Q27, FP64, p = 3 (2 x double2 loads per cell row).
#include "k_cell.h"

namespace natgpu {

void cell_kernels_q27d(std::vector<RowLaunch>& v) {
  using namespace cellreg;
  add_shapes<SD3Q27, double, COLL_KBC, 3, 32>(v, L_COLL_KBC);
  add_shapes<SD3Q27, double, COLL_BGK, 3, 32>(v, L_COLL_BGK);
  add_shapes<SD3Q27, double, COLL_KBC, 3, 32, true>(v, L_COLL_KBC);
}

}  // namespace natgpu
