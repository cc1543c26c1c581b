// Cell-row kernel instantiations: D3Q19, FE_Q (continuous) nodes, p = 4 (a
// lane owns its cell's 4 non-shared nodes: float4 / 2 x double2 loads).
#include "k_cell.h"

namespace natgpu {

void cell_kernels_q19feq(std::vector<RowLaunch>& v) {
  using namespace cellreg;
  add_shapes<SD3Q19, float, COLL_BGK, 4, 16, false, false>(v, L_COLL_BGK);
  add_shapes<SD3Q19, double, COLL_BGK, 4, 16, false, false>(v, L_COLL_BGK);
  add_shapes<SD3Q19, double, COLL_BGK, 4, 16, true, false>(v, L_COLL_BGK);  // z sharing
}

}  // namespace natgpu
