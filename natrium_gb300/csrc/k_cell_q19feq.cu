// Cell-row kernel instantiations on FE_Q (continuous) nodes: D3Q19 p = 4 (a
// lane owns its cell's 4 non-shared nodes: float4 / 2 x double2 loads) and
// D3Q27 KBC p = 3 (3 nodes per lane, FP32 deviation storage).
#include "k_cell.h"

namespace natgpu {

void cell_kernels_q19feq(std::vector<RowLaunch>& v) {
  using namespace cellreg;
  add_shapes<SD3Q19, float, COLL_BGK, 4, 16, false, false>(v, L_COLL_BGK);
  add_shapes<SD3Q19, double, COLL_BGK, 4, 16, false, false>(v, L_COLL_BGK);
  add_shapes<SD3Q19, double, COLL_BGK, 4, 16, true, false>(v, L_COLL_BGK);  // z sharing
  // the KBC collision needs 170-255 registers: 2 or 3 CTAs of 4 warps per SM
  v.push_back(centry<SD3Q27, float, COLL_KBC, 3, 32, 4, 2, false, false, false>(L_COLL_KBC));
  v.push_back(centry<SD3Q27, float, COLL_KBC, 3, 32, 4, 3, false, false, false>(L_COLL_KBC));
}

}  // namespace natgpu
