// Cell-row kernel instantiations: D3Q27, FP32 deviation storage, p = 3 (4 nodes per cell row, float4 loads).
#include "k_cell.h"

namespace natgpu {

void cell_kernels_q27f(std::vector<RowLaunch>& v) {
  using namespace cellreg;
  add_shapes<SD3Q27, float, COLL_KBC, 3, 32>(v, L_COLL_KBC);
  add_shapes<SD3Q27, float, COLL_KBC, 3, 16>(v, L_COLL_KBC);
  add_shapes<SD3Q27, float, COLL_BGK, 3, 32>(v, L_COLL_BGK);
  add_shapes<SD3Q27, float, COLL_BGK, 3, 16>(v, L_COLL_BGK);
  // the same with the 8 corner directions as tf32x3 tensor-core tiles (a CTA
  // is one y cell of one z row: 4 warps of one x row of 32 cells)
  v.push_back(centry<SD3Q27, float, COLL_KBC, 3, 32, 4, 2, true>(L_COLL_KBC));
  v.push_back(centry<SD3Q27, float, COLL_BGK, 3, 32, 4, 2, true>(L_COLL_BGK));
}

}  // namespace natgpu
