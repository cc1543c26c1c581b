// Cell-row kernel instantiations: D3Q27 KBC, FP32 deviation storage, p = 3,
// with z sharing of the directions with y and z components (yz-diagonals and
// corners).
#include "k_cell.h"

namespace natgpu {

void cell_kernels_q27fz(std::vector<RowLaunch>& v) {
  using namespace cellreg;
  add_shapes<SD3Q27, float, COLL_KBC, 3, 32, true>(v, L_COLL_KBC);
  // the z-shared form needs far fewer registers: four CTAs of 4 warps per
  // SM, or CTAs of 8 warps (two y cells, fewer union rows per output row)
  v.push_back(centry<SD3Q27, float, COLL_KBC, 3, 32, 4, 4, false, true>(L_COLL_KBC));
  v.push_back(centry<SD3Q27, float, COLL_KBC, 3, 32, 8, 2, false, true>(L_COLL_KBC));
  v.push_back(centry<SD3Q27, float, COLL_KBC, 3, 32, 8, 1, false, true>(L_COLL_KBC));
}

}  // namespace natgpu
