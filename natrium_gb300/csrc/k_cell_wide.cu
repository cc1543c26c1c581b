// Cell-row kernel instantiations for x rows of 64 cells (two warps per row,
// the edge cells' values exchanged through shared memory): D3Q19 p = 4 DG
// (FP32 deviation, FP64) and FE_Q (FP32), D3Q27 p = 3 DG KBC (FP32).
#include "k_cell.h"

namespace natgpu {

void cell_kernels_wide(std::vector<RowLaunch>& v) {
  using namespace cellreg;
  add_shapes<SD3Q19, float, COLL_BGK, 4, 64>(v, L_COLL_BGK);
  add_shapes<SD3Q19, double, COLL_BGK, 4, 64>(v, L_COLL_BGK);
  add_shapes<SD3Q19, float, COLL_BGK, 4, 64, false, false>(v, L_COLL_BGK);
  add_shapes<SD3Q27, float, COLL_KBC, 3, 64>(v, L_COLL_KBC);
}

}  // namespace natgpu
