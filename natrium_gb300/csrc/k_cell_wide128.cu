// Cell-row kernel instantiations for x rows of 128 cells (four warps per
// row): D3Q19 p = 4 DG (FP32 deviation, FP64) and FE_Q (FP32), D3Q27 p = 3
// DG KBC (FP32).
#include "k_cell.h"

namespace natgpu {

void cell_kernels_wide128(std::vector<RowLaunch>& v) {
  using namespace cellreg;
  add_shapes_128<SD3Q19, float, COLL_BGK, 4>(v, L_COLL_BGK);
  add_shapes_128<SD3Q19, double, COLL_BGK, 4>(v, L_COLL_BGK);
  add_shapes_128<SD3Q19, float, COLL_BGK, 4, false>(v, L_COLL_BGK);
  add_shapes_128<SD3Q27, float, COLL_KBC, 3>(v, L_COLL_KBC);
}

}  // namespace natgpu
