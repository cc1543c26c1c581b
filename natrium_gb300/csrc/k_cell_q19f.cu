// Cell-row kernel instantiations: D3Q19, FP32 deviation storage, p = 4 (5 nodes per cell row) and p = 3.
#include "k_cell.h"

namespace natgpu {

void cell_kernels_q19f(std::vector<RowLaunch>& v) {
  using namespace cellreg;
  add_shapes<SD3Q19, float, COLL_BGK, 4, 16>(v, L_COLL_BGK);
  add_shapes<SD3Q19, float, COLL_BGK, 4, 16, true>(v, L_COLL_BGK);
  add_shapes<SD3Q19, float, COLL_BGK, 3, 32>(v, L_COLL_BGK);
  add_shapes<SD3Q19, float, COLL_BGK, 3, 16>(v, L_COLL_BGK);
}

}  // namespace natgpu
