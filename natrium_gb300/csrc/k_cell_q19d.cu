// Cell-row kernel instantiations: D3Q19, FP64, p = 4.
#include "k_cell.h"

namespace natgpu {

void cell_kernels_q19d(std::vector<RowLaunch>& v) {
  using namespace cellreg;
  add_shapes<SD3Q19, double, COLL_BGK, 4, 16>(v, L_COLL_BGK);
  add_shapes<SD3Q19, double, COLL_BGK, 4, 16, true>(v, L_COLL_BGK);
}

}  // namespace natgpu
