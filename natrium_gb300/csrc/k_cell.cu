// Cell-row kernel (sl_cell.cuh) table: the instantiations live in the
// k_cell_*.cu units, one stencil and precision each.
#include "k_cell.h"

namespace natgpu {

void cell_kernels(std::vector<RowLaunch>& v) {
  cell_kernels_q27f(v);
  cell_kernels_q27fz(v);
  cell_kernels_q27d(v);
  cell_kernels_q19f(v);
  cell_kernels_q19d(v);
  cell_kernels_q19feq(v);
  cell_kernels_wide(v);
  cell_kernels_wide128(v);
}

}  // namespace natgpu
