// Cell-row kernel (sl_cell.cuh) instantiations: DG topology, one lane per
// cell row of P + 1 nodes, a warp per 32 / L whole x rows of L cells.
#include "launch.h"
#include "sl_cell.cuh"

namespace natgpu {

namespace {

template <class S, class Real, int COLL, int P, int L, int WARPS, int MINB>
RowLaunch centry(int coll) {
  RowLaunch e;
  e.stencil = S::ID;
  e.coll = coll;
  e.prec = sizeof(Real) == 8 ? 0 : 1;
  e.P = P;
  e.dg = true;
  e.wy = WARPS * (32 / L);  // rows per CTA
  e.wz = 1;
  e.kind = 11;
  e.g = L;                  // cells per x row: nx = L (P + 1)
  e.warps = WARPS;
  e.smem = (size_t)WARPS * cell_smem_per_warp<S, Real, P>();
  e.fn = (const void*)&k_sl_cell<S, Real, COLL, P, L, WARPS, MINB>;
  return e;
}

template <class S, class Real, int COLL, int P, int L>
void add_shapes(std::vector<RowLaunch>& v, int coll) {
  constexpr size_t per_warp = cell_smem_per_warp<S, Real, P>();
  // CTAs of 4 warps per SM within ~220 KB of shared memory; the same
  // register cap with CTAs of 2 warps; and one CTA fewer per SM (more
  // registers per thread, fewer spills)
  constexpr int M4 = (int)(220000 / (4 * per_warp)) > 0 ? (int)(220000 / (4 * per_warp)) : 1;
  constexpr int M4C = M4 > 8 ? 8 : M4;
  v.push_back(centry<S, Real, COLL, P, L, 4, M4C>(coll));
  v.push_back(centry<S, Real, COLL, P, L, 2, 2 * M4C>(coll));
  if constexpr (M4C > 1) v.push_back(centry<S, Real, COLL, P, L, 4, M4C - 1>(coll));
}

}  // namespace

void cell_kernels(std::vector<RowLaunch>& v) {
  // D3Q27, p = 3 (4 nodes per cell row, float4 / 2 x double2 loads)
  add_shapes<SD3Q27, float, COLL_KBC, 3, 32>(v, L_COLL_KBC);
  add_shapes<SD3Q27, float, COLL_KBC, 3, 16>(v, L_COLL_KBC);
  add_shapes<SD3Q27, float, COLL_BGK, 3, 32>(v, L_COLL_BGK);
  add_shapes<SD3Q27, float, COLL_BGK, 3, 16>(v, L_COLL_BGK);
  add_shapes<SD3Q27, double, COLL_KBC, 3, 32>(v, L_COLL_KBC);
  add_shapes<SD3Q27, double, COLL_BGK, 3, 32>(v, L_COLL_BGK);
  // D3Q19, p = 4 (5 nodes per cell row) and p = 3
  add_shapes<SD3Q19, float, COLL_BGK, 4, 16>(v, L_COLL_BGK);
  add_shapes<SD3Q19, double, COLL_BGK, 4, 16>(v, L_COLL_BGK);
  add_shapes<SD3Q19, float, COLL_BGK, 3, 32>(v, L_COLL_BGK);
  add_shapes<SD3Q19, float, COLL_BGK, 3, 16>(v, L_COLL_BGK);
}

}  // namespace natgpu
