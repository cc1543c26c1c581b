// Instantiations of the bulk-copy row-segment kernel (sl_rowt.cuh): D3Q19.
#include "launch.h"
#include "sl_rowt.cuh"

namespace natgpu {

namespace {

template <class S, class Real, int COLL, int P, bool DG, int WY, int WZ>
RowLaunch tentry(int coll) {
  RowLaunch e;
  e.stencil = S::ID;
  e.coll = coll;
  e.prec = sizeof(Real) == 8 ? 0 : 1;
  e.P = P;
  e.dg = DG;
  e.wy = WY;
  e.wz = WZ;
  e.fn = (const void*)&k_sl_rowt<S, Real, COLL, P, DG, WY, WZ>;
  e.kind = 6;
  e.smem = rowt_smem_bytes<S, Real, P, DG, WY, WZ>();
  e.align = 16 / (int)sizeof(Real);
  e.min_nx = RowtGeo<S, P, DG, sizeof(Real)>::XW;
  return e;
}

template <class S, int COLL, int P, int PMAXI>
void add_orders(std::vector<RowLaunch>& t, int coll) {
  t.push_back(tentry<S, float, COLL, P, true, 4, 2>(coll));
  t.push_back(tentry<S, float, COLL, P, false, 4, 2>(coll));
  t.push_back(tentry<S, double, COLL, P, true, 4, 2>(coll));
  t.push_back(tentry<S, double, COLL, P, false, 4, 2>(coll));
  if constexpr (P < PMAXI) add_orders<S, COLL, P + 1, PMAXI>(t, coll);
}

}  // namespace

void rowt_kernels_d3q19(std::vector<RowLaunch>& v) {
  add_orders<SD3Q19, COLL_BGK, 1, PMAX>(v, L_COLL_BGK);
}

}  // namespace natgpu
