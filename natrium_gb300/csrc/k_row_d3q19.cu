// Instantiations of the row-segment fused kernel (sl_row.cuh) for D3Q19.
#include "launch.h"
#include "sl_row.cuh"

namespace natgpu {

namespace {

template <class S, class Real, int COLL, int P, bool DG, int WY, int WZ, bool ZS = false>
RowLaunch rentry(int coll) {
  RowLaunch e;
  e.stencil = S::ID;
  e.coll = coll;
  e.prec = sizeof(Real) == 8 ? 0 : 1;
  e.P = P;
  e.dg = DG;
  e.wy = WY;
  e.wz = WZ;
  e.fn = (const void*)&k_sl_row<S, Real, COLL, P, DG, WY, WZ, false, (sizeof(Real) == 4 ? 2 : 1), ZS>;
  return e;
}

// every (stencil, collision) pair the reference supports, FE orders 1..6,
// both topologies, both precisions
template <class S, int COLL, int P>
void add_orders(std::vector<RowLaunch>& t, int coll) {
  constexpr int WY = 4, WZ = S::D == 3 ? 2 : 1;
  constexpr int WY2 = S::D == 3 ? 4 : 8;
  t.push_back(rentry<S, float, COLL, P, true, WY2, WZ>(coll));
  t.push_back(rentry<S, float, COLL, P, false, WY2, WZ>(coll));
  t.push_back(rentry<S, double, COLL, P, true, WY, WZ>(coll));
  t.push_back(rentry<S, double, COLL, P, false, WY, WZ>(coll));
  // FP64 with z sharing (a CTA of two cells of rows): the z-factored rows of
  // the yz-diagonal directions are computed once per CTA, which takes about
  // half of those directions' FP64 multiply-adds off the FP64 pipe
  t.push_back(rentry<S, double, COLL, P, true, 2 * (P + 1), 1, true>(coll));
  t.push_back(rentry<S, double, COLL, P, false, 2 * P, 1, true>(coll));
  if constexpr (P < PMAX) add_orders<S, COLL, P + 1>(t, coll);
}

}  // namespace

void row_kernels_d3q19(std::vector<RowLaunch>& v) {
  add_orders<SD3Q19, COLL_BGK, 1>(v, L_COLL_BGK);
}

}  // namespace natgpu
