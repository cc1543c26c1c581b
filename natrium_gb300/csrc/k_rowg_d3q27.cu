// Row-group kernel (sl_rowg.cuh) instantiations: D3Q27, FP32 deviation.
#include "launch.h"
#include "sl_rowg.cuh"

namespace natgpu {

namespace {

template <class S, int COLL, int P, bool DG, int G, int R>
RowLaunch gentry(int coll) {
  // registers per thread: 64 up to P = 2, 80 above (fewer spills in the collision)
  constexpr int MINB = 65536 / ((P <= 2 ? 64 : 80) * 32 * G * R);
  RowLaunch e;
  e.stencil = S::ID;
  e.coll = coll;
  e.prec = 1;
  e.P = P;
  e.dg = DG;
  e.wy = R;
  e.wz = 1;
  e.fn = (const void*)&k_sl_rowg<S, float, COLL, P, DG, G, R, MINB>;
  e.kind = 7;
  e.g = G;
  e.min_nx = Geo<P, DG>::PER + P + 1;
  return e;
}

template <class S, int COLL, int P>
void add_orders(std::vector<RowLaunch>& t, int coll) {
  t.push_back(gentry<S, COLL, P, true, 2, 4>(coll));
  t.push_back(gentry<S, COLL, P, false, 2, 4>(coll));
  t.push_back(gentry<S, COLL, P, true, 3, 2>(coll));
  t.push_back(gentry<S, COLL, P, false, 3, 2>(coll));
  t.push_back(gentry<S, COLL, P, true, 4, 2>(coll));
  t.push_back(gentry<S, COLL, P, false, 4, 2>(coll));
  if constexpr (P < PMAX) add_orders<S, COLL, P + 1>(t, coll);
}

}  // namespace

void rowg_kernels_d3q27(std::vector<RowLaunch>& v) {
  add_orders<SD3Q27, COLL_BGK, 1>(v, L_COLL_BGK);
  add_orders<SD3Q27, COLL_KBC, 1>(v, L_COLL_KBC);
}

}  // namespace natgpu
