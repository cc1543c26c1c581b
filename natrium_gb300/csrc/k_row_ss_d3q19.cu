// Row-segment kernel (sl_row.cuh) with the streamed values in shared memory
// and 64 registers per thread (more resident warps): D3Q19, FP32 deviation.
#include "launch.h"
#include "sl_row.cuh"

namespace natgpu {

namespace {

template <class S, int COLL, int P, bool DG, int WY, int MINB, bool ZS = false>
RowLaunch sentry(int coll) {
  RowLaunch e;
  e.stencil = S::ID;
  e.coll = coll;
  e.prec = 1;
  e.P = P;
  e.dg = DG;
  e.wy = WY;
  e.wz = 1;
  e.fn = (const void*)&k_sl_row<S, float, COLL, P, DG, WY, 1, true, MINB, ZS>;
  return e;
}

template <class S, int COLL, int P>
void add_orders(std::vector<RowLaunch>& t, int coll) {
  t.push_back(sentry<S, COLL, P, true, 8, 4>(coll));
  t.push_back(sentry<S, COLL, P, false, 8, 4>(coll));
  t.push_back(sentry<S, COLL, P, true, 4, 8>(coll));
  t.push_back(sentry<S, COLL, P, false, 4, 8>(coll));
  // z sharing: two cells of rows per CTA
  constexpr int WD = 2 * (P + 1), WQ = 2 * P;
  t.push_back(sentry<S, COLL, P, true, WD, 65536 / (32 * WD * 64), true>(coll));
  t.push_back(sentry<S, COLL, P, false, WQ, 65536 / (32 * WQ * 64), true>(coll));
  if constexpr (P < PMAX) add_orders<S, COLL, P + 1>(t, coll);
}

}  // namespace

void row_ss_kernels_d3q19(std::vector<RowLaunch>& v) { add_orders<SD3Q19, COLL_BGK, 1>(v, L_COLL_BGK); }

}  // namespace natgpu
