// Cell-row kernel (sl_cell.cuh) registration helpers: one RowLaunch per
// instantiation, included by the k_cell_*.cu units (one stencil and precision
// each, compiled in parallel).
#pragma once
#include "launch.h"
#include "sl_cell.cuh"

namespace natgpu {
namespace cellreg {
template <class S, class Real, int COLL, int P, int L, int WARPS, int MINB, bool MMA = false, bool ZS = false,
          bool DG = true>
RowLaunch centry(int coll) {
  RowLaunch e;
  e.stencil = S::ID;
  e.coll = coll;
  e.prec = sizeof(Real) == 8 ? 0 : 1;
  e.P = P;
  e.dg = DG;
  e.wy = L > 32 ? WARPS / (L / 32) : WARPS * (32 / L);  // rows per CTA
  e.wz = 1;
  e.kind = MMA ? 12 : (ZS ? 13 : 11);
  e.g = L;                  // cells per x row: nx = L (P + 1) in DG, L P in FE_Q
  e.warps = WARPS;
  e.smem = (size_t)WARPS * cell_smem_per_warp<S, Real, P, DG>() + (MMA ? CORNER_A_FLOATS * sizeof(float) : 0);
  e.fn = (const void*)&k_sl_cell<S, Real, COLL, P, L, WARPS, MINB, MMA, ZS, DG>;
  return e;
}

template <class S, class Real, int COLL, int P, int L, bool ZS = false, bool DG = true>
void add_shapes(std::vector<RowLaunch>& v, int coll) {
  constexpr size_t per_warp = cell_smem_per_warp<S, Real, P, DG>();
  // CTAs of 4 warps per SM within ~220 KB of shared memory; the same
  // register cap with CTAs of 2 warps; and one CTA fewer per SM (more
  // registers per thread, fewer spills)
  constexpr int M4 = (int)(220000 / (4 * per_warp)) > 0 ? (int)(220000 / (4 * per_warp)) : 1;
  constexpr int M4C = M4 > 8 ? 8 : M4;
  v.push_back(centry<S, Real, COLL, P, L, 4, M4C, false, ZS, DG>(coll));
  v.push_back(centry<S, Real, COLL, P, L, 2, 2 * M4C, false, ZS, DG>(coll));
  if constexpr (M4C > 1) v.push_back(centry<S, Real, COLL, P, L, 4, M4C - 1, false, ZS, DG>(coll));
}

// x rows of 128 cells: four warps per row, CTAs of one or two rows
template <class S, class Real, int COLL, int P, bool DG = true>
void add_shapes_128(std::vector<RowLaunch>& v, int coll) {
  constexpr size_t per_warp = cell_smem_per_warp<S, Real, P, DG>();
  constexpr int M4 = (int)(220000 / (4 * per_warp)) > 0 ? (int)(220000 / (4 * per_warp)) : 1;
  constexpr int M4C = M4 > 8 ? 8 : M4;
  constexpr int M8 = (int)(220000 / (8 * per_warp)) > 0 ? (int)(220000 / (8 * per_warp)) : 1;
  constexpr int M8C = M8 > 4 ? 4 : M8;
  v.push_back(centry<S, Real, COLL, P, 128, 4, M4C, false, false, DG>(coll));
  v.push_back(centry<S, Real, COLL, P, 128, 8, M8C, false, false, DG>(coll));
  if constexpr (M4C > 1) v.push_back(centry<S, Real, COLL, P, 128, 4, M4C - 1, false, false, DG>(coll));
}

}  // namespace cellreg

void cell_kernels_q27f(std::vector<RowLaunch>& v);
void cell_kernels_q27fz(std::vector<RowLaunch>& v);
void cell_kernels_q27d(std::vector<RowLaunch>& v);
void cell_kernels_q19f(std::vector<RowLaunch>& v);
void cell_kernels_q19d(std::vector<RowLaunch>& v);
void cell_kernels_q19feq(std::vector<RowLaunch>& v);
void cell_kernels_wide(std::vector<RowLaunch>& v);
void cell_kernels_wide128(std::vector<RowLaunch>& v);

}  // namespace natgpu
