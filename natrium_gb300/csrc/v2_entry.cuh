// Table entry of one instantiation of the specialised fused kernel
// (sl_step_v2.cuh): its key (stencil, collision, precision, order, topology),
// tile shape in cells and nodes, CTA size, function and shared memory.
#pragma once

#include <vector>

#include "launch.h"
#include "sl_step_v2.cuh"

namespace natgpu {

template <class S, class Real, int COLL, int P, bool DG, int CX, int CY, int CZ, int NTH, int MINB = 1>
V2Launch entry(int coll) {
  V2Launch e;
  e.stencil = S::ID;
  e.coll = coll;
  e.prec = sizeof(Real) == 8 ? 0 : 1;
  e.P = P;
  e.dg = DG;
  e.cells[0] = CX;
  e.cells[1] = CY;
  e.cells[2] = CZ;
  e.nth = NTH;
  e.fn = (const void*)&k_sl_step_v2<S, Real, COLL, P, DG, CX, CY, CZ, NTH, MINB>;
  e.smem = v2_smem_bytes<S, Real, P, DG, CX, CY, CZ>();
  using TL = Tile<S, P, DG, CX, CY, CZ, sizeof(Real)>;
  e.B[0] = TL::BX;
  e.B[1] = TL::BY;
  e.B[2] = TL::BZ;
  return e;
}

// entries of k_v2_small.cu (a translation unit of its own: the D3Q27
// instantiations take long to compile)
const std::vector<V2Launch>& v2_table_small_tiles();

}  // namespace natgpu
