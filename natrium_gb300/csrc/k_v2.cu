// Instantiations of the specialised fused kernel (sl_step_v2.cuh) and the
// lookup used by the host API.  One entry per (stencil, collision,
// precision, order, topology) with its tile shape in cells and CTA size.
#include "v2_entry.cuh"

namespace natgpu {

namespace {

const std::vector<V2Launch>& table() {
  static const std::vector<V2Launch> t = {
      // 3-D Taylor-Green, D3Q19, p = 4 (DG: 125 nodes / cell; FE_Q)
      entry<SD3Q19, float, COLL_BGK, 4, true, 4, 2, 2, 512>(L_COLL_BGK),
      entry<SD3Q19, float, COLL_BGK, 4, true, 4, 2, 1, 512>(L_COLL_BGK),
      entry<SD3Q19, float, COLL_BGK, 4, true, 4, 1, 1, 256>(L_COLL_BGK),
      entry<SD3Q19, double, COLL_BGK, 4, true, 2, 2, 1, 256>(L_COLL_BGK),
      entry<SD3Q19, float, COLL_BGK, 4, false, 4, 2, 2, 512>(L_COLL_BGK),
      entry<SD3Q19, double, COLL_BGK, 4, false, 2, 2, 2, 256>(L_COLL_BGK),
      // 3-D Taylor-Green, D3Q27, p = 3, BGK and KBC
      entry<SD3Q27, float, COLL_BGK, 3, true, 4, 2, 2, 512>(L_COLL_BGK),
      entry<SD3Q27, float, COLL_KBC, 3, true, 4, 2, 2, 512>(L_COLL_KBC),
      entry<SD3Q27, float, COLL_BGK, 3, true, 4, 2, 1, 512>(L_COLL_BGK),
      entry<SD3Q27, double, COLL_BGK, 3, true, 2, 2, 2, 256>(L_COLL_BGK),
      entry<SD3Q27, double, COLL_KBC, 3, true, 2, 2, 2, 256>(L_COLL_KBC),
  };
  return t;
}

}  // namespace

std::vector<V2Launch> find_v2(int stencil, int coll, int prec, int P, bool dg, const int cells[3], int dim,
                              int nx) {
  std::vector<V2Launch> out;
  std::vector<V2Launch> all = table();
  const std::vector<V2Launch>& more = v2_table_small_tiles();
  all.insert(all.end(), more.begin(), more.end());
  for (const V2Launch& e : all) {
    if (e.stencil != stencil || e.coll != coll || e.prec != prec || e.P != P || e.dg != dg) continue;
    bool ok = true;
    for (int a = 0; a < dim; ++a)
      if (cells[a] % e.cells[a] != 0) ok = false;
    // bulk row copies need 16-byte aligned rows
    const int al = e.prec == 0 ? 2 : 4;
    if (nx % al != 0) ok = false;
    if (ok) out.push_back(e);
  }
  return out;
}

}  // namespace natgpu
