// Small-tile instantiations of the specialised fused kernel for D3Q27, p = 3,
// FP32 deviation (BGK and KBC).  A 4 x 2 x 2-cell tile (171 KB of shared
// memory, 512 threads) leaves one CTA per SM, which then idles at each of
// its per-direction barriers; these tiles fit two (4 x 2 x 1, 2 x 2 x 2:
// 91 KB, 256 threads) or four (4 x 1 x 1: 51 KB, 128 threads) CTAs per SM,
// each at the same 128-register cap.  The autotuner picks among all.
#include "v2_entry.cuh"

namespace natgpu {

const std::vector<V2Launch>& v2_table_small_tiles() {
  static const std::vector<V2Launch> t = {
      entry<SD3Q27, float, COLL_KBC, 3, true, 4, 2, 1, 256, 2>(L_COLL_KBC),
      entry<SD3Q27, float, COLL_KBC, 3, true, 2, 2, 2, 256, 2>(L_COLL_KBC),
      entry<SD3Q27, float, COLL_KBC, 3, true, 4, 1, 1, 128, 4>(L_COLL_KBC),
      entry<SD3Q27, float, COLL_BGK, 3, true, 4, 2, 1, 256, 2>(L_COLL_BGK),
      entry<SD3Q27, float, COLL_BGK, 3, true, 4, 1, 1, 128, 4>(L_COLL_BGK),
  };
  return t;
}

}  // namespace natgpu
