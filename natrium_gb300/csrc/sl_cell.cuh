// Fused semi-Lagrangian stream + collide, cell-row kernel (DG topology).
//
// A lane owns one cell's PER = P + 1 nodes along x at a fixed (y, z): a
// "cell row".  A warp owns RPW whole periodic x rows (the row has L = nx /
// PER cells, RPW = 32 / L), so the x factor needs no halo: the neighbouring
// cell's values come from the neighbouring lane by a warp shuffle, which
// wraps the periodic row.
//
// Phase 1, per direction alpha with displacement signs (sx, sy, sz):
//   * the (p+1)^k source rows of the y/z window are loaded one cell row at a
//     time -- PER consecutive values, a vector load (float4 / 2 x double2 for
//     PER = 4) -- in the rotated order whose slot 0 is the dominant row, and
//     summed per node with the row-uniform y and z weights (sum
//     factorisation: y within each z row, then z, as running sums);
//   * if sx != 0, the x factor: classes whose departure point stays in the
//     node's own cell take the lane's own PER values, the one class that
//     leaves it (class 0 for sx > 0, class P for sx < 0) takes the
//     neighbouring lane's; the class and the window are compile-time, so the
//     x weights are read straight from the kernel's constant bank;
//   * the PER streamed values go to the warp's shared array S[alpha][32 PER].
// Phase 2: the warp collides its 32 PER nodes, lane l taking nodes l, l + 32,
// ... of the array (conflict-free shared reads), and writes f once,
// coalesced.  No CTA-wide barrier after the weight table: each warp only
// reads what it wrote.
//
// Compared with the row kernel (sl_row.cuh), one load instruction brings
// PER values, the row offsets are computed once per cell row instead of per
// node, and the x window costs shuffles instead of a shared-memory round
// trip with a halo.
//
// In the FP32 deviation mode a window sum is v_j0 + sum_{j != j0} w_j (v_j -
// v_j0), j0 the source node at the destination's own position (as in
// sl_row.cuh, in the same order of operations): constant fields are
// reproduced exactly.  Same operator, tables and window pattern as the row
// kernel: every departure point lies in the node's own cell or the adjacent
// upwind cell (checked on the host).
#pragma once

#include <cuda_runtime.h>

#include "collision.cuh"
#include "natgpu_common.h"
#include "sl_row.cuh"
#include "stencils.cuh"

namespace natgpu {

// PER consecutive values at p (aligned to PER * sizeof(Real) when that is 16
// or 32 bytes)
template <int PER, class Real>
__device__ __forceinline__ void load_cell(const Real* __restrict__ p, Real (&v)[PER]) {
  if constexpr (sizeof(Real) == 4 && PER == 4) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
  } else if constexpr (sizeof(Real) == 8 && PER == 4) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
  } else {
#pragma unroll
    for (int c = 0; c < PER; ++c) v[c] = __ldg(p + c);
  }
}

template <int PER, class Real>
__device__ __forceinline__ void store_cell(Real* p, const Real (&v)[PER]) {
  if constexpr (sizeof(Real) == 4 && PER == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  } else if constexpr (sizeof(Real) == 8 && PER == 4) {
    reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
  } else {
#pragma unroll
    for (int c = 0; c < PER; ++c) p[c] = v[c];
  }
}

// window sum with a compile-time dominant slot J0 over the natural order
// (x factor): v_J0 + sum_{j != J0} w_j (v_j - v_J0) in the deviation mode
template <bool DEV, int P, int J0, class Real>
__device__ __forceinline__ Real wsum_fixed(const Real (&w)[P + 1], const Real (&v)[P + 1]) {
  if constexpr (DEV) {
    Real acc = Real(0);
#pragma unroll
    for (int j = 0; j <= P; ++j)
      if (j != J0) acc = fma(w[j], v[j] - v[J0], acc);
    return acc + v[J0];
  } else {
    Real acc = w[0] * v[0];
#pragma unroll
    for (int j = 1; j <= P; ++j) acc = fma(w[j], v[j], acc);
    return acc;
  }
}

// Shared memory per warp: Q * 32 * PER values.
template <class S, class Real, int P>
__host__ __device__ constexpr size_t cell_smem_per_warp() {
  return (size_t)S::Q * 32 * (P + 1) * sizeof(Real);
}

// CTA: WARPS warps, each owning RPW = 32 / L consecutive x rows (y, z); the
// CTA covers WARPS * RPW rows of one z.  Requires nx = L (P + 1) (DG), ny a
// multiple of WARPS * RPW.
template <class S, class Real, int COLL, int P, int L, int WARPS, int MINB>
__global__ void __launch_bounds__(32 * WARPS, MINB) k_sl_cell(const __grid_constant__ RowParams<Real> prm) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q;
  constexpr int PER = P + 1;
  constexpr int RPW = 32 / L;
  constexpr int NPW = 32 * PER;  // nodes per warp
  static_assert(L * RPW == 32 && (L & (L - 1)) == 0, "L must be a power of two dividing 32");
  extern __shared__ __align__(16) unsigned char cell_smem[];
  __shared__ Real sw[row_table_size<P, true>()];
  fill_row_table<Real, P, true>(sw, prm.W.w, threadIdx.x, 32 * WARPS);
  __syncthreads();
  using Tab = const Real (*)[2][PER][P + 1];
  Tab tw = reinterpret_cast<Tab>(sw);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Real* Sw = reinterpret_cast<Real*>(cell_smem) + (size_t)warp * Q * NPW;
  const int nx = prm.nx, ny = prm.ny, nz = prm.nz;
  const int nxy = nx * ny;
  const int rows_per_cta = WARPS * RPW;
  const int by = blockIdx.x % (ny / rows_per_cta);
  const int z = blockIdx.x / (ny / rows_per_cta);
  const int r = lane / L;  // row of this lane within the warp
  const int X = lane % L;  // cell along x
  const int y = by * rows_per_cta + warp * RPW + r;
  const int cy = y % PER, cz = z % PER;
  const int x0 = X * PER;

  // rest population: copied
  {
    Real v[PER];
    load_cell<PER>(prm.f_in + (size_t)z * nxy + (size_t)y * nx + x0, v);
    store_cell<PER>(Sw + lane * PER, v);
  }

  static_for<1, Q>([&](auto I) {
    constexpr int A = decltype(I)::value;
    constexpr int sx = S::e(A, 0), sy = S::e(A, 1), sz = S::D == 3 ? S::e(A, 2) : 0;
    constexpr int NJY = sy != 0 ? P + 1 : 1;
    constexpr int NJZ = sz != 0 ? P + 1 : 1;
    constexpr int dy = sy > 0 ? 0 : 1, dz = sz > 0 ? 0 : 1, dx = sx > 0 ? 0 : 1;
    const Real* __restrict__ src = prm.f_in + ((size_t)A * prm.n + x0);  // + 32-bit row offsets
    int ys = y, zs = z, j0y = 0, j0z = 0;
    if constexpr (sy != 0) {
      ys = win_start<P, true, sy>(y, cy);
      j0y = win_j0<P, true, sy>(cy);
    }
    if constexpr (sz != 0) {
      zs = win_start<P, true, sz>(z, cz);
      j0z = win_j0<P, true, sz>(cz);
    }
    (void)dy;
    (void)dz;
    // y/z factors: T[c] for the lane's PER nodes.  The z rows are taken in
    // the rotated order (slot 0 the dominant one) and accumulated one at a
    // time: T = Y_0 + sum_{jz >= 1} w_jz (Y_jz - Y_0) in the deviation mode
    // (Y_jz the y-factored value of z row jz), so only Y_0 and the sum stay
    // live; the y factor is accumulated the same way.
    Real T[PER];
    {
      Real Y0[PER], acc[PER];
#pragma unroll
      for (int jz = 0; jz < NJZ; ++jz) {
        const int rz = j0z + jz;
        const int gz = wrap(zs + (rz > P ? rz - (P + 1) : rz), nz);
        Real Y[PER];
        if constexpr (sy != 0) {
          Real y0v[PER], yacc[PER];
#pragma unroll
          for (int jy = 0; jy < NJY; ++jy) {
            const int ry = j0y + jy;
            const int gy = wrap(ys + (ry > P ? ry - (P + 1) : ry), ny);
            Real v[PER];
            load_cell<PER>(src + (gz * nxy + gy * nx), v);
            const Real wy = tw[1][dy][cy][jy];
#pragma unroll
            for (int c = 0; c < PER; ++c) {
              if (jy == 0) {
                y0v[c] = v[c];
                yacc[c] = DEV ? Real(0) : wy * v[c];
              } else {
                yacc[c] = DEV ? fma(wy, v[c] - y0v[c], yacc[c]) : fma(wy, v[c], yacc[c]);
              }
            }
          }
#pragma unroll
          for (int c = 0; c < PER; ++c) Y[c] = DEV ? yacc[c] + y0v[c] : yacc[c];
        } else {
          load_cell<PER>(src + (gz * nxy + ys * nx), Y);
        }
        if constexpr (sz != 0) {
          const Real wz = tw[2][dz][cz][jz];
#pragma unroll
          for (int c = 0; c < PER; ++c) {
            if (jz == 0) {
              Y0[c] = Y[c];
              acc[c] = DEV ? Real(0) : wz * Y[c];
            } else {
              acc[c] = DEV ? fma(wz, Y[c] - Y0[c], acc[c]) : fma(wz, Y[c], acc[c]);
            }
          }
        } else {
#pragma unroll
          for (int c = 0; c < PER; ++c) Y0[c] = Y[c];
        }
      }
#pragma unroll
      for (int c = 0; c < PER; ++c) T[c] = sz != 0 ? (DEV ? acc[c] + Y0[c] : acc[c]) : Y0[c];
    }
    Real out[PER];
    if constexpr (sx == 0) {
#pragma unroll
      for (int c = 0; c < PER; ++c) out[c] = T[c];
    } else {
      // the neighbouring cell along -sx (periodic within the row)
      const int nb = sx > 0 ? (X + L - 1) % L : (X + 1) % L;
      Real U[PER];
#pragma unroll
      for (int c = 0; c < PER; ++c) U[c] = __shfl_sync(0xffffffffu, T[c], r * L + nb);
      static_for<0, PER>([&](auto C) {
        constexpr int c = decltype(C)::value;
        Real w[P + 1];
#pragma unroll
        for (int j = 0; j <= P; ++j) w[j] = prm.W.w[0][dx][c][j];
        constexpr bool other = sx > 0 ? (c == 0) : (c == P);
        if constexpr (other) {
          // window = the neighbouring cell, dominant its nearest node
          constexpr int J0 = sx > 0 ? P : 0;
          out[c] = wsum_fixed<DEV, P, J0>(w, U);
        } else {
          out[c] = wsum_fixed<DEV, P, c>(w, T);
        }
      });
    }
    store_cell<PER>(Sw + (size_t)A * NPW + lane * PER, out);
  });
  __syncwarp();

  // phase 2: collide the warp's nodes, lane-strided
  const int row0 = by * rows_per_cta + warp * RPW;
#pragma unroll 1
  for (int k = 0; k < PER; ++k) {
    const int t = lane + 32 * k;  // node within the warp's rows
    const int rr = t / nx, xx = t % nx;
    const int node = z * nxy + (row0 + rr) * nx + xx;
    Real fs[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) fs[q] = Sw[(size_t)q * NPW + t];
    Real u[3] = {0, 0, 0};
    Real rho = Real(1);
    if constexpr (COLL == COLL_BGK) {
      rho = collide_bgk<S, DEV, false>(fs, Real(1) / Real(prm.tau), u, false);
    } else if constexpr (COLL == COLL_KBC) {
      rho = collide_kbc<S, DEV, false>(fs, Real(prm.tau), u, false);
    }
    if constexpr (DEV && COLL != COLL_NONE) {
      // the pre-collision values are read back from the warp's array (not
      // held in registers through the collision)
      Real pre[Q];
#pragma unroll
      for (int q = 0; q < Q; ++q) pre[q] = Sw[(size_t)q * NPW + t];
      conserve<S>(fs, pre);
    }
    if constexpr (COLL != COLL_NONE) {
      int bad = 0;
      if (!(rho >= Real(1e-10))) bad |= (rho != rho) ? ST_NAN : ST_DENSITY;
      if (prm.write_macro) {
        prm.rho[node] = (double)rho;
        prm.u[node] = (double)u[0] * prm.scaling;
        prm.u[prm.n + node] = (double)u[1] * prm.scaling;
        if constexpr (S::D == 3) prm.u[2 * prm.n + node] = (double)u[2] * prm.scaling;
      }
      if (bad) atomicOr(prm.status, bad);
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) prm.f_out[(size_t)q * prm.n + node] = fs[q];
  }
}

}  // namespace natgpu
