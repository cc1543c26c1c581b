// Fused semi-Lagrangian stream + collide, row-group kernel.
//
// The row kernel (sl_row.cuh) gives each warp a 32-node x segment and
// computes the y/z-factored values of the segment's x-window halo itself:
// BW = 32 + PER + P + 1 > 32 positions, i.e. two full warp passes per
// direction with an x component for ~1.3 passes of useful work, and a
// partially filled last segment whenever nx is not a multiple of 32.
//
// Here G warps (32 G >= nx) own a whole periodic x row.  Every lane
// computes the y/z-factored value at its own x exactly once; the lanes near
// the two ends also store it at its periodic image, so the row buffer holds
// [-PER, nx + P] and no halo is ever recomputed.  A named barrier of the G
// warps orders the buffer writes before the x-window reads (one per
// direction with an x component; two alternating buffers).  A CTA holds R
// such rows (consecutive y, same z).  The streamed values live in shared
// memory (as the SS row kernel) so that 64 registers per thread suffice.
//
// Host-checked requirements: 32 (G - 1) < nx <= 32 G, nx >= PER + P + 1,
// ny a multiple of R.
#pragma once

#include <cuda_runtime.h>

#include "collision.cuh"
#include "natgpu_common.h"
#include "sl_row.cuh"
#include "stencils.cuh"

namespace natgpu {

__device__ __forceinline__ void named_barrier(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(nthreads) : "memory");
}

template <class S, class Real, int COLL, int P, bool DG, int G, int R, int MINB>
__global__ void __launch_bounds__(32 * G * R, MINB) k_sl_rowg(const __grid_constant__ RowParams<Real> prm) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q;
  constexpr int PER = Geo<P, DG>::PER;
  constexpr int HL = PER;     // left reach of a window
  constexpr int HR = P + 1;   // right reach
  constexpr int RBW = 32 * G + HL + HR;
  constexpr int NW = G * R;
  using Tab = const Real (*)[2][PER][P + 1];
  __shared__ Real rowbuf[R][2][RBW];
  __shared__ Real fs_sh[NW][Q * 32];
  __shared__ Real swt[row_table_size<P, DG>()];
  fill_row_table<Real, P, DG>(swt, prm.W.w, threadIdx.x, 32 * NW);
  __syncthreads();
  Tab sw = reinterpret_cast<Tab>(swt);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = warp / G;
  const int xi = (warp % G) * 32 + lane;
  const int nx = prm.nx, ny = prm.ny, nz = prm.nz;
  const int by = blockIdx.x % (ny / R);
  const int z = blockIdx.x / (ny / R);
  const int y = by * R + r;
  const bool valid = xi < nx;
  const int x = valid ? xi : 0;
  const int nxy = nx * ny;
  const int node = z * nxy + y * nx + x;
  const int cx = x % PER, cy = y % PER, cz = z % PER;
  Real* fs_s = fs_sh[warp];
  fs_s[lane] = valid ? prm.f_in[node] : Real(0);

  static_for<1, Q>([&](auto I) {
    constexpr int A = decltype(I)::value;
    constexpr int sx = S::e(A, 0), sy = S::e(A, 1), sz = S::D == 3 ? S::e(A, 2) : 0;
    constexpr int NJY = sy != 0 ? P + 1 : 1;
    constexpr int NJZ = sz != 0 ? P + 1 : 1;
    constexpr int dy = sy > 0 ? 0 : 1, dz = sz > 0 ? 0 : 1, dx = sx > 0 ? 0 : 1;
    (void)dz;
    (void)dy;
    (void)dx;
    const Real* __restrict__ src = prm.f_in + (long long)A * prm.n;
    int ys = y, zs = z, j0y = 0, j0z = 0;
    if constexpr (sy != 0) {
      ys = win_start<P, DG, sy>(y, cy);
      j0y = win_j0<P, DG, sy>(cy);
    }
    if constexpr (sz != 0) {
      zs = win_start<P, DG, sz>(z, cz);
      j0z = win_j0<P, DG, sz>(cz);
    }
    // y/z-factored value at x position gx (rotated window order: slot 0 is
    // the dominant row)
    auto yz = [&](int gx) -> Real {
      Real zv[P + 1];
#pragma unroll
      for (int jz = 0; jz < NJZ; ++jz) {
        const int rz = j0z + jz;
        const int gz = wrap(zs + (rz > P ? rz - (P + 1) : rz), nz);
        Real yv[P + 1];
#pragma unroll
        for (int jy = 0; jy < NJY; ++jy) {
          const int ry = j0y + jy;
          const int gy = wrap(ys + (ry > P ? ry - (P + 1) : ry), ny);
          yv[jy] = __ldg(src + gz * nxy + gy * nx + gx);
        }
        if constexpr (sy != 0)
          zv[jz] = wsum<DEV, P>(sw[1][dy][cy], yv);
        else
          zv[jz] = yv[0];
      }
      if constexpr (sz != 0)
        return wsum<DEV, P>(sw[2][dz][cz], zv);
      else
        return zv[0];
    };
    Real out;
    if constexpr (sx == 0) {
      out = yz(x);
    } else {
      Real* buf = &rowbuf[r][xorder<S>(A) & 1][0];
      if (valid) {
        const Real v = yz(x);
        buf[HL + x] = v;
        if (x < HR) buf[HL + nx + x] = v;        // periodic image right of the row
        if (x >= nx - HL) buf[HL + x - nx] = v;  // periodic image left of the row
      }
      named_barrier(1 + r, 32 * G);
      const int st = HL + win_start<P, DG, sx>(x, cx);
      Real xv[P + 1];
#pragma unroll
      for (int j = 0; j <= P; ++j) xv[j] = buf[st + j];
      out = wsum_j0<DEV, P>(sw[0][dx][cx], xv, win_j0<P, DG, sx>(cx));
    }
    fs_s[A * 32 + lane] = out;
  });

  if (!valid) return;
  RowArgs<Real> a;
  a.f_in = prm.f_in;
  a.f_out = prm.f_out;
  a.rho = prm.rho;
  a.u = prm.u;
  a.status = prm.status;
  a.n = prm.n;
  a.nx = nx;
  a.ny = ny;
  a.nz = nz;
  a.tau = prm.tau;
  a.scaling = prm.scaling;
  a.write_macro = prm.write_macro;
  row_collide<S, Real, COLL>(a, fs_s, node, lane);
}

}  // namespace natgpu
