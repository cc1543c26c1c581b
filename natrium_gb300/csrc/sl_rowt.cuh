// Fused semi-Lagrangian stream + collide, row-segment kernel with a
// per-warp bulk-copy pipeline.
//
// Same work decomposition, operator and arithmetic as the row kernel
// (sl_row.cuh): one warp owns 32 consecutive x-nodes of one (y, z) row and
// keeps all Q streamed values of its nodes in registers.  What changes is
// how the source rows reach the warp.  The row kernel loads them with
// per-lane global loads, and its warps spend most of their time waiting on
// those loads.  Here every warp runs its own three-stage pipeline of
// cp.async.bulk row copies (one copy per source row of a direction's
// window, issued by the lanes, completed on a per-stage mbarrier): while
// direction A is computed from shared memory, the rows of A+1 and A+2 are
// already in flight.  All window reads are then shared-memory reads at
// compile-time offsets; the warp never synchronises with other warps after
// the set-up.
//
// Rows of a direction with an x component cover the 16-byte aligned
// segment around [x0 - PER, x0 + 32 + P] (periodic, at most two pieces);
// rows without one cover [x0, x0 + 32).  Requirements checked on the host:
// nx a multiple of 16 bytes / sizeof(Real) (aligned row starts) and nx at
// least one x row's width (at most two pieces per row).
//
// Every wait on an mbarrier is bounded (MBAR_MAX_POLLS); when one runs
// out the warp sets ST_TIMEOUT, waits (bounded) for the copies it still has
// in flight and stops.
#pragma once

#include <cuda_runtime.h>

#include "collision.cuh"
#include "natgpu_common.h"
#include "sl_row.cuh"
#include "sl_step_v2.cuh"
#include "stencils.cuh"

namespace natgpu {

constexpr int RT_NST = 3;  // pipeline stages per warp

template <class S, int P, bool DG, int ES>
struct RowtGeo {
  static constexpr int PER = Geo<P, DG>::PER;
  static constexpr int HL = PER;                 // left halo of the x buffer
  static constexpr int BW = 32 + PER + P + 1;    // x buffer width (as sl_row.cuh)
  static constexpr int AL = 16 / ES;             // elements per 16 bytes
  static constexpr int XS = Geo<P, DG>::fl(-HL, AL);           // copy start relative to x0
  static constexpr int XC = -HL - XS;                          // column of x0 - HL in a copied row
  static constexpr int XW = Geo<P, DG>::ce(-HL + BW, AL) - XS;  // width of a row with x component
  static constexpr int NW = 32;                                // width of a row without
  // rows of a direction and its row width
  static constexpr int rows(int A) {
    return (S::e(A, 1) != 0 ? P + 1 : 1) * (S::D == 3 && S::e(A, 2) != 0 ? P + 1 : 1);
  }
  static constexpr int width(int A) { return S::e(A, 0) != 0 ? XW : NW; }
  static constexpr int stage() {
    int m = 0;
    for (int A = 1; A < S::Q; ++A) m = rows(A) * width(A) > m ? rows(A) * width(A) : m;
    return m;
  }
};

template <class S, class Real, int P, bool DG, int WY, int WZ>
struct RowtSmem {
  using RG = RowtGeo<S, P, DG, sizeof(Real)>;
  static constexpr int NWARP = WY * WZ;
  static constexpr size_t al(size_t x) { return (x + 127) & ~size_t(127); }
  static constexpr size_t BARS = 0;
  static constexpr size_t TAB = al(BARS + sizeof(unsigned long long) * NWARP * RT_NST);
  static constexpr size_t XBUF = al(TAB + sizeof(Real) * row_table_size<P, DG>());
  static constexpr size_t STG = al(XBUF + sizeof(Real) * NWARP * 2 * (RG::BW + 1));
  static constexpr size_t TOTAL = al(STG + sizeof(Real) * (size_t)NWARP * RT_NST * RG::stage());
};

template <class S, class Real, int P, bool DG, int WY, int WZ>
constexpr size_t rowt_smem_bytes() {
  return RowtSmem<S, Real, P, DG, WY, WZ>::TOTAL;
}

// Issue the row copies of direction A into stage buffer dst (called by the
// whole warp; lane 0 arms the barrier first).
template <class S, class Real, int P, bool DG, int A>
__device__ __forceinline__ void rowt_issue(const Real* __restrict__ f_in, long long n, Real* dst,
                                           unsigned long long* bar, int x0, int y, int z, int nx, int ny,
                                           int nz, int lane) {
  using RG = RowtGeo<S, P, DG, sizeof(Real)>;
  constexpr int PER = RG::PER;
  constexpr int sx = S::e(A, 0), sy = S::e(A, 1), sz = S::D == 3 ? S::e(A, 2) : 0;
  constexpr int NY = sy != 0 ? P + 1 : 1;
  constexpr int ROWS = RG::rows(A);
  constexpr bool XD = sx != 0;
  const int W = XD ? RG::XW : min(RG::NW, nx - x0);
  if (lane == 0) mbar_expect_tx(bar, (unsigned)(ROWS * W * (int)sizeof(Real)));
  __syncwarp();
  for (int r = lane; r < ROWS; r += 32) {
    const int jz = r / NY, jy = r % NY;
    int gy = y, gz = z;
    // rotated window order: slot 0 is the row of the dominant weight
    if constexpr (sy != 0) {
      const int cy = y % PER;
      const int ry = win_j0<P, DG, sy>(cy) + jy;
      gy = wrap(win_start<P, DG, sy>(y, cy) + (ry > P ? ry - (P + 1) : ry), ny);
    }
    if constexpr (sz != 0) {
      const int cz = z % PER;
      const int rz = win_j0<P, DG, sz>(cz) + jz;
      gz = wrap(win_start<P, DG, sz>(z, cz) + (rz > P ? rz - (P + 1) : rz), nz);
    }
    (void)jz;
    const Real* row = f_in + (long long)A * n + ((long long)gz * ny + gy) * nx;
    Real* d = dst + r * RG::width(A);
    if constexpr (XD) {
      int pos = x0 + RG::XS;
      pos += pos < 0 ? nx : 0;
      const int l1 = min(RG::XW, nx - pos);
      bulk_copy(d, row + pos, (unsigned)(l1 * (int)sizeof(Real)), bar);
      if (l1 < RG::XW) bulk_copy(d + l1, row, (unsigned)((RG::XW - l1) * (int)sizeof(Real)), bar);
    } else {
      bulk_copy(d, row + x0, (unsigned)(W * (int)sizeof(Real)), bar);
    }
  }
}

template <class S, class Real, int COLL, int P, bool DG, int WY, int WZ>
__global__ void __launch_bounds__(32 * WY * WZ, (sizeof(Real) == 4 ? 2 : 1))
    k_sl_rowt(const __grid_constant__ RowParams<Real> prm) {
  using RG = RowtGeo<S, P, DG, sizeof(Real)>;
  using SM = RowtSmem<S, Real, P, DG, WY, WZ>;
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q;
  constexpr int PER = RG::PER, HL = RG::HL, BW = RG::BW, STAGE = RG::stage();
  constexpr int NWARP = WY * WZ;
  using Tab = const Real (*)[2][PER][P + 1];
  extern __shared__ __align__(128) unsigned char smem_rt[];

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem_rt + SM::BARS) + warp * RT_NST;
  Real* swt = reinterpret_cast<Real*>(smem_rt + SM::TAB);
  Real* xbuf = reinterpret_cast<Real*>(smem_rt + SM::XBUF) + warp * 2 * (BW + 1);
  Real* stg = reinterpret_cast<Real*>(smem_rt + SM::STG) + (size_t)warp * RT_NST * STAGE;
  Tab sw = reinterpret_cast<Tab>(swt);

  fill_row_table<Real, P, DG>(swt, prm.W.w, threadIdx.x, 32 * NWARP);
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < RT_NST; ++s) mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();

  const int wyi = warp % WY, wzi = warp / WY;
  const int bid = blockIdx.x;
  const int seg = bid % prm.nseg;
  const int by = (bid / prm.nseg) % (prm.ny / WY);
  const int bz = bid / (prm.nseg * (prm.ny / WY));
  const int y = by * WY + wyi, z = bz * WZ + wzi, x0 = seg * 32;
  const int nx = prm.nx, ny = prm.ny, nz = prm.nz;
  const long long n = prm.n;
  const int x = x0 + lane;
  const bool valid = x < nx;
  const int node = (z * ny + y) * nx + (valid ? x : 0);
  const int cx = (valid ? x : 0) % PER, cy = y % PER, cz = z % PER;

  // prologue: directions 1 .. RT_NST in flight
  static_for<1, RT_NST + 1>([&](auto Ic) {
    constexpr int A = decltype(Ic)::value;
    if constexpr (A < Q)
      rowt_issue<S, Real, P, DG, A>(prm.f_in, n, stg + ((A - 1) % RT_NST) * STAGE, &bar[(A - 1) % RT_NST], x0, y,
                                     z, nx, ny, nz, lane);
  });

  Real fs[Q];
  fs[0] = valid ? prm.f_in[node] : Real(0);
  int fail_at = 0;  // direction whose wait ran out (0: none)

  static_for<1, Q>([&](auto Ic) {
    constexpr int A = decltype(Ic)::value;
    constexpr int sx = S::e(A, 0), sy = S::e(A, 1), sz = S::D == 3 ? S::e(A, 2) : 0;
    constexpr int NY = sy != 0 ? P + 1 : 1, NZ = sz != 0 ? P + 1 : 1;
    constexpr int W = RG::width(A);
    constexpr int s = (A - 1) % RT_NST;
    constexpr unsigned parity = ((A - 1) / RT_NST) & 1;
    constexpr int dy = sy > 0 ? 0 : 1, dz = sz > 0 ? 0 : 1, dx = sx > 0 ? 0 : 1;
    (void)dy;
    (void)dz;
    (void)dx;
    if (fail_at) return;
    if (!mbar_wait(&bar[s], parity, prm.wait_polls)) {
      fail_at = A;
      return;
    }
    const Real* st = stg + s * STAGE;
    // yz-factored value at column k of the stage rows
    auto yz = [&](int k) -> Real {
      Real zv[P + 1];
#pragma unroll
      for (int jz = 0; jz < NZ; ++jz) {
        Real yv[P + 1];
#pragma unroll
        for (int jy = 0; jy < NY; ++jy) yv[jy] = st[(jz * NY + jy) * W + k];
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
      out = yz(lane);
    } else {
      const int wst = win_start<P, DG, sx>(valid ? x : x0, cx) - (x0 - HL);  // window start in buffer columns
      Real xv[P + 1];
      if constexpr (NY * NZ == 1) {
        // axis direction: the window straight from the copied row
#pragma unroll
        for (int j = 0; j <= P; ++j) xv[j] = st[RG::XC + wst + j];
      } else {
        Real* buf = xbuf + (xorder<S>(A) & 1) * (BW + 1);
        buf[lane] = yz(RG::XC + lane);
        if (lane + 32 < BW) buf[lane + 32] = yz(RG::XC + lane + 32);
        __syncwarp();
#pragma unroll
        for (int j = 0; j <= P; ++j) xv[j] = buf[wst + j];
      }
      out = wsum_j0<DEV, P>(sw[0][dx][cx], xv, win_j0<P, DG, sx>(cx));
    }
    fs[A] = out;
    // every lane is done with stage s: refill it with direction A + RT_NST
    __syncwarp();
    if constexpr (A + RT_NST < Q) {
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      rowt_issue<S, Real, P, DG, A + RT_NST>(prm.f_in, n, stg + s * STAGE, &bar[s], x0, y, z, nx, ny, nz, lane);
    }
  });

  if (fail_at) {
    // a copy never completed: report, wait (bounded) for the copies still in
    // flight (directions fail_at .. fail_at + RT_NST - 1), stop this warp
    if (lane == 0) atomicOr(prm.status, ST_TIMEOUT);
    for (int d = fail_at; d < fail_at + RT_NST && d < Q; ++d)
      mbar_wait(&bar[(d - 1) % RT_NST], ((d - 1) / RT_NST) & 1, MBAR_MAX_POLLS);
    return;
  }
  if (!valid) return;

  Real u[3] = {0, 0, 0};
  Real rho = Real(1);
  Real pre[Q];
  if constexpr (DEV) {
#pragma unroll
    for (int q = 0; q < Q; ++q) pre[q] = fs[q];
  }
  if constexpr (COLL == COLL_BGK) {
    rho = collide_bgk<S, DEV, false>(fs, Real(1) / Real(prm.tau), u, false);
    if constexpr (DEV) conserve<S>(fs, pre);
  } else if constexpr (COLL == COLL_BGK_INC) {
    rho = collide_bgk_inc<DEV, false>(fs, Real(1) / Real(prm.tau), u, false);
  } else if constexpr (COLL == COLL_KBC) {
    rho = collide_kbc<S, DEV, false>(fs, Real(prm.tau), u, false);
    if constexpr (DEV) conserve<S>(fs, pre);
  }
  (void)pre;
  if constexpr (COLL != COLL_NONE) {
    int bad = 0;
    if (!(rho >= Real(1e-10))) bad |= (rho != rho) ? ST_NAN : ST_DENSITY;
    if (prm.write_macro) {
      prm.rho[node] = (double)rho;
      prm.u[node] = (double)u[0] * prm.scaling;
      prm.u[n + node] = (double)u[1] * prm.scaling;
      if constexpr (S::D == 3) prm.u[2 * n + node] = (double)u[2] * prm.scaling;
    }
    if (bad) atomicOr(prm.status, bad);
  }
#pragma unroll
  for (int q = 0; q < Q; ++q) prm.f_out[q * n + node] = fs[q];
}

}  // namespace natgpu
