// Fused semi-Lagrangian stream + collide, row-segment kernel.
//
// One warp owns a segment of 32 consecutive lattice nodes along x at a fixed
// (y, z); lane l owns node x0 + l and keeps all Q streamed populations of it
// in registers.  For a direction alpha with displacement signs (sx, sy, sz):
//   * the y and z Lagrange factors are applied in registers: the warp loads
//     the (p+1)^k source rows of its window (coalesced, L1/L2-cached) and sums
//     them with the warp-uniform weights of its node classes in y and z;
//   * if sx != 0, the yz-factored row (segment plus the window halo) goes
//     through a warp-private shared-memory row buffer and every lane applies
//     its own x weights (node class in x) to its window; only __syncwarp
//     orders it, there is no CTA-wide barrier anywhere in the kernel.
// The collision then runs on the registers and f is written once, coalesced.
// In the FP32 deviation mode a window sum is evaluated as
//   v_j0 + sum_{j != j0} w_j (v_j - v_j0),
// j0 being the source node at the destination's own position (weight ~ 1):
// a constant field is reproduced exactly and the float rounding of the small
// off-diagonal weights only multiplies differences of neighbouring values.
// For y and z (warp-uniform node classes) the window rows are loaded in the
// rotated order j0, j0+1, ... so that j0 is always slot 0.
// Same operator, tables and window pattern as the specialised tile kernel
// (sl_step_v2.cuh, Geo<P, DG>): every departure point lies in the node's own
// cell or the adjacent upwind cell (checked on the host).
#pragma once

#include <cuda_runtime.h>

#include "collision.cuh"
#include "natgpu_common.h"
#include "sl_step_v2.cuh"
#include "stencils.cuh"

namespace natgpu {

template <class Real>
struct RowParams {
  const Real* f_in;
  Real* f_out;
  double* rho;
  double* u;
  int* status;
  int n;  // nodes per block
  int nx, ny, nz;
  int nseg;  // 32-node segments per row
  double tau;
  double scaling;
  int write_macro;
  unsigned wait_polls;  // bulk-copy row kernel: limit of each wait for a stage (MBAR_MAX_POLLS)
  SpecWeights<Real> W;  // [axis][sign][class][j]
};

// window of one node along an axis: start (absolute lattice index, before
// the periodic wrap) and the index of the dominant weight
template <int P, bool DG, int SG>
__device__ __forceinline__ int win_start(int node, int c) {
  constexpr int PER = Geo<P, DG>::PER;
  int shift = 0;
  if constexpr (SG > 0) shift = (c == 0) ? -1 : 0;
  if constexpr (SG < 0 && DG) shift = (c == P) ? 1 : 0;
  return node - c + shift * PER;
}
template <int P, bool DG, int SG>
__device__ __forceinline__ int win_j0(int c) {
  if constexpr (SG > 0) return c == 0 ? P : c;
  if constexpr (SG < 0 && DG) return c == P ? 0 : c;
  return c;
}

__device__ __forceinline__ int wrap(int g, int n) {
  g += g < 0 ? n : 0;
  g -= g >= n ? n : 0;
  return g;
}

// sum_s w_s v_s over a window whose slot 0 holds the dominant node; in the
// deviation mode v_0 + sum_{s >= 1} w_s (v_s - v_0)
template <bool DEV, int P, class Real>
__device__ __forceinline__ Real wsum(const Real* w, const Real (&v)[P + 1]) {
  if constexpr (DEV) {
    Real acc = Real(0);
#pragma unroll
    for (int j = 1; j <= P; ++j) acc = fma(w[j], v[j] - v[0], acc);
    return acc + v[0];
  } else {
    Real acc = w[0] * v[0];
#pragma unroll
    for (int j = 1; j <= P; ++j) acc = fma(w[j], v[j], acc);
    return acc;
  }
}

// the same over a window in natural order with the dominant slot j0 known
// at run time (x factor, per-lane class); w_j0 is stored as 0 in the
// deviation mode
template <bool DEV, int P, class Real>
__device__ __forceinline__ Real wsum_j0(const Real* w, const Real (&v)[P + 1], int j0) {
  if constexpr (DEV) {
    Real v0 = v[0];
#pragma unroll
    for (int j = 1; j <= P; ++j) v0 = (j == j0) ? v[j] : v0;
    Real acc = Real(0);
#pragma unroll
    for (int j = 0; j <= P; ++j) acc = fma(w[j], v[j] - v0, acc);
    return acc + v0;
  } else {
    Real acc = w[0] * v[0];
#pragma unroll
    for (int j = 1; j <= P; ++j) acc = fma(w[j], v[j], acc);
    return acc;
  }
}

// number of directions before ALPHA that have an x component
template <class S>
__host__ __device__ constexpr int xorder(int alpha) {
  int k = 0;
  for (int i = 1; i < alpha; ++i) k += S::e(i, 0) != 0;
  return k;
}

// number of yz-diagonal directions (no x component, y and z components)
// before ALPHA
template <class S>
__host__ __device__ constexpr int yzorder(int alpha) {
  int k = 0;
  if constexpr (S::D == 3)
    for (int i = 1; i < alpha; ++i) k += S::e(i, 0) == 0 && S::e(i, 1) != 0 && S::e(i, 2) != 0;
  return k;
}

// Rows of the z-factored union buffer of a CTA of ZWY rows aligned to cell
// starts (ZWY a multiple of PER): the windows of its rows span at most the
// CTA's cells, one cell before or after them, and one shared node (FE_Q).
template <int PER, int ZWY>
__host__ __device__ constexpr int zs_rows() {
  return (ZWY / PER + 1) * PER + 1;
}

// Arguments of one row-segment work item (one solve).
template <class Real>
struct RowArgs {
  const Real* f_in;
  Real* f_out;
  double* rho;
  double* u;
  int* status;
  int n;
  int nx, ny, nz;
  double tau;
  double scaling;
  int write_macro;
};

// Element count of a weight table [3][2][PER][P+1] for order P, topology DG.
template <int P, bool DG>
__host__ __device__ constexpr int row_table_size() {
  return 3 * 2 * Geo<P, DG>::PER * (P + 1);
}

// Fill a weight table from [axis][sign][class][j] weights: y and z in the
// rotated slot order (slot s = window index (j0 + s) mod (P+1)), x in
// natural order with the dominant weight zeroed in the deviation mode.
// Threads t0, t0 + stride, ... of the caller cooperate.
template <class Real, int P, bool DG>
__device__ __forceinline__ void fill_row_table(Real* sw, const Real (&W)[3][2][PER_MAX][PMAX1], int t0,
                                               int stride) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int PER = Geo<P, DG>::PER;
  for (int i = t0; i < row_table_size<P, DG>(); i += stride) {
    const int j = i % (P + 1), c = (i / (P + 1)) % PER, sd = (i / ((P + 1) * PER)) % 2, a = i / ((P + 1) * PER * 2);
    const int j0 = sd == 0 ? win_j0<P, DG, 1>(c) : win_j0<P, DG, -1>(c);
    Real w;
    if (a == 0)
      w = (DEV && j == j0) ? Real(0) : W[a][sd][c][j];
    else
      w = W[a][sd][c][(j0 + j) % (P + 1)];
    sw[i] = w;
  }
}

// Collision of one node whose streamed values are in fs_s[q * 32 + lane]
// (shared memory written by the same lane), and the single write of f.
template <class S, class Real, int COLL>
__device__ __forceinline__ void row_collide(const RowArgs<Real>& prm, const Real* fs_s, int node, int lane) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q;
  Real fs[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) fs[q] = fs_s[q * 32 + lane];
  Real u[3] = {0, 0, 0};
  Real rho = Real(1);
  if constexpr (COLL == COLL_BGK) {
    rho = collide_bgk<S, DEV, false>(fs, Real(1) / Real(prm.tau), u, false);
  } else if constexpr (COLL == COLL_BGK_INC) {
    rho = collide_bgk_inc<DEV, false>(fs, Real(1) / Real(prm.tau), u, false);
  } else if constexpr (COLL == COLL_KBC) {
    rho = collide_kbc<S, DEV, false>(fs, Real(prm.tau), u, false);
  }
  if constexpr (DEV && (COLL == COLL_BGK || COLL == COLL_KBC)) {
    Real pre[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) pre[q] = fs_s[q * 32 + lane];
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
  for (int q = 0; q < Q; ++q) prm.f_out[q * prm.n + node] = fs[q];
}

// One warp: stream + collide the 32-node segment starting at x0 of row
// (y, z).  swt: the weight table (fill_row_table); buf: this warp's two
// row buffers of BW + 1 elements.  With fs_s != nullptr (SS) the streamed
// values go to this warp's shared array fs_s[Q][32] instead of registers:
// far fewer live registers while streaming (more resident warps to hide the
// load latency); the collision reads them back, and its mass/momentum
// projection takes the pre-collision values from there as well.
//
// ZWY > 0 (z sharing): the CTA's ZWY warps own rows y0 .. y0 + ZWY - 1 of one
// z (y0 a multiple of PER).  For a yz-diagonal direction the z-factored rows
// of the union of their y windows are computed once per CTA into zsh
// (round-robin over the warps, one barrier), and each warp then applies its
// y factor from there: ~1.6 z-window sums per lane instead of P + 1.
template <class S, class Real, int COLL, int P, bool DG, bool SS = false, int ZWY = 0>
__device__ __forceinline__ void row_body(const RowArgs<Real>& prm, const Real* swt, Real* buf2, int y, int z,
                                         int x0, int lane, Real* fs_s = nullptr, Real* zsh = nullptr,
                                         int zwarp = 0, int y0 = 0) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q;
  constexpr int PER = Geo<P, DG>::PER;
  constexpr int HL = PER;               // left halo of the x window buffer
  constexpr int BW = 32 + PER + P + 1;  // buffer width
  using Tab = const Real (*)[2][PER][P + 1];
  Tab sw = reinterpret_cast<Tab>(swt);

  const int nx = prm.nx, ny = prm.ny, nz = prm.nz;
  const int x = x0 + lane;
  const bool valid = x < nx;
  const int nxy = nx * ny;
  const int node = z * nxy + y * nx + (valid ? x : 0);
  // node classes
  const int cx = (valid ? x : 0) % PER, cy = y % PER, cz = z % PER;
  // x positions of this lane's two buffer slots (full modulo: a row can be
  // shorter than the 32-lane segment)
  const int gxa = ((x0 - HL + lane) % nx + nx) % nx;
  const bool hasb = lane + 32 < BW;
  const int gxb = ((x0 - HL + 32 + (hasb ? lane : 0)) % nx + nx) % nx;

  Real fs[SS ? 1 : Q];
  if constexpr (SS)
    fs_s[lane] = valid ? prm.f_in[node] : Real(0);
  else
    fs[0] = valid ? prm.f_in[node] : Real(0);

  static_for<1, Q>([&](auto I) {
    constexpr int A = decltype(I)::value;
    constexpr int sx = S::e(A, 0), sy = S::e(A, 1), sz = S::D == 3 ? S::e(A, 2) : 0;
    constexpr int NJY = sy != 0 ? P + 1 : 1;
    constexpr int NJZ = sz != 0 ? P + 1 : 1;
    const Real* __restrict__ src = prm.f_in + (long long)A * prm.n;
    // warp-uniform row windows
    int ys = y, zs = z, j0y = 0, j0z = 0;
    if constexpr (sy != 0) {
      ys = win_start<P, DG, sy>(y, cy);
      j0y = win_j0<P, DG, sy>(cy);
    }
    if constexpr (sz != 0) {
      zs = win_start<P, DG, sz>(z, cz);
      j0z = win_j0<P, DG, sz>(cz);
    }
    constexpr int dy = sy > 0 ? 0 : 1, dz = sz > 0 ? 0 : 1, dx = sx > 0 ? 0 : 1;
    (void)dz;
    (void)dy;
    (void)dx;
    // Row offsets of the window in the rotated order (slot 0 is the
    // dominant row), computed once per direction in the z-sharing form
    // (there the yz-diagonals do not go through yz()).  The other forms
    // compute them inline: holding the offsets across the two yz() calls of
    // an x direction spills at 64 registers (measured 19 % slower).
    constexpr bool HOIST = ZWY > 0;
    int zo[NJZ], yo[NJY];
    (void)zo;
    (void)yo;
    if constexpr (HOIST) {
#pragma unroll
      for (int jz = 0; jz < NJZ; ++jz) {
        const int rz = j0z + jz;
        zo[jz] = wrap(zs + (rz > P ? rz - (P + 1) : rz), nz) * nxy;
      }
#pragma unroll
      for (int jy = 0; jy < NJY; ++jy) {
        const int ry = j0y + jy;
        yo[jy] = wrap(ys + (ry > P ? ry - (P + 1) : ry), ny) * nx;
      }
    }
    // yz-factored value at x position gx
    auto yz = [&](int gx) -> Real {
      Real zv[P + 1];
#pragma unroll
      for (int jz = 0; jz < NJZ; ++jz) {
        Real yv[P + 1];
        if constexpr (HOIST) {
          const Real* __restrict__ px = src + gx;
#pragma unroll
          for (int jy = 0; jy < NJY; ++jy) yv[jy] = __ldg(px + (zo[jz] + yo[jy]));
        } else {
          const int rz = j0z + jz;
          const int gz = wrap(zs + (rz > P ? rz - (P + 1) : rz), nz);
#pragma unroll
          for (int jy = 0; jy < NJY; ++jy) {
            const int ry = j0y + jy;
            const int gy = wrap(ys + (ry > P ? ry - (P + 1) : ry), ny);
            yv[jy] = __ldg(src + gz * nxy + gy * nx + gx);
          }
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
    if constexpr (ZWY > 0 && sx == 0 && sy != 0 && sz != 0) {
      // z-factored rows of the CTA's window union, then this row's y factor
      constexpr int U = zs_rows<PER, ZWY>();
      Real* Z = zsh + (yzorder<S>(A) & 1) * (U * 32);
      const int ybase = sy > 0 ? y0 - PER : y0;
      const int gxx = valid ? x : 0;
      for (int uu = zwarp; uu < U; uu += ZWY) {
        const int gy = wrap(ybase + uu, ny);
        Real zv[P + 1];
        const Real* __restrict__ pr = src + gy * nx + gxx;
#pragma unroll
        for (int jz = 0; jz <= P; ++jz) zv[jz] = __ldg(pr + zo[jz]);
        Z[uu * 32 + lane] = wsum<DEV, P>(sw[2][dz][cz], zv);
      }
      __syncthreads();
      Real yv[P + 1];
#pragma unroll
      for (int jy = 0; jy <= P; ++jy) {
        const int ry = j0y + jy;
        yv[jy] = Z[(ys - ybase + (ry > P ? ry - (P + 1) : ry)) * 32 + lane];
      }
      out = wsum<DEV, P>(sw[1][dy][cy], yv);
    } else if constexpr (sx == 0) {
      out = yz(valid ? x : 0);
    } else {
      // alternate buffers between consecutive x factors: the __syncwarp of
      // the next one orders this one's reads before its writes
      Real* buf = buf2 + (xorder<S>(A) & 1) * (BW + 1);
      buf[lane] = yz(gxa);
      if (hasb) buf[lane + 32] = yz(gxb);
      __syncwarp();
      const int st = win_start<P, DG, sx>(x, cx) - (x0 - HL);
      Real xv[P + 1];
#pragma unroll
      for (int j = 0; j <= P; ++j) xv[j] = buf[st + j];
      out = wsum_j0<DEV, P>(sw[0][dx][cx], xv, win_j0<P, DG, sx>(cx));
    }
    if constexpr (SS)
      fs_s[A * 32 + lane] = out;
    else
      fs[A] = out;
  });

  if (!valid) return;
  if constexpr (SS) {
    row_collide<S, Real, COLL>(prm, fs_s, node, lane);
    return;
  } else {
    int bad = 0;
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
    for (int q = 0; q < Q; ++q) prm.f_out[q * prm.n + node] = fs[q];
  }
}

// Single-solve kernel: CTA = WY x WZ warps over rows (y, z) and one 32-node
// x segment.
// SS: streamed values in shared memory (row_body), MINB: resident CTAs per
// SM the register allocation is sized for.
// ZS: z sharing of the yz-diagonal directions (row_body, ZWY = WY; WY a
// multiple of PER, WZ = 1).
template <class S, class Real, int COLL, int P, bool DG, int WY, int WZ, bool SS = false,
          int MINB = (sizeof(Real) == 4 ? 2 : 1), bool ZS = false>
__global__ void __launch_bounds__(32 * WY * WZ, MINB) k_sl_row(const __grid_constant__ RowParams<Real> prm) {
  constexpr int PER = Geo<P, DG>::PER;
  constexpr int BW = 32 + PER + P + 1;
  constexpr int NW = WY * WZ;
  static_assert(!ZS || (WZ == 1 && WY % PER == 0), "z sharing needs cell-aligned y rows");
  __shared__ Real rowbuf[NW][2][BW + 1];
  __shared__ Real zbuf[ZS ? 2 : 1][ZS ? zs_rows<PER, WY>() * 32 : 1];
  __shared__ Real fs_sh[SS ? NW : 1][SS ? S::Q * 32 : 1];
  __shared__ Real sw[row_table_size<P, DG>()];
  fill_row_table<Real, P, DG>(sw, prm.W.w, threadIdx.x, 32 * NW);
  __syncthreads();

  const int lane = threadIdx.x & 31;
  // a one-warp CTA derives (y, z) from blockIdx alone: the compiler then
  // keeps the row windows, offsets and y/z weights in uniform registers
  const int warp = NW == 1 ? 0 : (int)(threadIdx.x >> 5);
  const int wyi = warp % WY, wzi = warp / WY;
  const int bid = blockIdx.x;
  const int seg = bid % prm.nseg;
  const int by = (bid / prm.nseg) % (prm.ny / WY);
  const int bz = bid / (prm.nseg * (prm.ny / WY));
  RowArgs<Real> a;
  a.f_in = prm.f_in;
  a.f_out = prm.f_out;
  a.rho = prm.rho;
  a.u = prm.u;
  a.status = prm.status;
  a.n = prm.n;
  a.nx = prm.nx;
  a.ny = prm.ny;
  a.nz = prm.nz;
  a.tau = prm.tau;
  a.scaling = prm.scaling;
  a.write_macro = prm.write_macro;
  row_body<S, Real, COLL, P, DG, SS, ZS ? WY : 0>(a, sw, &rowbuf[warp][0][0], by * WY + wyi, bz * WZ + wzi,
                                                 seg * 32, lane, SS ? fs_sh[SS ? warp : 0] : nullptr,
                                                 &zbuf[0][0], wyi, by * WY);
}

}  // namespace natgpu
