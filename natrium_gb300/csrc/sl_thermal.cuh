// Compressible two-population model on D2Q25H: fused semi-Lagrangian
// stream of f and g + relaxWithG collision, one pass over HBM per step.
//
// Replaces, per time step, the reference's
//   CompressibleCFDSolver::stream() and gStream()  (solver/CompressibleCFDSolver.h:181-314):
//       f_tmp = f; fStream = A f_tmp.fStream; g_tmp = g; gStream = A g_tmp.gStream
//       with the same streaming matrix A for both populations;
//   CompressibleCFDSolver::collide()               (:739-788) ->
//   CollisionOperator::collideAll(f, g, rho, u, T, mask)
//                                                  (collision_advanced/CollisionOperator.h:113-224)
//   BGKCollision::relaxWithG                        (collision_advanced/CollisionSchemes.h:43-118)
//   QuarticEquilibrium                              (collision_advanced/Equilibria.h:88-267)
//
// Work decomposition (the row-segment scheme of sl_row.cuh, generalised to
// run-time order and table-driven windows): one warp owns 32 consecutive
// x-nodes of one row y; lane l keeps all 25 streamed values of f AND of g of
// its node in registers.  Per direction the warp-uniform y window is summed
// straight from global memory (L1/L2), the x window through a warp-private
// shared-memory row; no CTA barrier after the table set-up.  The window
// offset and weights of every (axis, displacement class, node class) come
// from the host tables (FP64 departure points), so any order p <= 6, both
// node topologies and departure points several cells upwind are handled.
//
// The collision works on the symmetry groups of D2Q25H (directions with the
// same |e_x|, |e_y|): the quartic equilibrium is a degree-4 polynomial in
// (e_x, e_y) whose parts even/odd in e_x and e_y are evaluated once per
// group, and the members follow by sign changes.  Moments use group sums;
// the temperature uses sum |e - u|^2 f = sum |e|^2 f - u . j.  All FP64 in
// the plain form; the GB300's FP64 rate makes this kernel FP64-pipe bound,
// so the formulation minimises FP64 operations per node.
#pragma once

#include <cuda_runtime.h>

#include "natgpu_common.h"
#include "stencils.cuh"

namespace natgpu {

// Number of directions before A with an x component (alternating x buffers).
__host__ __device__ constexpr int th_xorder(int A) {
  int k = 0;
  for (int i = 1; i < A; ++i) k += SD2Q25H::code(i, 0) != 0;
  return k;
}

// Coefficients of the equilibrium polynomial P(e) with f^eq_i = w_i rho P(e_i):
//   even part  E  = c0 + kx X^2 + ky Y^2 + k4xxxx Hxxxx + k4xxyy Hxxyy + k4yyyy Hyyyy
//   odd in x   Ox = kox X + k3xxx Hxxx + k3xyy Hxyy
//   odd in y   Oy = koy Y + k3xxy Hxxy + k3yyy Hyyy
//   odd in xy  Oxy = kxy X Y + k4xxxy Hxxxy + k4xyyy Hxyyy
// and P(sx X, sy Y) = E + sx Ox + sy Oy + sx sy Oxy.  Term by term this is
// the reference's polynomial (Equilibria.h:145-263):
//   1 + u.e/c^2 + (u.e)^2/(2 c^4) - u^2/(2 c^2) + (T-1)/(2 c^2) (|e|^2 - D c^2)
//   + a3 : H3 / (6 c^6) + a4 : H4 / (24 c^8)
// with the Hermite tensors H3, H4 of AuxiliaryCollisionFunctions.h:520-566
// and a3, a4 the velocity/temperature tensors of Equilibria.h:157-181.
struct EqCoef {
  double c0, kx, ky, kxy, kox, koy;
  double k3xxx, k3xxy, k3xyy, k3yyy;
  double k4xxxx, k4xxxy, k4xxyy, k4xyyy, k4yyyy;
};

__device__ __forceinline__ EqCoef eq_coef(const ThermalModel& M, bool quartic, double ux, double uy, double T) {
  const double cs2 = M.cs2;
  const double i2 = 1.0 / (2.0 * cs2);
  const double i4 = 1.0 / (2.0 * cs2 * cs2);
  EqCoef k;
  const double Tm1 = quartic ? T - 1.0 : 0.0;
  k.c0 = 1.0 - (ux * ux + uy * uy) * i2 - Tm1;
  k.kx = ux * ux * i4 + Tm1 * i2;
  k.ky = uy * uy * i4 + Tm1 * i2;
  k.kxy = ux * uy * (2.0 * i4);
  k.kox = ux * (2.0 * i2);
  k.koy = uy * (2.0 * i2);
  if (quartic) {
    const double T1 = cs2 * Tm1;
    const double c3 = 1.0 / (6.0 * cs2 * cs2 * cs2);
    const double c4 = 1.0 / (24.0 * cs2 * cs2 * cs2 * cs2);
    const double ux2 = ux * ux, uy2 = uy * uy, uxy = ux * uy;
    k.k3xxx = c3 * (ux2 * ux + 3.0 * T1 * ux);
    k.k3xxy = 3.0 * c3 * (ux2 * uy + T1 * uy);
    k.k3xyy = 3.0 * c3 * (ux * uy2 + T1 * ux);
    k.k3yyy = c3 * (uy2 * uy + 3.0 * T1 * uy);
    k.k4xxxx = c4 * (ux2 * ux2 + 6.0 * T1 * ux2 + 3.0 * T1 * T1);
    k.k4yyyy = c4 * (uy2 * uy2 + 6.0 * T1 * uy2 + 3.0 * T1 * T1);
    k.k4xxxy = 4.0 * c4 * (ux2 * uxy + 3.0 * T1 * uxy);
    k.k4xyyy = 4.0 * c4 * (uxy * uy2 + 3.0 * T1 * uxy);
    k.k4xxyy = 6.0 * c4 * (ux2 * uy2 + T1 * (ux2 + uy2) + T1 * T1);
  } else {
    k.k3xxx = k.k3xxy = k.k3xyy = k.k3yyy = 0.0;
    k.k4xxxx = k.k4xxxy = k.k4xxyy = k.k4xyyy = k.k4yyyy = 0.0;
  }
  return k;
}

// Group parts (E, Ox, Oy, Oxy) of the equilibrium polynomial for group G.
template <int G>
__device__ __forceinline__ void eq_parts(const ThermalModel& M, const EqCoef& k, double& E, double& Ox, double& Oy,
                                         double& Oxy) {
  constexpr bool HX = SD2Q25H::gx(G) != 0, HY = SD2Q25H::gy(G) != 0;
  const double X = M.X[G], Y = M.Y[G];
  E = k.c0;
  if constexpr (HX) E = fma(k.kx, X * X, E);
  if constexpr (HY) E = fma(k.ky, Y * Y, E);
  E = fma(k.k4xxxx, M.h4[G][0], E);
  E = fma(k.k4xxyy, M.h4[G][2], E);
  E = fma(k.k4yyyy, M.h4[G][4], E);
  Ox = Oy = Oxy = 0.0;
  if constexpr (HX) Ox = fma(k.kox, X, fma(k.k3xxx, M.h3[G][0], k.k3xyy * M.h3[G][2]));
  if constexpr (HY) Oy = fma(k.koy, Y, fma(k.k3xxy, M.h3[G][1], k.k3yyy * M.h3[G][3]));
  if constexpr (HX && HY) Oxy = fma(k.kxy, X * Y, fma(k.k4xxxy, M.h4[G][1], k.k4xyyy * M.h4[G][3]));
}

// Value of P for direction I of group G from the group parts.
template <int I>
__device__ __forceinline__ double eq_member(double E, double Ox, double Oy, double Oxy) {
  constexpr int G = SD2Q25H::group(I);
  constexpr int sx = SD2Q25H::sgn(I, 0), sy = SD2Q25H::sgn(I, 1);
  constexpr bool HX = SD2Q25H::gx(G) != 0, HY = SD2Q25H::gy(G) != 0;
  double a = E, b = 0.0;
  if constexpr (HX) a = sx > 0 ? a + Ox : a - Ox;
  if constexpr (HY) b = sy > 0 ? Oy : -Oy;
  if constexpr (HX && HY) b = (sx * sy > 0) ? b + Oxy : b - Oxy;
  return a + b;
}

// relaxWithG on one node.  f, g: the 25 post-streaming values, overwritten
// with the post-collision ones.  With given_u the velocity (unscaled) is the
// prescribed one (initialisation procedure), otherwise it is computed.
// Returns the status bits (density underflow / NaN).
__device__ __forceinline__ int thermal_relax(const ThermalModel& M, double (&f)[TH_Q], double (&g)[TH_Q],
                                             bool given_u, double& ux, double& uy, double& rho_o, double& T_o,
                                             double& kn_o) {
  // ---- moments by symmetry group ----------------------------------------
  double rho = 0.0, jx = 0.0, jy = 0.0, s2 = 0.0, gsum = 0.0;
  static_for<0, TH_NG>([&](auto Gc) {
    constexpr int G = decltype(Gc)::value;
    double s = 0.0, sxs = 0.0, sys = 0.0;
    static_for<0, TH_Q>([&](auto Ic) {
      constexpr int I = decltype(Ic)::value;
      if constexpr (SD2Q25H::group(I) == G) {
        s += f[I];
        if constexpr (SD2Q25H::gx(G) != 0) sxs = SD2Q25H::sgn(I, 0) > 0 ? sxs + f[I] : sxs - f[I];
        if constexpr (SD2Q25H::gy(G) != 0) sys = SD2Q25H::sgn(I, 1) > 0 ? sys + f[I] : sys - f[I];
      }
    });
    rho += s;
    if constexpr (G != 0) s2 = fma(M.e2[G], s, s2);
    if constexpr (SD2Q25H::gx(G) != 0) jx = fma(M.X[G], sxs, jx);
    if constexpr (SD2Q25H::gy(G) != 0) jy = fma(M.Y[G], sys, jy);
  });
#pragma unroll
  for (int i = 0; i < TH_Q; ++i) gsum += g[i];
  int bad = 0;
  if (!(rho >= 1e-10)) bad = (rho != rho) ? ST_NAN : ST_DENSITY;
  const double rinv = 1.0 / rho;
  double vx = jx * rinv, vy = jy * rinv;
  // T = 0.5 / (rho C_v) sum_i (|e_i - u|^2 f_i / c_s^2 + g_i)   (AuxiliaryCollisionFunctions.h:289-307)
  const double T = 0.5 * ((s2 - (vx * jx + vy * jy)) / M.cs2 + gsum) * rinv / M.C_v;
  if (given_u) {
    vx = ux;
    vy = uy;
  }
  // ---- relaxation parameters (CollisionSchemes.h:81-113) -----------------
  double suth = 1.0;
  if (M.sutherland_set) suth = pow(T / 0.85, 0.7);
  const double visc_tau = (M.tau - 0.5) * suth / (T * rho) + 0.5;
  const double omega = 1.0 / visc_tau;
  const double Tg = T * M.gfac;  // g^eq = f^eq T (2 C_v - D)
  const EqCoef k = eq_coef(M, M.quartic != 0, vx, vy, T);
  double kn = 0.0;
  if (!M.prandtl_set) {
    // single pass: f -= omega (f - f^eq), g -= omega (g - g^eq)
    static_for<0, TH_NG>([&](auto Gc) {
      constexpr int G = decltype(Gc)::value;
      double E, Ox, Oy, Oxy;
      eq_parts<G>(M, k, E, Ox, Oy, Oxy);
      const double wr = M.w[G] * rho;
      static_for<0, TH_Q>([&](auto Ic) {
        constexpr int I = decltype(Ic)::value;
        if constexpr (SD2Q25H::group(I) == G) {
          const double feq = wr * eq_member<I>(E, Ox, Oy, Oxy);
          const double fneq = f[I] - feq;
          kn = fma(fabs(fneq), M.winv[G], kn);
          f[I] = fma(-omega, fneq, f[I]);
          const double gneq = g[I] - feq * Tg;
          g[I] = fma(-omega, gneq, g[I]);
        }
      });
    });
  } else {
    // Prandtl correction (CollisionSchemes.h:63-79, AuxiliaryCollisionFunctions.h:445-516):
    // pass 1 -> non-equilibrium parts, centred heat flux of f^neq and centred
    // flux of g^neq; pass 2 -> f = f^eq + (1 - omega) f^neq + (omega - omega_Pr) f*.
    double qxxx = 0.0, qxxy = 0.0, qxyy = 0.0, qyyy = 0.0, fx = 0.0, fy = 0.0;
    static_for<0, TH_NG>([&](auto Gc) {
      constexpr int G = decltype(Gc)::value;
      double E, Ox, Oy, Oxy;
      eq_parts<G>(M, k, E, Ox, Oy, Oxy);
      const double wr = M.w[G] * rho;
      static_for<0, TH_Q>([&](auto Ic) {
        constexpr int I = decltype(Ic)::value;
        if constexpr (SD2Q25H::group(I) == G) {
          const double feq = wr * eq_member<I>(E, Ox, Oy, Oxy);
          const double fneq = f[I] - feq;
          const double gneq = g[I] - feq * Tg;
          kn = fma(fabs(fneq), M.winv[G], kn);
          f[I] = fneq;
          g[I] = gneq;
          const double dx = SD2Q25H::sgn(I, 0) * M.X[G] - vx;
          const double dy = SD2Q25H::sgn(I, 1) * M.Y[G] - vy;
          const double tx = dx * fneq, ty = dy * fneq;
          qxxx = fma(dx * dx, tx, qxxx);
          qxxy = fma(dx * dx, ty, qxxy);
          qxyy = fma(dy * dy, tx, qxyy);
          qyyy = fma(dy * dy, ty, qyyy);
          fx = fma(dx, gneq, fx);
          fy = fma(dy, gneq, fy);
        }
      });
    });
    const double prandtl_tau = (visc_tau - 0.5) / M.prandtl + 0.5;
    const double pdiff = omega - 1.0 / prandtl_tau;
    const double cs6 = 6.0 * M.cs2 * M.cs2 * M.cs2;
    const double a3 = pdiff / cs6;      // f* = w (Q : H3) / (6 c^6)
    const double ag = pdiff / T;        // g* = w (F . e) / T
    const double om1 = 1.0 - omega;
    static_for<0, TH_NG>([&](auto Gc) {
      constexpr int G = decltype(Gc)::value;
      double E, Ox, Oy, Oxy;
      eq_parts<G>(M, k, E, Ox, Oy, Oxy);
      const double wr = M.w[G] * rho;
      // odd-in-x and odd-in-y parts of Q : H3 and of F . e for this group
      const double qx = fma(qxxx, M.h3[G][0], 3.0 * qxyy * M.h3[G][2]);
      const double qy = fma(3.0 * qxxy, M.h3[G][1], qyyy * M.h3[G][3]);
      const double gx = fx * M.X[G], gy = fy * M.Y[G];
      static_for<0, TH_Q>([&](auto Ic) {
        constexpr int I = decltype(Ic)::value;
        if constexpr (SD2Q25H::group(I) == G) {
          constexpr double sx = SD2Q25H::sgn(I, 0), sy = SD2Q25H::sgn(I, 1);
          constexpr bool HX = SD2Q25H::gx(G) != 0, HY = SD2Q25H::gy(G) != 0;
          const double feq = wr * eq_member<I>(E, Ox, Oy, Oxy);
          double qh = 0.0, ge = 0.0;
          if constexpr (HX) {
            qh = sx * qx;
            ge = sx * gx;
          }
          if constexpr (HY) {
            qh = fma(sy, qy, qh);
            ge = fma(sy, gy, ge);
          }
          const double fstar = M.w[G] * qh;
          const double gstar = M.w[G] * ge;
          f[I] = fma(a3, fstar, fma(om1, f[I], feq));
          g[I] = fma(ag, gstar, fma(om1, g[I], feq * Tg));
        }
      });
    });
  }
  rho_o = rho;
  ux = vx;
  uy = vy;
  T_o = T;
  kn_o = kn * (1.0 / TH_Q);
  return bad;
}

// Fused step: stream f and g (same operator), then (COLLIDE) relaxWithG.
template <bool COLLIDE>
__global__ void __launch_bounds__(32 * TH_WARPS, 1) k_thermal_step(const __grid_constant__ ThermalStep P) {
  __shared__ double swx[ND_MAX][PER_MAX][PMAX1];
  __shared__ int soffx[ND_MAX][PER_MAX];
  __shared__ double bufs[TH_WARPS][4][TH_BWMAX + 1];
  for (int i = threadIdx.x; i < ND_MAX * PER_MAX * PMAX1; i += blockDim.x)
    (&swx[0][0][0])[i] = (&P.tb.w[0][0][0][0])[i];
  for (int i = threadIdx.x; i < ND_MAX * PER_MAX; i += blockDim.x) (&soffx[0][0])[i] = (&P.tb.off[0][0][0])[i];
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wid = blockIdx.x * TH_WARPS + warp;
  if (wid >= P.nseg * P.ny) return;  // warp-uniform
  const int nx = P.nx, ny = P.ny, n = P.n;
  const int p = P.tb.p, per = P.tb.per;
  const int seg = wid % P.nseg, y = wid / P.nseg;
  const int x0 = seg * 32, x = x0 + lane;
  const bool valid = x < nx;
  const int xs = valid ? x : x0;
  const int node = y * nx + xs;
  const int cx = xs % per, cy = y % per;

  double fs[TH_Q], gs[TH_Q];
  fs[0] = P.f_in[node];
  gs[0] = P.g_in[node];

  static_for<1, TH_Q>([&](auto Ic) {
    constexpr int A = decltype(Ic)::value;
    constexpr int dx = SD2Q25H::dcls(A, 0), dy = SD2Q25H::dcls(A, 1);
    const double* __restrict__ fsrc = P.f_in + (long long)A * n;
    const double* __restrict__ gsrc = P.g_in + (long long)A * n;
    // warp-uniform y window: rows and weights
    int rowoff[PMAX1];
    double wy[PMAX1];
    if constexpr (dy >= 0) {
      const int ys = y + P.tb.off[1][dy][cy];
#pragma unroll
      for (int j = 0; j < PMAX1; ++j) {
        int r = ys + j;
        r = ((r % ny) + ny) % ny;
        rowoff[j] = r * nx;
        wy[j] = P.tb.w[1][dy][cy][j];
      }
    } else {
      rowoff[0] = y * nx;
    }
    auto ysum = [&](int gx, double& vf, double& vg) {
      if constexpr (dy >= 0) {
        double af = 0.0, ag = 0.0;
#pragma unroll
        for (int j = 0; j < PMAX1; ++j)
          if (j <= p) {
            af = fma(wy[j], __ldg(fsrc + rowoff[j] + gx), af);
            ag = fma(wy[j], __ldg(gsrc + rowoff[j] + gx), ag);
          }
        vf = af;
        vg = ag;
      } else {
        vf = __ldg(fsrc + rowoff[0] + gx);
        vg = __ldg(gsrc + rowoff[0] + gx);
      }
    };
    if constexpr (dx < 0) {
      ysum(xs, fs[A], gs[A]);
    } else {
      double* bf = &bufs[warp][(th_xorder(A) & 1) * 2][0];
      double* bg = &bufs[warp][(th_xorder(A) & 1) * 2 + 1][0];
      for (int k = lane; k < P.tb.bw; k += 32) {
        int gx = x0 + P.tb.xl + k;
        gx = ((gx % nx) + nx) % nx;
        double vf, vg;
        ysum(gx, vf, vg);
        bf[k] = vf;
        bg[k] = vg;
      }
      __syncwarp();
      const int st = lane * (valid ? 1 : 0) + soffx[dx][cx] - P.tb.xl;
      double af = 0.0, ag = 0.0;
#pragma unroll
      for (int j = 0; j < PMAX1; ++j)
        if (j <= p) {
          af = fma(swx[dx][cx][j], bf[st + j], af);
          ag = fma(swx[dx][cx][j], bg[st + j], ag);
        }
      fs[A] = af;
      gs[A] = ag;
    }
  });

  if (!valid) return;
  if constexpr (COLLIDE) {
    double ux = 0.0, uy = 0.0, rho, T, kn;
    const int bad = thermal_relax(P.M, fs, gs, false, ux, uy, rho, T, kn);
    if (bad) atomicOr(P.status, bad);
    if (P.write_macro) {
      P.rho[node] = rho;
      P.u[node] = ux * P.M.scaling;
      P.u[n + node] = uy * P.M.scaling;
      P.T[node] = T;
      P.mask[node] = kn;
    }
  }
#pragma unroll
  for (int q = 0; q < TH_Q; ++q) {
    P.f_out[(long long)q * n + node] = fs[q];
    P.g_out[(long long)q * n + node] = gs[q];
  }
}

// Collision only (CollisionOperator::collideAll(f, g, ...)), in place.
__global__ void __launch_bounds__(256) k_thermal_collide(const __grid_constant__ ThermalPoint P) {
  const long long n = P.n;
  int bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double f[TH_Q], g[TH_Q];
#pragma unroll
    for (int q = 0; q < TH_Q; ++q) {
      f[q] = P.f[q * n + i];
      g[q] = P.g[q * n + i];
    }
    double ux = 0.0, uy = 0.0, rho, T, kn;
    if (P.in_init) {
      ux = P.u[i] / P.M.scaling;
      uy = P.u[n + i] / P.M.scaling;
    }
    bad |= thermal_relax(P.M, f, g, P.in_init != 0, ux, uy, rho, T, kn);
    P.rho[i] = rho;
    if (!P.in_init) {
      P.u[i] = ux * P.M.scaling;
      P.u[n + i] = uy * P.M.scaling;
    }
    P.T[i] = T;
    P.mask[i] = kn;
#pragma unroll
    for (int q = 0; q < TH_Q; ++q) {
      P.f[q * n + i] = f[q];
      P.g[q * n + i] = g[q];
    }
  }
  if (bad) atomicOr(P.status, bad);
}

// Equilibrium initialisation (CompressibleCFDSolver::initializeDistributions,
// CompressibleCFDSolver.h:849-899): f = f^eq(rho, u, T) of the quartic
// equilibrium, g = f^eq T (2 C_v - D), from the device fields rho, u (scaled)
// and T.
__global__ void __launch_bounds__(256) k_thermal_init(const __grid_constant__ ThermalPoint P) {
  const long long n = P.n;
  const ThermalModel& M = P.M;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double rho = P.rho[i], T = P.T[i];
    const double ux = P.u[i] / M.scaling, uy = P.u[n + i] / M.scaling;
    const EqCoef k = eq_coef(M, true, ux, uy, T);  // the initialisation uses the quartic form
    const double Tg = T * M.gfac;
    static_for<0, TH_NG>([&](auto Gc) {
      constexpr int G = decltype(Gc)::value;
      double E, Ox, Oy, Oxy;
      eq_parts<G>(M, k, E, Ox, Oy, Oxy);
      const double wr = M.w[G] * rho;
      static_for<0, TH_Q>([&](auto Ic) {
        constexpr int I = decltype(Ic)::value;
        if constexpr (SD2Q25H::group(I) == G) {
          const double feq = wr * eq_member<I>(E, Ox, Oy, Oxy);
          P.f[(long long)I * n + i] = feq;
          P.g[(long long)I * n + i] = feq * Tg;
        }
      });
    });
  }
}

}  // namespace natgpu
