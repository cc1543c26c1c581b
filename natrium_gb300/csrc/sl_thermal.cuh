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
// the temperature uses sum |e - u|^2 f = sum |e|^2 f - u . j.  The plain
// form is FP64 throughout; the GB300's FP64 rate makes it FP64-pipe bound,
// so the formulation minimises FP64 operations per node.
//
// FP32 deviation form (Real = float): f - w_i and g - w_i g_ref are stored
// and streamed in float, the windows in difference form
// v_j0 + sum_{j != j0} w_j (v_j - v_j0) (j0: the dominant weight), and the
// collision works on deviations throughout: rho - 1 = sum (f - w), T - 1 and
// P - 1 (P: the equilibrium polynomial) are formed without cancellation,
// f^eq - w = w (rho (P - 1) + (rho - 1)) and g^eq - w g_ref =
// g_fac ((f^eq - w) T + w (T - 1)) + w (g_fac - g_ref).
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

// Coefficients of the equilibrium polynomial P(e) with f^eq_i = w_i rho P(e_i),
// kept as P - 1:
//   even part  E - 1 = c0m1 + kx X^2 + ky Y^2 + k4xxxx Hxxxx + k4xxyy Hxxyy + k4yyyy Hyyyy
//   odd in x   Ox = kox X + k3xxx Hxxx + k3xyy Hxyy
//   odd in y   Oy = koy Y + k3xxy Hxxy + k3yyy Hyyy
//   odd in xy  Oxy = kxy X Y + k4xxxy Hxxxy + k4xyyy Hxyyy
// and P(sx X, sy Y) - 1 = (E - 1) + sx Ox + sy Oy + sx sy Oxy.  Term by term
// this is the reference's polynomial (Equilibria.h:145-263):
//   1 + u.e/c^2 + (u.e)^2/(2 c^4) - u^2/(2 c^2) + (T-1)/(2 c^2) (|e|^2 - D c^2)
//   + a3 : H3 / (6 c^6) + a4 : H4 / (24 c^8)
// with the Hermite tensors H3, H4 of AuxiliaryCollisionFunctions.h:520-566
// and a3, a4 the velocity/temperature tensors of Equilibria.h:157-181.
template <class Real>
struct EqCoef {
  Real c0m1, kx, ky, kxy, kox, koy;
  Real k3xxx, k3xxy, k3xyy, k3yyy;
  Real k4xxxx, k4xxxy, k4xxyy, k4xyyy, k4yyyy;
};

template <class Real>
__device__ __forceinline__ EqCoef<Real> eq_coef(const ThermalModelT<Real>& M, bool quartic, Real ux, Real uy,
                                                Real Tm1_in) {
  const Real cs2 = M.cs2;
  const Real i2 = Real(1) / (Real(2) * cs2);
  const Real i4 = Real(1) / (Real(2) * cs2 * cs2);
  EqCoef<Real> k;
  const Real Tm1 = quartic ? Tm1_in : Real(0);
  k.c0m1 = -(ux * ux + uy * uy) * i2 - Tm1;
  k.kx = ux * ux * i4 + Tm1 * i2;
  k.ky = uy * uy * i4 + Tm1 * i2;
  k.kxy = ux * uy * (Real(2) * i4);
  k.kox = ux * (Real(2) * i2);
  k.koy = uy * (Real(2) * i2);
  if (quartic) {
    const Real T1 = cs2 * Tm1;
    const Real c3 = Real(1) / (Real(6) * cs2 * cs2 * cs2);
    const Real c4 = Real(1) / (Real(24) * cs2 * cs2 * cs2 * cs2);
    const Real ux2 = ux * ux, uy2 = uy * uy, uxy = ux * uy;
    k.k3xxx = c3 * (ux2 * ux + Real(3) * T1 * ux);
    k.k3xxy = Real(3) * c3 * (ux2 * uy + T1 * uy);
    k.k3xyy = Real(3) * c3 * (ux * uy2 + T1 * ux);
    k.k3yyy = c3 * (uy2 * uy + Real(3) * T1 * uy);
    k.k4xxxx = c4 * (ux2 * ux2 + Real(6) * T1 * ux2 + Real(3) * T1 * T1);
    k.k4yyyy = c4 * (uy2 * uy2 + Real(6) * T1 * uy2 + Real(3) * T1 * T1);
    k.k4xxxy = Real(4) * c4 * (ux2 * uxy + Real(3) * T1 * uxy);
    k.k4xyyy = Real(4) * c4 * (uxy * uy2 + Real(3) * T1 * uxy);
    k.k4xxyy = Real(6) * c4 * (ux2 * uy2 + T1 * (ux2 + uy2) + T1 * T1);
  } else {
    k.k3xxx = k.k3xxy = k.k3xyy = k.k3yyy = Real(0);
    k.k4xxxx = k.k4xxxy = k.k4xxyy = k.k4xyyy = k.k4yyyy = Real(0);
  }
  return k;
}

// Group parts (E - 1, Ox, Oy, Oxy) of the equilibrium polynomial for group G.
template <int G, class Real>
__device__ __forceinline__ void eq_parts(const ThermalModelT<Real>& M, const EqCoef<Real>& k, Real& Em1, Real& Ox,
                                         Real& Oy, Real& Oxy) {
  constexpr bool HX = SD2Q25H::gx(G) != 0, HY = SD2Q25H::gy(G) != 0;
  const Real X = M.X[G], Y = M.Y[G];
  Real E = k.c0m1;
  if constexpr (HX) E = fma(k.kx, X * X, E);
  if constexpr (HY) E = fma(k.ky, Y * Y, E);
  E = fma(k.k4xxxx, M.h4[G][0], E);
  E = fma(k.k4xxyy, M.h4[G][2], E);
  E = fma(k.k4yyyy, M.h4[G][4], E);
  Em1 = E;
  Ox = Oy = Oxy = Real(0);
  if constexpr (HX) Ox = fma(k.kox, X, fma(k.k3xxx, M.h3[G][0], k.k3xyy * M.h3[G][2]));
  if constexpr (HY) Oy = fma(k.koy, Y, fma(k.k3xxy, M.h3[G][1], k.k3yyy * M.h3[G][3]));
  if constexpr (HX && HY) Oxy = fma(k.kxy, X * Y, fma(k.k4xxxy, M.h4[G][1], k.k4xyyy * M.h4[G][3]));
}

// P - 1 for direction I from its group's parts.
template <int I, class Real>
__device__ __forceinline__ Real eq_member(Real Em1, Real Ox, Real Oy, Real Oxy) {
  constexpr int G = SD2Q25H::group(I);
  constexpr int sx = SD2Q25H::sgn(I, 0), sy = SD2Q25H::sgn(I, 1);
  constexpr bool HX = SD2Q25H::gx(G) != 0, HY = SD2Q25H::gy(G) != 0;
  Real a = Em1, b = Real(0);
  if constexpr (HX) a = sx > 0 ? a + Ox : a - Ox;
  if constexpr (HY) b = sy > 0 ? Oy : -Oy;
  if constexpr (HX && HY) b = (sx * sy > 0) ? b + Oxy : b - Oxy;
  return a + b;
}

// relaxWithG on one node.  f, g: the 25 post-streaming values (plain values
// for double, deviations for float), overwritten with the post-collision
// ones.  With given_u the velocity (unscaled) is the prescribed one
// (initialisation procedure), otherwise it is computed.  Returns the status
// bits (density underflow / NaN).
// f, g: the node's 25 + 25 values, indexable by direction (register arrays,
// or SmemPop views of a warp's shared-memory slots)
template <class Real, class FA, class GA>
__device__ __forceinline__ int thermal_relax(const ThermalModelT<Real>& M, FA& f, GA& g,
                                             bool given_u, Real& ux, Real& uy, double& rho_o, double& T_o,
                                             double& kn_o) {
  constexpr bool DEV = sizeof(Real) == 4;
  // ---- moments by symmetry group ----------------------------------------
  // DEV: r = rho - 1, s2 = sum |e|^2 (f - w), gsum = sum (g - w g_ref)
  Real r = Real(0), jx = Real(0), jy = Real(0), s2 = Real(0), gsum = Real(0);
  static_for<0, TH_NG>([&](auto Gc) {
    constexpr int G = decltype(Gc)::value;
    Real s = Real(0), sxs = Real(0), sys = Real(0);
    static_for<0, TH_Q>([&](auto Ic) {
      constexpr int I = decltype(Ic)::value;
      if constexpr (SD2Q25H::group(I) == G) {
        s += f[I];
        if constexpr (SD2Q25H::gx(G) != 0) sxs = SD2Q25H::sgn(I, 0) > 0 ? sxs + f[I] : sxs - f[I];
        if constexpr (SD2Q25H::gy(G) != 0) sys = SD2Q25H::sgn(I, 1) > 0 ? sys + f[I] : sys - f[I];
      }
    });
    r += s;
    if constexpr (G != 0) s2 = fma(M.e2[G], s, s2);
    if constexpr (SD2Q25H::gx(G) != 0) jx = fma(M.X[G], sxs, jx);
    if constexpr (SD2Q25H::gy(G) != 0) jy = fma(M.Y[G], sys, jy);
  });
#pragma unroll
  for (int i = 0; i < TH_Q; ++i) gsum += g[i];
  const Real rho = DEV ? Real(1) + r : r;
  int bad = 0;
  if (!(rho >= Real(1e-10))) bad = (rho != rho) ? ST_NAN : ST_DENSITY;
  const Real rinv = Real(1) / rho;
  Real vx = jx * rinv, vy = jy * rinv;
  // T = 0.5 / (rho C_v) sum_i (|e_i - u|^2 f_i / c_s^2 + g_i)   (AuxiliaryCollisionFunctions.h:289-307);
  // on deviations (sum w |e|^2 = D c_s^2, D + g_fac = 2 C_v):
  // T - 1 = ((g_ref - g_fac) + (s2 - u.j) / c_s^2 + gsum - 2 C_v (rho - 1)) / (2 rho C_v)
  Real T, Tm1;
  if constexpr (DEV) {
    Tm1 = ((M.gref - M.gfac) + (s2 - (vx * jx + vy * jy)) / M.cs2 + gsum - Real(2) * M.C_v * r) * rinv /
          (Real(2) * M.C_v);
    T = Real(1) + Tm1;
  } else {
    T = Real(0.5) * ((s2 - (vx * jx + vy * jy)) / M.cs2 + gsum) * rinv / M.C_v;
    Tm1 = T - Real(1);
  }
  if (given_u) {
    vx = ux;
    vy = uy;
  }
  // ---- relaxation parameters (CollisionSchemes.h:81-113) -----------------
  Real suth = Real(1);
  if (M.sutherland_set) suth = pow(T / Real(0.85), Real(0.7));
  const Real visc_tau = (M.tau - Real(0.5)) * suth / (T * rho) + Real(0.5);
  const Real omega = Real(1) / visc_tau;
  const Real Tg = T * M.gfac;  // g^eq = f^eq T (2 C_v - D)
  // f^eq (DEV: f^eq - w) = w fma(rho, P - 1, base); g^eq (DEV: - w g_ref) = f^eq Tg + w gadd
  const Real base = DEV ? r : rho;
  const Real gadd = DEV ? fma(M.gfac, Tm1, M.gfac - M.gref) : Real(0);
  const EqCoef<Real> k = eq_coef(M, M.quartic != 0, vx, vy, Tm1);
  Real kn = Real(0);
  if (!M.prandtl_set) {
    // single pass: f -= omega (f - f^eq), g -= omega (g - g^eq)
    static_for<0, TH_NG>([&](auto Gc) {
      constexpr int G = decltype(Gc)::value;
      Real Em1, Ox, Oy, Oxy;
      eq_parts<G>(M, k, Em1, Ox, Oy, Oxy);
      const Real wG = M.w[G], gw = wG * gadd;
      static_for<0, TH_Q>([&](auto Ic) {
        constexpr int I = decltype(Ic)::value;
        if constexpr (SD2Q25H::group(I) == G) {
          const Real feq = wG * fma(rho, eq_member<I>(Em1, Ox, Oy, Oxy), base);
          const Real fneq = f[I] - feq;
          kn = fma(fabs(fneq), M.winv[G], kn);
          f[I] = fma(-omega, fneq, f[I]);
          const Real gneq = g[I] - fma(feq, Tg, gw);
          g[I] = fma(-omega, gneq, g[I]);
        }
      });
    });
  } else {
    // Prandtl correction (CollisionSchemes.h:63-79, AuxiliaryCollisionFunctions.h:445-516):
    // pass 1 -> non-equilibrium parts, centred heat flux of f^neq and centred
    // flux of g^neq; pass 2 -> f = f^eq + (1 - omega) f^neq + (omega - omega_Pr) f*.
    Real qxxx = Real(0), qxxy = Real(0), qxyy = Real(0), qyyy = Real(0), fx = Real(0), fy = Real(0);
    static_for<0, TH_NG>([&](auto Gc) {
      constexpr int G = decltype(Gc)::value;
      Real Em1, Ox, Oy, Oxy;
      eq_parts<G>(M, k, Em1, Ox, Oy, Oxy);
      const Real wG = M.w[G], gw = wG * gadd;
      static_for<0, TH_Q>([&](auto Ic) {
        constexpr int I = decltype(Ic)::value;
        if constexpr (SD2Q25H::group(I) == G) {
          const Real feq = wG * fma(rho, eq_member<I>(Em1, Ox, Oy, Oxy), base);
          const Real fneq = f[I] - feq;
          const Real gneq = g[I] - fma(feq, Tg, gw);
          kn = fma(fabs(fneq), M.winv[G], kn);
          f[I] = fneq;
          g[I] = gneq;
          const Real dx = Real(SD2Q25H::sgn(I, 0)) * M.X[G] - vx;
          const Real dy = Real(SD2Q25H::sgn(I, 1)) * M.Y[G] - vy;
          const Real tx = dx * fneq, ty = dy * fneq;
          qxxx = fma(dx * dx, tx, qxxx);
          qxxy = fma(dx * dx, ty, qxxy);
          qxyy = fma(dy * dy, tx, qxyy);
          qyyy = fma(dy * dy, ty, qyyy);
          fx = fma(dx, gneq, fx);
          fy = fma(dy, gneq, fy);
        }
      });
    });
    const Real prandtl_tau = (visc_tau - Real(0.5)) / M.prandtl + Real(0.5);
    const Real pdiff = omega - Real(1) / prandtl_tau;
    const Real cs6 = Real(6) * M.cs2 * M.cs2 * M.cs2;
    const Real a3 = pdiff / cs6;  // f* = w (Q : H3) / (6 c^6)
    const Real ag = pdiff / T;    // g* = w (F . e) / T
    const Real om1 = Real(1) - omega;
    static_for<0, TH_NG>([&](auto Gc) {
      constexpr int G = decltype(Gc)::value;
      Real Em1, Ox, Oy, Oxy;
      eq_parts<G>(M, k, Em1, Ox, Oy, Oxy);
      const Real wG = M.w[G], gw = wG * gadd;
      // odd-in-x and odd-in-y parts of Q : H3 and of F . e for this group
      const Real qx = fma(qxxx, M.h3[G][0], Real(3) * qxyy * M.h3[G][2]);
      const Real qy = fma(Real(3) * qxxy, M.h3[G][1], qyyy * M.h3[G][3]);
      const Real gx = fx * M.X[G], gy = fy * M.Y[G];
      static_for<0, TH_Q>([&](auto Ic) {
        constexpr int I = decltype(Ic)::value;
        if constexpr (SD2Q25H::group(I) == G) {
          constexpr bool HX = SD2Q25H::gx(G) != 0, HY = SD2Q25H::gy(G) != 0;
          const Real sx = Real(SD2Q25H::sgn(I, 0)), sy = Real(SD2Q25H::sgn(I, 1));
          const Real feq = wG * fma(rho, eq_member<I>(Em1, Ox, Oy, Oxy), base);
          Real qh = Real(0), ge = Real(0);
          if constexpr (HX) {
            qh = sx * qx;
            ge = sx * gx;
          }
          if constexpr (HY) {
            qh = fma(sy, qy, qh);
            ge = fma(sy, gy, ge);
          }
          f[I] = fma(a3, wG * qh, fma(om1, f[I], feq));
          g[I] = fma(ag, wG * ge, fma(om1, g[I], fma(feq, Tg, gw)));
        }
      });
    });
  }
  rho_o = (double)rho;
  ux = vx;
  uy = vy;
  T_o = (double)T;
  kn_o = (double)(kn * (Real(1) / Real(TH_Q)));
  return bad;
}

// Window sum over j <= p: plain sum_j w_j v_j (double) or the difference form
// v_j0 + sum_{j != j0} w_j (v_j - v_j0) (float deviations).
template <class Real>
__device__ __forceinline__ Real th_wsum(const Real* w, const Real (&v)[PMAX1], int p, int j0) {
  if constexpr (sizeof(Real) == 4) {
    Real v0 = v[0];
#pragma unroll
    for (int j = 1; j < PMAX1; ++j) v0 = (j == j0) ? v[j] : v0;
    Real acc = Real(0);
#pragma unroll
    for (int j = 0; j < PMAX1; ++j)
      if (j <= p && j != j0) acc = fma(w[j], v[j] - v0, acc);
    return acc + v0;
  } else {
    Real acc = Real(0);
#pragma unroll
    for (int j = 0; j < PMAX1; ++j)
      if (j <= p) acc = fma(w[j], v[j], acc);
    return acc;
  }
}

// Fused step: stream f and g (same operator), then (COLLIDE) relaxWithG.
// The populations of one lane kept in its warp's shared-memory slots
// (stride 32 between directions).
template <class Real>
struct SmemPop {
  Real* p;
  __device__ __forceinline__ Real& operator[](int i) const { return p[i * 32]; }
};

// FORM 0: W warps per CTA, f and g of the node in 50 registers (FP32:
// 126 registers, 16 resident warps per SM).  FORM 1 / 2: 4 warps per CTA,
// the streamed f and g wait in the warp's shared-memory slots and the
// collision works on them there; the registers are capped for 5 / 6
// resident CTAs (20 / 24 warps per SM; the collision's temporaries then
// spill a little).  The autotuner picks the form.
template <int FORM, bool F32>
constexpr int th_minb() {
  return FORM == 1 ? 5 : (FORM == 2 ? 6 : (F32 ? 2 : 1));
}

// warps per CTA of each form (3: the register form with staged rows)
template <int FORM>
constexpr int th_warps() {
  return (FORM == 1 || FORM == 2) ? TH_WARPS_SS : TH_WARPS;
}

// 4-byte asynchronous global -> shared copies (the staged form's rows)
__device__ __forceinline__ void th_cp_async4(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void th_cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void th_cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// FORM 3 (FP32, compile-time order): the register form whose y-window rows
// arrive by cp.async in a per-warp double buffer, one direction ahead: the
// register form waits on its global loads (long-scoreboard stalls, 16
// resident warps at 124 registers); the copies in flight hold no registers.
//
// PC > 0: the order p as a compile-time constant (the window loops then run
// over p + 1 slots instead of PMAX1 predicated ones); PC = 0: any order.
template <class Real, bool COLLIDE, int W = TH_WARPS, int FORM = 0, int PC = 0>
__global__ void __launch_bounds__(32 * W, (th_minb<FORM, sizeof(Real) == 4>()))
    k_thermal_step(const __grid_constant__ ThermalStepT<Real> P) {
  __shared__ Real swx[ND_MAX][PER_MAX][PMAX1];
  __shared__ int soffx[ND_MAX][PER_MAX];
  __shared__ int sj0x[ND_MAX][PER_MAX];
  constexpr bool SS = FORM == 1 || FORM == 2;
  constexpr bool STG = FORM == 3;
  static_assert(!STG || (PC > 0 && PC < PMAX1 && sizeof(Real) == 4), "staged form: FP32, compile-time order");
  constexpr int NR = STG ? PC + 1 : 1;  // rows of a y window
  // stage buffers: directions in flight + 1 (three, two directions ahead,
  // measured the same as two on the 128 x 128-cell order-2 problem)
  constexpr int NB = STG ? 2 : 1;
  __shared__ Real bufs[W][4][TH_BWMAX + 1];
  __shared__ Real pops[SS ? W : 1][2][SS ? TH_Q : 1][32];
  // [warp][buffer][f, g][window row][x slot]
  __shared__ Real stg[STG ? W : 1][NB][2][NR][STG ? TH_BWMAX : 1];
  for (int i = threadIdx.x; i < ND_MAX * PER_MAX * PMAX1; i += blockDim.x)
    (&swx[0][0][0])[i] = (&P.tb.w[0][0][0][0])[i];
  for (int i = threadIdx.x; i < ND_MAX * PER_MAX; i += blockDim.x) {
    (&soffx[0][0])[i] = (&P.tb.off[0][0][0])[i];
    (&sj0x[0][0])[i] = (&P.tb.j0[0][0][0])[i];
  }
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wid = blockIdx.x * W + warp;
  if (wid >= P.nseg * P.ny) return;  // warp-uniform
  const int nx = P.nx, ny = P.ny, n = P.n;
  const int p = PC > 0 ? PC : P.tb.p, per = P.tb.per;
  const int seg = wid % P.nseg, y = wid / P.nseg;
  const int x0 = seg * 32, x = x0 + lane;
  const bool valid = x < nx;
  const int xs = valid ? x : x0;
  const int node = y * nx + xs;
  const int cx = xs % per, cy = y % per;
  // x position of this lane's first buffer slot (the buffer spans at most 64)
  const int gxa = ((x0 + P.tb.xl + lane) % nx + nx) % nx;
  const bool hasb = lane + 32 < P.tb.bw;
  int gxb = gxa + 32;  // x position of the lane's second buffer slot
  while (gxb >= nx) gxb -= nx;
  // wall node: its rows were streamed from the sparse rows into f_out / g_out
  const bool wall = COLLIDE && P.wall_bits && ((__ldg(P.wall_bits + wid) >> lane) & 1u);

  // FORM 3: copy direction A's window rows (its lane slots: the node's own x,
  // or the buffer slots gxa and gxb) into stage buffer A % NB; one commit
  // group per direction (empty past the last)
  auto stage = [&](auto Ac) {
    if constexpr (STG) {
      constexpr int A = decltype(Ac)::value;
      if constexpr (A < TH_Q) {
        constexpr int dx = SD2Q25H::dcls(A, 0), dy = SD2Q25H::dcls(A, 1);
        constexpr int b = A % NB;
        const Real* fsrc = P.f_in + (long long)A * n;
        const Real* gsrc = P.g_in + (long long)A * n;
        const int ys = dy >= 0 ? y + P.tb.offy[dy < 0 ? 0 : dy][cy] : y;
        const int ca = dx < 0 ? xs : gxa;
#pragma unroll
        for (int j = 0; j < (dy >= 0 ? NR : 1); ++j) {
          int rr = ys + j;
          rr -= rr >= ny ? ny : 0;
          rr -= rr >= ny ? ny : 0;
          const int o = rr * nx;
          th_cp_async4(&stg[warp][b][0][j][lane], fsrc + o + ca);
          th_cp_async4(&stg[warp][b][1][j][lane], gsrc + o + ca);
          if (dx >= 0 && hasb) {
            th_cp_async4(&stg[warp][b][0][j][lane + 32], fsrc + o + gxb);
            th_cp_async4(&stg[warp][b][1][j][lane + 32], gsrc + o + gxb);
          }
        }
      }
      th_cp_async_commit();
    }
  };

  // the step on the node's populations fs, gs (registers or shared memory)
  auto body = [&](auto& fs, auto& gs) {
  static_for<1, NB>([&](auto Sc) { stage(IC<decltype(Sc)::value>{}); });
  fs[0] = P.f_in[node];
  gs[0] = P.g_in[node];

  static_for<1, TH_Q>([&](auto Ic) {
    constexpr int A = decltype(Ic)::value;
    constexpr int dx = SD2Q25H::dcls(A, 0), dy = SD2Q25H::dcls(A, 1);
    const Real* __restrict__ fsrc = P.f_in + (long long)A * n;
    const Real* __restrict__ gsrc = P.g_in + (long long)A * n;
    // warp-uniform y window start (y + offy + j < 2 ny + p < 3 ny: two
    // conditional subtractions wrap a row index)
    const int ys = dy >= 0 ? y + P.tb.offy[dy < 0 ? 0 : dy][cy] : y;
    if constexpr (STG) {
      // the next NB - 1 directions' rows in flight; this direction's rows
      // (this lane's own copies) have landed
      stage(IC<A + NB - 1>{});
      th_cp_async_wait<NB - 1>();
    }
    // the y-window sums at x position gx (stage slot col in FORM 3)
    auto ysum = [&](int gx, int col, Real& vf, Real& vg) {
      if constexpr (STG) {
        constexpr int b = A % NB;
        if constexpr (dy >= 0) {
          Real af[PMAX1], ag[PMAX1];
#pragma unroll
          for (int j = 0; j < PMAX1; ++j) {
            af[j] = Real(0);
            ag[j] = Real(0);
            if (j < NR) {
              af[j] = stg[warp][b][0][j < NR ? j : 0][col];
              ag[j] = stg[warp][b][1][j < NR ? j : 0][col];
            }
          }
          vf = th_wsum<Real>(P.tb.w[1][dy][cy], af, p, P.tb.j0[1][dy][cy]);
          vg = th_wsum<Real>(P.tb.w[1][dy][cy], ag, p, P.tb.j0[1][dy][cy]);
        } else {
          vf = stg[warp][b][0][0][col];
          vg = stg[warp][b][1][0][col];
        }
      } else if constexpr (dy >= 0) {
        Real af[PMAX1], ag[PMAX1];
#pragma unroll
        for (int j = 0; j < PMAX1; ++j) {
          af[j] = Real(0);
          ag[j] = Real(0);
          if (j <= p) {
            int rr = ys + j;
            rr -= rr >= ny ? ny : 0;
            rr -= rr >= ny ? ny : 0;
            const int o = rr * nx + gx;
            af[j] = __ldg(fsrc + o);
            ag[j] = __ldg(gsrc + o);
          }
        }
        vf = th_wsum<Real>(P.tb.w[1][dy][cy], af, p, P.tb.j0[1][dy][cy]);
        vg = th_wsum<Real>(P.tb.w[1][dy][cy], ag, p, P.tb.j0[1][dy][cy]);
      } else {
        vf = __ldg(fsrc + ys * nx + gx);
        vg = __ldg(gsrc + ys * nx + gx);
      }
    };
    if constexpr (dx < 0) {
      ysum(xs, lane, fs[A], gs[A]);
    } else {
      Real* bf = &bufs[warp][(th_xorder(A) & 1) * 2][0];
      Real* bg = &bufs[warp][(th_xorder(A) & 1) * 2 + 1][0];
      {
        Real vf, vg;
        ysum(gxa, lane, vf, vg);
        bf[lane] = vf;
        bg[lane] = vg;
        if (hasb) {
          ysum(gxb, lane + 32, vf, vg);
          bf[lane + 32] = vf;
          bg[lane + 32] = vg;
        }
      }
      __syncwarp();
      const int st = lane * (valid ? 1 : 0) + soffx[dx][cx] - P.tb.xl;
      Real xf[PMAX1], xg[PMAX1];
#pragma unroll
      for (int j = 0; j < PMAX1; ++j) {
        xf[j] = Real(0);
        xg[j] = Real(0);
        if (j <= p) {
          xf[j] = bf[st + j];
          xg[j] = bg[st + j];
        }
      }
      fs[A] = th_wsum<Real>(swx[dx][cx], xf, p, sj0x[dx][cx]);
      gs[A] = th_wsum<Real>(swx[dx][cx], xg, p, sj0x[dx][cx]);
    }
  });

  if (!valid) return;
  if constexpr (COLLIDE) {
    if (wall) {
      // the rows kernel's output: wait for that grid (a no-op unless this
      // kernel was launched as its programmatic dependent); plain loads, this
      // thread writes the same words below
      asm volatile("griddepcontrol.wait;" ::: "memory");
#pragma unroll
      for (int q = 1; q < TH_Q; ++q) {
        fs[q] = P.f_out[(long long)q * n + node];
        gs[q] = P.g_out[(long long)q * n + node];
      }
    }
    Real ux = Real(0), uy = Real(0);
    double rho, T, kn;
    const int bad = thermal_relax<Real>(P.M, fs, gs, false, ux, uy, rho, T, kn);
    if (bad) atomicOr(P.status, bad);
    if (P.write_macro) {
      P.rho[node] = rho;
      P.u[node] = (double)ux * P.M.scaling;
      P.u[n + node] = (double)uy * P.M.scaling;
      P.T[node] = T;
      P.mask[node] = kn;
    }
  }
#pragma unroll
  for (int q = 0; q < TH_Q; ++q) {
    P.f_out[(long long)q * n + node] = fs[q];
    P.g_out[(long long)q * n + node] = gs[q];
  }
  };
  if constexpr (SS) {
    SmemPop<Real> fsm{&pops[warp][0][0][lane]}, gsm{&pops[warp][1][0][lane]};
    body(fsm, gsm);
  } else {
    Real fs[TH_Q], gs[TH_Q];
    body(fs, gs);
  }
}

// Wall nodes of the two-population model:
//  1. k_thermal_rows: one thread per sparse row (node, direction) streams f
//     and g of that row into the output buffers (constant slots: f, g);
//  2. the collision of those nodes: on the Cartesian lattice k_thermal_step
//     itself (launched after the rows as their programmatic dependent, so
//     the lattice streams while the rows run; ThermalStepT::wall_bits marks
//     the nodes, whose lanes wait for the rows grid); on mapped cells, where every node is a wall node,
//     k_thermal_collide_nodes, one thread per node, rest population from the
//     input.
// (One thread walking all 24 rows of its node, ~430 dependent loads, left
// the few hundred warps latency-bound: ~50 us for 3,000 nodes.  A separate
// collision pass after the step cost 11.7 us (FP32) / 31 us (FP64) per step
// on the 128 x 128 cell, order-2 two-dimensional Riemann problem with four
// open faces.)
template <class Real>
__global__ void __launch_bounds__(256) k_thermal_rows(const __grid_constant__ ThermalStepT<Real> P, int nrows,
                                                      const int* __restrict__ bnode, const int* __restrict__ ptr,
                                                      const int* __restrict__ col, const Real* __restrict__ w,
                                                      const double* __restrict__ cst) {
  constexpr bool DEV = sizeof(Real) == 4;
  const int n = P.n;
  // the step kernel may start now (its wall lanes wait for this grid)
  asm volatile("griddepcontrol.launch_dependents;");
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    const int node = bnode[r / (TH_Q - 1)];
    const int a = r % (TH_Q - 1) + 1;
    Real af = Real(cst[4 * r + (DEV ? 1 : 0)]), ag = Real(cst[4 * r + (DEV ? 3 : 2)]);
    for (int j = ptr[r]; j < ptr[r + 1]; ++j) {
      const int c = col[j];
      af = fma(w[j], P.f_in[c], af);
      ag = fma(w[j], P.g_in[c], ag);
    }
    P.f_out[(long long)a * n + node] = af;
    P.g_out[(long long)a * n + node] = ag;
  }
}

template <class Real>
__global__ void __launch_bounds__(128) k_thermal_collide_nodes(const __grid_constant__ ThermalStepT<Real> P, int nbn,
                                                               const int* __restrict__ bnode) {
  const int n = P.n;
  int bad = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nbn; k += gridDim.x * blockDim.x) {
    const int node = bnode[k];
    Real f[TH_Q], g[TH_Q];
    f[0] = P.f_in[node];
    g[0] = P.g_in[node];
#pragma unroll
    for (int a = 1; a < TH_Q; ++a) {
      f[a] = P.f_out[(long long)a * n + node];
      g[a] = P.g_out[(long long)a * n + node];
    }
    Real ux = Real(0), uy = Real(0);
    double rho, T, kn;
    bad |= thermal_relax<Real>(P.M, f, g, false, ux, uy, rho, T, kn);
    if (P.write_macro) {
      P.rho[node] = rho;
      P.u[node] = (double)ux * P.M.scaling;
      P.u[n + node] = (double)uy * P.M.scaling;
      P.T[node] = T;
      P.mask[node] = kn;
    }
#pragma unroll
    for (int q = 0; q < TH_Q; ++q) {
      P.f_out[(long long)q * n + node] = f[q];
      P.g_out[(long long)q * n + node] = g[q];
    }
  }
  if (bad) atomicOr(P.status, bad);
}

// Collision only (CollisionOperator::collideAll(f, g, ...)), in place.
template <class Real>
__global__ void __launch_bounds__(256) k_thermal_collide(const __grid_constant__ ThermalPointT<Real> P) {
  const long long n = P.n;
  int bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    Real f[TH_Q], g[TH_Q];
#pragma unroll
    for (int q = 0; q < TH_Q; ++q) {
      f[q] = P.f[q * n + i];
      g[q] = P.g[q * n + i];
    }
    Real ux = Real(0), uy = Real(0);
    double rho, T, kn;
    if (P.in_init) {
      ux = (Real)(P.u[i] / P.M.scaling);
      uy = (Real)(P.u[n + i] / P.M.scaling);
    }
    bad |= thermal_relax<Real>(P.M, f, g, P.in_init != 0, ux, uy, rho, T, kn);
    P.rho[i] = rho;
    if (!P.in_init) {
      P.u[i] = (double)ux * P.M.scaling;
      P.u[n + i] = (double)uy * P.M.scaling;
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
// and T.  Evaluated in FP64; the float form stores the deviations.
template <class Real>
__global__ void __launch_bounds__(256) k_thermal_init(const __grid_constant__ ThermalPointT<double> P, Real* f,
                                                      Real* g) {
  constexpr bool DEV = sizeof(Real) == 4;
  const long long n = P.n;
  const ThermalModelT<double>& M = P.M;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double rho = P.rho[i], T = P.T[i];
    const double ux = P.u[i] / M.scaling, uy = P.u[n + i] / M.scaling;
    const EqCoef<double> k = eq_coef<double>(M, true, ux, uy, T - 1.0);  // always the quartic form
    const double Tg = T * M.gfac;
    static_for<0, TH_NG>([&](auto Gc) {
      constexpr int G = decltype(Gc)::value;
      double Em1, Ox, Oy, Oxy;
      eq_parts<G>(M, k, Em1, Ox, Oy, Oxy);
      static_for<0, TH_Q>([&](auto Ic) {
        constexpr int I = decltype(Ic)::value;
        if constexpr (SD2Q25H::group(I) == G) {
          const double pm1 = eq_member<I>(Em1, Ox, Oy, Oxy);
          if constexpr (DEV) {
            // f - w = w (rho (P - 1) + rho - 1); g - w g_ref = (f - w) T g_fac + w (T g_fac - g_ref)
            const double fd = M.w[G] * fma(rho, pm1, rho - 1.0);
            f[(long long)I * n + i] = (Real)fd;
            g[(long long)I * n + i] = (Real)fma(fd, Tg, M.w[G] * (Tg - M.gref));
          } else {
            const double feq = M.w[G] * fma(rho, pm1, rho);
            f[(long long)I * n + i] = feq;
            g[(long long)I * n + i] = feq * Tg;
          }
        }
      });
    });
  }
}

}  // namespace natgpu
