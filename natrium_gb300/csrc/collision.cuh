// Collision epilogues of the fused stream + collide kernel.
//
// Two storage modes:
//   DEV == false (plain FP64): v holds f.
//   DEV == true  (FP32 deviation): v holds g = f - r, where r is the model's
//       rest state (the equilibrium at rho = 1, u = 0: r_i = w_i for BGK and
//       KBC; the incompressible equilibrium at rho = 1 for BGK_INCOMPRESSIBLE).
//       Every quantity is computed in deviation form so that float keeps the
//       small non-equilibrium part accurate.
// u is the unscaled velocity (lattice units, c_s^2 = 1/3); the reference
// stores scaling * u (CollisionOperator.h:79-82).
#pragma once

#include <math.h>

#include "stencils.cuh"

namespace natgpu {

// Neumaier-compensated running sum (float moments of the FP32 path).
template <class Real>
struct CSum {
  Real s = Real(0), c = Real(0);
  __device__ __forceinline__ void add(Real x) {
    Real t = s + x;
    c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ Real value() const { return s + c; }
};

template <class S>
__host__ __device__ constexpr int opp(int i);

// first direction i < opp(i) with a non-zero component along axis a
template <class S>
__host__ __device__ constexpr int first_pair(int a) {
  for (int i = 1; i < S::Q; ++i)
    if (i < opp<S>(i) && S::e(i, a) != 0) return i;
  return -1;
}

// Moments: density (or its deviation) and momentum.  COMP selects
// compensated summation (used for the float path).
template <class S, bool COMP, class Real>
__device__ __forceinline__ void moments(const Real (&v)[S::Q], Real& m0,
                                        Real (&j)[3]) {
  if constexpr (COMP) {
    CSum<Real> a0, ax, ay, az;
    static_for<0, S::Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      a0.add(v[i]);
      if constexpr (S::e(i, 0) > 0) ax.add(v[i]);
      if constexpr (S::e(i, 0) < 0) ax.add(-v[i]);
      if constexpr (S::e(i, 1) > 0) ay.add(v[i]);
      if constexpr (S::e(i, 1) < 0) ay.add(-v[i]);
      if constexpr (S::e(i, 2) > 0) az.add(v[i]);
      if constexpr (S::e(i, 2) < 0) az.add(-v[i]);
    });
    m0 = a0.value();
    j[0] = ax.value();
    j[1] = ay.value();
    j[2] = az.value();
  } else {
    // per pair of opposite directions (i, i'): s = v_i + v_i' enters the
    // density, d = v_i - v_i' each momentum component e_i has (fewer
    // additions than summing the Q values into four accumulators)
    Real a0 = v[0], jj[3] = {0, 0, 0};
    static_for<1, S::Q>([&](auto I) {
      constexpr int i = decltype(I)::value;
      constexpr int o = opp<S>(i);
      if constexpr (i < o) {
        a0 += v[i] + v[o];
        const Real d = v[i] - v[o];
        static_for<0, 3>([&](auto A) {
          constexpr int a = decltype(A)::value;
          constexpr int e = S::e(i, a);
          if constexpr (e != 0) {
            if constexpr (i == first_pair<S>(a))
              jj[a] = e > 0 ? d : -d;
            else
              jj[a] = e > 0 ? jj[a] + d : jj[a] - d;
          }
        });
      }
    });
    m0 = a0;
    j[0] = jj[0];
    j[1] = jj[1];
    j[2] = jj[2];
  }
}

// e_i . u with compile-time e
template <class S, int i, class Real>
__device__ __forceinline__ Real edot(const Real (&u)[3]) {
  Real r = Real(0);
  if constexpr (S::e(i, 0) == 1) r += u[0];
  if constexpr (S::e(i, 0) == -1) r -= u[0];
  if constexpr (S::e(i, 1) == 1) r += u[1];
  if constexpr (S::e(i, 1) == -1) r -= u[1];
  if constexpr (S::D == 3) {
    if constexpr (S::e(i, 2) == 1) r += u[2];
    if constexpr (S::e(i, 2) == -1) r -= u[2];
  }
  return r;
}

// index of the direction opposite to i (e_opp = -e_i)
template <class S>
__host__ __device__ constexpr int opp(int i) {
  for (int j = 0; j < S::Q; ++j)
    if (S::e(j, 0) == -S::e(i, 0) && S::e(j, 1) == -S::e(i, 1) && S::e(j, 2) == -S::e(i, 2)) return j;
  return -1;
}

// ---------------------------------------------------------------------------
// BGK with the second-order equilibrium
// (collision_advanced/CollisionSchemes.h:28-41, Equilibria.h:33-83).
// Returns the density.  If given_u, u is input (inInitializationProcedure).
//
// Evaluated per pair of opposite directions (i, i'): with c = e_i . u,
//   feq_{i,i'} = w rho (1 - 1.5 u^2 + 4.5 c^2) +- 3 w rho c,
// and the relaxation f + omega (feq - f) = (1 - omega) f + omega feq, so a
// pair costs one even and one odd term (the same arithmetic as the
// reference's per-direction form, regrouped; in the deviation storage the
// even term carries w m0 instead of w).
// ---------------------------------------------------------------------------
template <class S, bool DEV, bool COMP, class Real>
__device__ __forceinline__ Real collide_bgk(Real (&v)[S::Q], Real inv_tau,
                                            Real (&u)[3], bool given_u) {
  Real m0, j[3];
  moments<S, COMP>(v, m0, j);
  const Real rho = DEV ? (Real(1) + m0) : m0;
  if (!given_u) {
    const Real inv = Real(1) / rho;
    u[0] = j[0] * inv;
    u[1] = j[1] * inv;
    u[2] = (S::D == 3) ? j[2] * inv : Real(0);
  }
  const Real uu = Real(1.5) * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  const Real keep = Real(1) - inv_tau;  // 1 - omega
  const Real orho = inv_tau * rho;
  // even part without the 4.5 c^2 term, times omega: omega w (rho (1 - uu))
  // (plain) or omega w (m0 - rho uu) (deviation)
  const Real base = DEV ? inv_tau * m0 - orho * uu : orho - orho * uu;
  static_for<0, S::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int o = opp<S>(i);
    if constexpr (i == 0) {
      v[0] = fma(v[0], keep, Real(S::w(0)) * base);
    } else if constexpr (i < o) {
      const Real c = edot<S, i>(u);
      const Real ow = Real(S::w(i)) * orho;                       // omega w rho
      const Real even = fma(Real(4.5) * ow * c, c, Real(S::w(i)) * base);
      const Real k3 = Real(3) * ow;                               // odd term 3 omega w rho c
      v[i] = fma(v[i], keep, fma(k3, c, even));
      v[o] = fma(v[o], keep, fma(-k3, c, even));
    }
  });
  return rho;
}

// ---------------------------------------------------------------------------
// BGK with a constant body force F: the advanced collision of the time loop
// (CollisionOperator.h:76-90, AuxiliaryCollisionFunctions.h:332-414) and the
// legacy BGKStandard's GUO scheme (collision/BGKStandard.cpp:128-133, 222-225
// for D2Q9; :374-380, 470-473 for D3Q19).
// dF = dt F / scaling (unscaled momentum gained per step).
//   scheme 1 (SHIFTING_VELOCITY): equilibrium velocity u + tau dF / rho;
//   scheme 2 (EXACT_DIFFERENCE): relax with u, then
//     f += f^eq(rho, u + dF / rho) - f^eq(rho, u);
//   scheme 3 (GUO): equilibrium velocity u' = u + dF / (2 rho), then
//     f_i += w_i (1 - omega/2) (3 e_i.dF - 3 scaling u'.dF + 9 (e_i.u')(e_i.dF))
//     (collision/ExternalForceFunctions.h:119-200, applyGuoForcingD2Q9, written
//     in unscaled variables: its u.F term carries the stencil scaling, as in
//     the reference).  For D3Q19 the reference adds that source term to a
//     local copy after the relaxed values are stored (BGKStandard.cpp:441-473),
//     so only the shifted equilibrium acts; restated as written.
// All report the velocity u + dF / (2 rho).  Not applied with a prescribed
// velocity (inInitializationProcedure).  Returns rho; tgt receives the mass
// and momentum the collision adds (the FP32 projection's targets).
// ---------------------------------------------------------------------------
template <class S>
__host__ __device__ constexpr bool guo_source() {
  return S::Q == 9;  // D2Q9; the D3Q19 source term is discarded by the reference
}

template <class S, bool DEV, bool COMP, class Real>
__device__ __forceinline__ Real collide_bgk_force(Real (&v)[S::Q], Real inv_tau, Real tau, Real (&u)[3],
                                                  bool given_u, const Real (&dF)[3], int scheme, Real scaling,
                                                  Real (&tgt)[4]) {
  if (given_u) return collide_bgk<S, DEV, COMP>(v, inv_tau, u, true);
  Real m0, j[3];
  moments<S, COMP>(v, m0, j);
  const Real rho = DEV ? (Real(1) + m0) : m0;
  const Real inv = Real(1) / rho;
  u[0] = j[0] * inv;
  u[1] = j[1] * inv;
  u[2] = (S::D == 3) ? j[2] * inv : Real(0);
  Real ue[3] = {u[0], u[1], u[2]};
  if (scheme == 1)
    for (int a = 0; a < S::D; ++a) ue[a] += tau * dF[a] * inv;
  if (scheme == 3)
    for (int a = 0; a < S::D; ++a) ue[a] += Real(0.5) * dF[a] * inv;
  Real us[3] = {ue[0], ue[1], ue[2]};
  if (scheme == 2)
    for (int a = 0; a < S::D; ++a) us[a] += dF[a] * inv;
  const Real uu = Real(1.5) * (ue[0] * ue[0] + ue[1] * ue[1] + ue[2] * ue[2]);
  const Real uus = Real(1.5) * (us[0] * us[0] + us[1] * us[1] + us[2] * us[2]);
  const Real guo = (Real(1) - Real(0.5) * inv_tau);  // 1 - omega / 2
  const Real uF = ue[0] * dF[0] + ue[1] * dF[1] + ue[2] * dF[2];
  static_for<0, S::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const Real ee = Real(3) * edot<S, i>(ue);
    const Real poly = ee * (Real(1) + Real(0.5) * ee) - uu;
    Real eq;
    if constexpr (DEV)
      eq = Real(S::w(i)) * (m0 + rho * poly);
    else
      eq = Real(S::w(i)) * rho * (Real(1) + poly);
    v[i] = v[i] - inv_tau * (v[i] - eq);
    if (scheme == 2) {
      const Real es = Real(3) * edot<S, i>(us);
      const Real polys = es * (Real(1) + Real(0.5) * es) - uus;
      v[i] += Real(S::w(i)) * rho * (polys - poly);
    }
    if constexpr (guo_source<S>()) {
      if (scheme == 3) {
        const Real eF = edot<S, i>(dF);
        const Real eu = edot<S, i>(ue);
        v[i] += Real(S::w(i)) * guo * (Real(3) * eF - Real(3) * scaling * uF + Real(9) * eu * eF);
      }
    }
  });
  for (int a = 0; a < S::D; ++a) u[a] += Real(0.5) * dF[a] * inv;
  // mass and momentum added: dF for schemes 1 and 2; for GUO the relaxation
  // towards u' adds omega dF / 2 and the source term (1 - omega/2) dF, and the
  // source's mass is 3 (1 - omega/2)(1 - scaling) u'.dF
  tgt[0] = Real(0);
  for (int a = 0; a < 3; ++a) tgt[1 + a] = dF[a];
  if (scheme == 3) {
    if constexpr (guo_source<S>()) {
      tgt[0] = Real(3) * guo * (Real(1) - scaling) * uF;
    } else {
      for (int a = 0; a < 3; ++a) tgt[1 + a] = Real(0.5) * inv_tau * dF[a];
    }
  }
  return rho;
}

// ---------------------------------------------------------------------------
// BGK incompressible, D2Q9 only (collision/BGKIncompressible.cpp:62-190):
// feq_0 = -4 sigma rho + 4/9 (1 + usq), feq_1..4 = lambda rho + 1/9 (1 + ...),
// feq_5..8 = gamma rho + rho/36 (1 + ...), lambda = 1/3, gamma = 1/12,
// sigma = lambda + gamma.  (The reference weights directions 5-8 with rho and
// 0-4 without; kept as written.)
// ---------------------------------------------------------------------------
__host__ __device__ constexpr double inc_c(int i) {
  return i == 0 ? -4.0 * (1.0 / 3.0 + 1.0 / 12.0) : (i <= 4 ? 1.0 / 3.0 : 1.0 / 12.0);
}
__host__ __device__ constexpr double inc_w(int i) {
  return i == 0 ? 4.0 / 9.0 : (i <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
}
// rest state of the incompressible model (rho = 1, u = 0)
__host__ __device__ constexpr double inc_rest(int i) { return inc_c(i) + inc_w(i); }

template <bool DEV, bool COMP, class Real>
__device__ __forceinline__ Real collide_bgk_inc(Real (&v)[9], Real inv_tau,
                                                Real (&u)[3], bool given_u) {
  using S = SD2Q9;
  Real m0, j[3];
  moments<S, COMP>(v, m0, j);
  const Real rho = DEV ? (Real(1) + m0) : m0;
  if (!given_u) {
    const Real inv = Real(1) / rho;
    u[0] = j[0] * inv;
    u[1] = j[1] * inv;
    u[2] = Real(0);
  }
  const Real usq = -Real(1.5) * (u[0] * u[0] + u[1] * u[1]);
  static_for<0, 9>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const Real ue = Real(3) * edot<S, i>(u);
    const Real poly = ue * (Real(1) + Real(0.5) * ue) + usq;
    Real eq;
    if constexpr (DEV) {
      // feq - rest, written so float keeps the small part
      if constexpr (i >= 5)
        eq = Real(inc_c(i)) * m0 + Real(inc_w(i)) * (m0 + rho * poly);
      else
        eq = Real(inc_c(i)) * m0 + Real(inc_w(i)) * poly;
    } else {
      if constexpr (i >= 5)
        eq = Real(inc_c(i)) * rho + Real(inc_w(i)) * rho * (Real(1) + poly);
      else
        eq = Real(inc_c(i)) * rho + Real(inc_w(i)) * (Real(1) + poly);
    }
    v[i] = v[i] - inv_tau * (v[i] - eq);
  });
  return rho;
}

// ---------------------------------------------------------------------------
// KBC (entropic multi-relaxation), D2Q9 as collision/KBCStandard.cpp:88-497
// (KBC_C: the shear part keeps the trace), extended to D3Q27 with the same
// construction (no reference implementation for D3Q27).  Equilibrium in the
// product form of KBCStandard.cpp:26-63 / :250-271.
//   ds_i: shear part of f - feq (from the second-moment differences),
//   dh_i = (f_i - feq_i) - ds_i,
//   gamma = 1/beta - (2 - 1/beta) <ds|dh> / <dh|dh>, <x|y> = sum x y / feq,
//   gamma = 2 when <dh|dh> < 1e-16,  f_i -= beta (2 ds_i + gamma dh_i),
//   beta = 1 / (2 tau).
// ---------------------------------------------------------------------------
// 1 / x and sqrt(x): IEEE in FP64; with FAST in FP32 the hardware
// approximations (MUFU.RCP / MUFU.RSQ based, a few ulp, no special-case path)
template <bool FAST, class Real>
__device__ __forceinline__ Real approx_rcp(Real x) {
  if constexpr (FAST && sizeof(Real) == 4)
    return __fdividef(1.0f, x);
  else
    return Real(1) / x;
}
template <bool FAST, class Real>
__device__ __forceinline__ Real approx_sqrt(Real x) {
  if constexpr (FAST && sizeof(Real) == 4)
    return x * rsqrtf(x);
  else
    return sqrt(x);
}

// weights of a tensor-product stencil: w_i = prod_a w1(e_ia), w1(0) = 2/3,
// w1(+-1) = 1/6 (D2Q9, D3Q27), to a relative 1e-14
template <class S>
__host__ __device__ constexpr bool tensor_weights() {
  for (int i = 0; i < S::Q; ++i) {
    double p = 1.0;
    for (int a = 0; a < S::D; ++a) p *= S::e(i, a) == 0 ? 2.0 / 3.0 : 1.0 / 6.0;
    const double d = p - S::w(i);
    if (d > 1e-14 * p || -d > 1e-14 * p) return false;
  }
  return true;
}

template <class S, int i, class Real>
__device__ __forceinline__ Real kbc_shear(const Real (&M)[3][3]) {
  constexpr int ex = S::e(i, 0), ey = S::e(i, 1), ez = S::e(i, 2);
  constexpr int nz = (ex != 0) + (ey != 0) + (ez != 0);
  if constexpr (nz == 0) {
    return -(M[0][0] + M[1][1] + M[2][2]);
  } else if constexpr (nz == 1) {
    constexpr int a = ex != 0 ? 0 : (ey != 0 ? 1 : 2);
    return Real(0.5) * M[a][a];
  } else if constexpr (nz == 2) {
    constexpr int a = ex != 0 ? 0 : 1;
    constexpr int b = ez != 0 ? 2 : 1;
    constexpr int sgn = S::e(i, a) * S::e(i, b);
    return Real(0.25 * sgn) * M[a][b];
  } else {
    return Real(0);
  }
}

template <class S, bool DEV, bool COMP, class Real>
__device__ __forceinline__ Real collide_kbc(Real (&v)[S::Q], Real tau,
                                            Real (&u)[3], bool given_u) {
  Real m0, j[3];
  moments<S, COMP>(v, m0, j);
  const Real rho = DEV ? (Real(1) + m0) : m0;
  const Real irho = Real(1) / rho;
  if (!given_u) {
    u[0] = j[0] * irho;
    u[1] = j[1] * irho;
    u[2] = (S::D == 3) ? j[2] * irho : Real(0);
  }
  // per axis: factor - 1 for c = -1, 0, +1 (stable small-number form of
  // base = 2 - sqrt(1 + 3u^2), post = (2u + sqrt(1+3u^2)) / (1 - u)), and
  // the reciprocals of the factors, 1 / base, 1 / (base post), post / base,
  // from the two reciprocals 1 / base and 1 / post.  In the FP32 deviation
  // path these use the hardware's approximate reciprocal and square root
  // (a few ulp): the factors enter f^eq as corrections of order u and u^2,
  // where that error stays below the storage's own rounding.
  Real dm[3][3], rinv[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const Real ua = u[a];
    const Real s = approx_sqrt<DEV>(Real(1) + Real(3) * ua * ua);
    const Real sm1 = Real(3) * ua * ua * approx_rcp<DEV>(Real(1) + s);     // s - 1
    const Real pm1 = (Real(3) * ua + sm1) * approx_rcp<DEV>(Real(1) - ua);  // post - 1
    const Real rb = approx_rcp<DEV>(Real(1) - sm1);                         // 1 / base
    const Real ip = approx_rcp<DEV>(Real(1) + pm1);                         // 1 / post
    dm[a][1] = -sm1;                                       // base - 1
    dm[a][2] = pm1 - sm1 - sm1 * pm1;                      // base*post - 1
    dm[a][0] = (-sm1 - pm1) * ip;                          // base/post - 1
    rinv[a][1] = rb;
    rinv[a][2] = rb * ip;
    rinv[a][0] = (Real(1) + pm1) * rb;
  }
  // q_i = prod_a (1 + d_a) - 1 of direction i, f^eq_i = w_i rho (1 + q_i)
  auto qof = [&](auto I) -> Real {
    constexpr int i = decltype(I)::value;
    Real q = dm[0][S::e(i, 0) + 1];
#pragma unroll
    for (int a = 1; a < S::D; ++a) {
      const int c = (a == 1 ? S::e(i, 1) : S::e(i, 2)) + 1;
      const Real d = dm[a][c];
      q = fma(q, d, q + d);
    }
    return q;
  };
  // 1 / f^eq_i = (1 / (w_i rho)) prod_a 1 / (1 + d_a) from the per-axis
  // reciprocals above instead of one division per direction;
  // (1 / rho) / (1 + d_x) / (1 + d_y) per (c_x, c_y): nine products shared by
  // the directions of each pair.  With tensor-product weights (D2Q9, D3Q27:
  // w_i = prod_a w1(e_ia), w1(0) = 2/3, w1(+-1) = 1/6) the 1 / w_i factor is
  // folded into the per-axis reciprocals as well.
  constexpr bool TW = tensor_weights<S>();
  if constexpr (TW) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      rinv[a][0] *= Real(6);
      rinv[a][1] *= Real(1.5);
      rinv[a][2] *= Real(6);
    }
  }
  Real rxy[3][3];
#pragma unroll
  for (int cx = 0; cx < 3; ++cx)
#pragma unroll
    for (int cy = 0; cy < 3; ++cy) rxy[cx][cy] = (irho * rinv[0][cx]) * rinv[1][cy];
  // f - f^eq (the only per-direction array kept; f^eq and the shear part
  // are recomputed where needed, which keeps the register footprint small)
  Real df[S::Q];
  static_for<0, S::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const Real q = qof(I);
    const Real w = Real(S::w(i));
    if constexpr (DEV)
      df[i] = fma(-w, fma(m0, q, m0 + q), v[i]);  // v - w (m0 (1 + q) + q)
    else
      df[i] = fma(-w * rho, q, v[i] - w * rho);  // v - w rho (1 + q)
  });
  // second-moment differences of f - feq, per pair of opposite directions
  // (e_a e_b is even in e: one sum df_i + df_i' per pair)
  Real M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  static_for<1, S::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int o = opp<S>(i);
    if constexpr (i < o) {
      constexpr int ex = S::e(i, 0), ey = S::e(i, 1), ez = S::e(i, 2);
      const Real sp = df[i] + df[o];
      if constexpr (ex != 0) M[0][0] += sp;
      if constexpr (ey != 0) M[1][1] += sp;
      if constexpr (ez != 0) M[2][2] += sp;
      if constexpr (ex * ey > 0) M[0][1] += sp;
      if constexpr (ex * ey < 0) M[0][1] -= sp;
      if constexpr (ex * ez > 0) M[0][2] += sp;
      if constexpr (ex * ez < 0) M[0][2] -= sp;
      if constexpr (ey * ez > 0) M[1][2] += sp;
      if constexpr (ey * ez < 0) M[1][2] -= sp;
    }
  });
  M[1][0] = M[0][1];
  M[2][0] = M[0][2];
  M[2][1] = M[1][2];
  // the shear part ds is zero for the directions with three non-zero
  // components (D3Q27's corners): there dh = df and ds drops out of the sums
  Real ss = Real(0), sh = Real(0);
  static_for<0, S::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr bool DS0 = S::D == 3 && S::e(i, 0) != 0 && S::e(i, 1) != 0 && S::e(i, 2) != 0;
    Real inv = rxy[S::e(i, 0) + 1][S::e(i, 1) + 1];
    if constexpr (S::D == 3) inv *= rinv[2][S::e(i, 2) + 1];
    if constexpr (!TW) inv *= Real(1.0 / S::w(i));
    if constexpr (DS0) {
      sh = fma(df[i], df[i] * inv, sh);
    } else {
      const Real ds = kbc_shear<S, i>(M);
      const Real dh = df[i] - ds;
      const Real t = dh * inv;
      ss = fma(ds, t, ss);
      sh = fma(dh, t, sh);
    }
  });
  const Real beta = Real(0.5) / tau;
  const Real ib = Real(1) / beta;
  Real gamma = ib - (Real(2) - ib) * (ss / sh);
  if (sh < Real(1e-16)) gamma = Real(2);
  // f - beta (2 ds + gamma dh)
  const Real b2 = Real(2) * beta, bg = beta * gamma;
  static_for<0, S::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr bool DS0 = S::D == 3 && S::e(i, 0) != 0 && S::e(i, 1) != 0 && S::e(i, 2) != 0;
    if constexpr (DS0) {
      v[i] = fma(-bg, df[i], v[i]);
    } else {
      const Real ds = kbc_shear<S, i>(M);
      const Real dh = df[i] - ds;
      v[i] = fma(-bg, dh, fma(-b2, ds, v[i]));
    }
  });
  return rho;
}

// Mass / momentum projection of the FP32 collision: removes the float
// rounding defect of the conserved moments (post - pre - target, target the
// mass and momentum a body force adds) through the rest and the axis populations, so
// that the collision conserves them exactly up to the (unbiased) rounding of
// small differences.
template <class S, class Real>
__device__ __forceinline__ void conserve(Real (&v)[S::Q], const Real (&pre)[S::Q],
                                         const Real (&target)[3] = {Real(0), Real(0), Real(0)},
                                         Real mass_target = Real(0)) {
  // per pair of opposite directions: the sum of the two changes enters the
  // mass defect, their difference the momentum components
  Real dm = (v[0] - pre[0]) - mass_target, dj[3] = {-target[0], -target[1], -target[2]};
  static_for<1, S::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int o = opp<S>(i);
    if constexpr (i < o) {
      const Real di = v[i] - pre[i], dn = v[o] - pre[o];
      dm += di + dn;
      const Real dd = di - dn;
      if constexpr (S::e(i, 0) > 0) dj[0] += dd;
      if constexpr (S::e(i, 0) < 0) dj[0] -= dd;
      if constexpr (S::e(i, 1) > 0) dj[1] += dd;
      if constexpr (S::e(i, 1) < 0) dj[1] -= dd;
      if constexpr (S::e(i, 2) > 0) dj[2] += dd;
      if constexpr (S::e(i, 2) < 0) dj[2] -= dd;
    }
  });
  // axis populations: +a and -a; changing them by -+dj/2 removes the
  // momentum defect and leaves the mass unchanged
  static_for<1, S::Q>([&](auto I) {
    constexpr int i = decltype(I)::value;
    constexpr int nz = (S::e(i, 0) != 0) + (S::e(i, 1) != 0) + (S::e(i, 2) != 0);
    if constexpr (nz == 1) {
      constexpr int a = S::e(i, 0) != 0 ? 0 : (S::e(i, 1) != 0 ? 1 : 2);
      constexpr int sg = S::e(i, 0) + S::e(i, 1) + S::e(i, 2);
      if constexpr (a < S::D) v[i] -= Real(0.5 * sg) * dj[a];
    }
  });
  v[0] -= dm;
}

// BGK of a StepParams kernel: plain, or with the body force of the handle.
// FORCE = false compiles the plain collision only (the force term costs
// registers that a latency-bound kernel needs for resident warps).
template <class S, bool DEV, bool COMP, bool FORCE = true, class Real, class Prm>
__device__ __forceinline__ Real bgk_collide(const Prm& P, Real (&v)[S::Q], const Real (&pre)[S::Q], Real (&u)[3],
                                            bool given_u) {
  Real rho;
  if (!FORCE || P.force_scheme == 0) {
    rho = collide_bgk<S, DEV, COMP>(v, Real(1) / Real(P.tau), u, given_u);
    if constexpr (DEV) {
      if (!given_u) conserve<S>(v, pre);
    }
  } else {
    const Real dF[3] = {Real(P.dF[0]), Real(P.dF[1]), Real(P.dF[2])};
    Real tgt[4];
    rho = collide_bgk_force<S, DEV, COMP>(v, Real(1) / Real(P.tau), Real(P.tau), u, given_u, dF, P.force_scheme,
                                          Real(P.scaling), tgt);
    if constexpr (DEV) {
      if (!given_u) {
        const Real tj[3] = {tgt[1], tgt[2], tgt[3]};
        conserve<S>(v, pre, tj, tgt[0]);
      }
    }
  }
  return rho;
}


}  // namespace natgpu
