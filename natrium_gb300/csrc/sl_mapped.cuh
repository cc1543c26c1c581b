// Fused semi-Lagrangian stream + collide on MappingQ1 (deformed) cells:
// the departure-point kernel.
//
// The reference assembles the streaming operator of a mapped mesh into a
// sparse matrix (SemiLagrangian.cpp:403-522): per (node, direction) a row of
// (p+1)^D shape values of the cell that holds the departure point.  Those
// values are products of 1-D Lagrange polynomials at the departure point's
// UNIT coordinates, so a row is fully described by
//   base   source index of the cell's first node (source direction * n + node),
//   u[D]   unit coordinates of the departure point in that cell (FP32; the
//          FP64 form stores the D (P+1) 1-D Lagrange values instead),
//   cst    additive constant (bounce-back wall terms, deviation-form offset),
//   flags  bits 0-2: the local node p of this cell along x / y / z is node 0
//          of the axis (FE_Q, last cell of a periodic axis); bit 3: the row
//          had entries 0 < |v| < 1e-10, which the reference drops
//          (SemiLagrangian.cpp:483), so the row takes the per-entry path.
// The kernel evaluates the 1-D Lagrange values on the fly and gathers the
// (p+1)^D source values in factorised order -- ~20-40 bytes of row data per
// (node, direction) instead of the matrix's (p+1)^D x (index + value).
//
// One thread per node: the Q-1 rows are gathered into shared memory (per
// thread slot), then the node collides in registers and writes f (and rho, u
// on output steps).  Row arrays are direction-major, node-minor, so
// consecutive threads read consecutive row entries.
#pragma once

#include <cuda_runtime.h>

#include "collision.cuh"
#include "natgpu_common.h"
#include "stencils.cuh"

namespace natgpu {

constexpr int MAP_THREADS = 128;
constexpr unsigned MAP_TINY = 8u;

template <class Real>
struct MappedRows {
  const int* base;             // (Q-1) n
  const Real* u;               // FP32: unit coordinates, (Q-1) D n: [(a-1) D + d] n + node;
                               // FP64: 1-D Lagrange values, [((a-1) D + d) (P+1) + j] n + node
  const Real* cst;             // (Q-1) n
  const unsigned char* flags;  // (Q-1) n
  int nax[3];                  // lattice nodes per axis
};

// Gauss-Lobatto points of one order and R_j = prod_{m != j} 1 / (xi_j - xi_m).
template <class Real>
struct LagrangeTab {
  Real xi[PMAX1];
  Real R[PMAX1];
};

// l_j(u) = R_j prod_{m != j} (u - xi_m), j = 0..P, from prefix and suffix
// products of d_m = u - xi_m (4P + 2 multiplications; exact zeros at the
// other nodes).
template <int P, class Real>
__device__ __forceinline__ void lagrange_values(Real u, const LagrangeTab<Real>& L, Real* l) {
  Real d[P + 1], left[P + 1];
#pragma unroll
  for (int m = 0; m <= P; ++m) d[m] = u - L.xi[m];
  left[0] = Real(1);
#pragma unroll
  for (int j = 1; j <= P; ++j) left[j] = left[j - 1] * d[j - 1];
  Real right = Real(1);
#pragma unroll
  for (int j = P; j >= 0; --j) {
    l[j] = left[j] * right * L.R[j];
    right *= d[j];
  }
}

// (One direction per loop iteration: unrolling two, which overlaps their row
// loads and gathers, measured 25 % slower in 2-D and 7 % in 3-D.)
template <class S, class Real, int COLL, int P, bool FORCE = false>
__global__ void __launch_bounds__(MAP_THREADS) k_mapped(const StepParams prm, const MappedRows<Real> R,
                                                      const LagrangeTab<Real> L) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q, D = S::D, NP = P + 1;
  constexpr int NZ = D == 3 ? NP : 1;
  __shared__ Real vs[Q - 1][MAP_THREADS];
  const int n = (int)prm.n;
  const int nx = R.nax[0], nxy = R.nax[0] * R.nax[1];
  const Real* __restrict__ fin = static_cast<const Real*>(prm.f_in);
  Real* __restrict__ fout = static_cast<Real*>(prm.f_out);
  int bad = 0;
  for (int node0 = blockIdx.x * MAP_THREADS; node0 < n; node0 += gridDim.x * MAP_THREADS) {
    const int node = node0 + threadIdx.x;
    const bool live = node < n;
    if (!live) continue;
#pragma unroll 1
    for (int a = 1; a < Q; ++a) {
      const long long r = (long long)(a - 1) * n + node;
      const int base = __ldg(R.base + r);
      const unsigned fl = __ldg(R.flags + r);
      Real lx[NP], ly[NP], lz[NP];
      if constexpr (sizeof(Real) == 8) {
        // FP64: the 1-D Lagrange values are stored (the FP64 pipe is the
        // bound; evaluating them here cost as much as the gather itself)
        const Real* lr = R.u + (long long)(a - 1) * D * NP * n + node;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          lx[j] = __ldg(lr + (long long)j * n);
          ly[j] = __ldg(lr + (long long)(NP + j) * n);
          if constexpr (D == 3) lz[j] = __ldg(lr + (long long)(2 * NP + j) * n);
        }
        if constexpr (D == 2) lz[0] = Real(1);
      } else {
        const Real* ur = R.u + (long long)(a - 1) * D * n + node;
        lagrange_values<P>(__ldg(ur), L, lx);
        lagrange_values<P>(__ldg(ur + n), L, ly);
        if constexpr (D == 3) lagrange_values<P>(__ldg(ur + 2 * n), L, lz);
        else lz[0] = Real(1);
      }
      // offsets of the local nodes; node p wraps to node 0 of the axis on the
      // last FE_Q cell of a periodic axis
      int ox[NP], oy[NP], oz[NZ];
#pragma unroll
      for (int j = 0; j < NP; ++j) {
        ox[j] = j;
        oy[j] = j * nx;
      }
#pragma unroll
      for (int j = 0; j < NZ; ++j) oz[j] = j * nxy;
      if (fl & 1u) ox[P] = P - R.nax[0];
      if (fl & 2u) oy[P] = (P - R.nax[1]) * nx;
      if constexpr (D == 3) {
        if (fl & 4u) oz[P] = (P - R.nax[2]) * nxy;
      }
      Real acc = Real(0);
      if (!(fl & MAP_TINY)) {
#pragma unroll
        for (int k = 0; k < NZ; ++k) {
          Real sy = Real(0);
#pragma unroll
          for (int j = 0; j < NP; ++j) {
            Real sx = Real(0);
#pragma unroll
            for (int i = 0; i < NP; ++i) sx = fma(lx[i], __ldg(fin + base + ox[i] + oy[j] + oz[k]), sx);
            sy = fma(ly[j], sx, sy);
          }
          acc = fma(lz[k], sy, acc);
        }
      } else {
        // the reference's entry rule: shape values below 1e-10 are dropped
#pragma unroll
        for (int k = 0; k < NZ; ++k)
#pragma unroll
          for (int j = 0; j < NP; ++j)
#pragma unroll
            for (int i = 0; i < NP; ++i) {
              const Real w = lx[i] * ly[j] * lz[k];
              if (fabs(w) >= Real(1e-10)) acc = fma(w, __ldg(fin + base + ox[i] + oy[j] + oz[k]), acc);
            }
      }
      vs[a - 1][threadIdx.x] = acc + __ldg(R.cst + r);
    }
    Real v[Q];
    v[0] = fin[node];
#pragma unroll
    for (int a = 1; a < Q; ++a) v[a] = vs[a - 1][threadIdx.x];
    Real u[3] = {0, 0, 0};
    Real rho = Real(1);
    Real pre[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) pre[q] = v[q];
    if constexpr (COLL == COLL_BGK) {
      rho = bgk_collide<S, DEV, DEV, FORCE>(prm, v, pre, u, false);
    } else if constexpr (COLL == COLL_BGK_INC) {
      rho = collide_bgk_inc<DEV, DEV>(v, Real(1) / Real(prm.tau), u, false);
    } else if constexpr (COLL == COLL_KBC) {
      rho = collide_kbc<S, DEV, DEV>(v, Real(prm.tau), u, false);
      if constexpr (DEV) conserve<S>(v, pre);
    }
    (void)pre;
    if constexpr (COLL != COLL_NONE) {
      if (!(rho >= Real(1e-10))) bad |= (rho != rho) ? ST_NAN : ST_DENSITY;
      if (prm.write_macro) {
        prm.rho[node] = (double)rho;
        prm.u[node] = (double)u[0] * prm.scaling;
        prm.u[n + node] = (double)u[1] * prm.scaling;
        if constexpr (D == 3) prm.u[2 * (long long)n + node] = (double)u[2] * prm.scaling;
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) fout[(long long)q * n + node] = v[q];
  }
  if (bad) atomicOr(prm.status, bad);
}

// the instantiation of one order (1..PMAX), NULL outside that range;
// FORCE: the BGK form with the body-force term
template <class S, class Real, int COLL, bool FORCE = false>
const void* mapped_for_order(int p) {
  switch (p) {
    case 1: return (const void*)&k_mapped<S, Real, COLL, 1, FORCE>;
    case 2: return (const void*)&k_mapped<S, Real, COLL, 2, FORCE>;
    case 3: return (const void*)&k_mapped<S, Real, COLL, 3, FORCE>;
    case 4: return (const void*)&k_mapped<S, Real, COLL, 4, FORCE>;
    case 5: return (const void*)&k_mapped<S, Real, COLL, 5, FORCE>;
    case 6: return (const void*)&k_mapped<S, Real, COLL, 6, FORCE>;
  }
  return nullptr;
}

}  // namespace natgpu
