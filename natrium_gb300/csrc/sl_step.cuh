// Fused semi-Lagrangian stream + collide kernel (one time step).
//
// Replaces, per time step, the reference's
//   stream():  f_tmp = f; fStream = A * f_tmp.fStream   (solver/CFDSolver.cpp:669-673,
//              advection/SemiLagrangian.h:150-161, Trilinos BlockSparseMatrix::vmult)
//   collide(): CollisionOperator::collideAll             (collision_advanced/CollisionOperator.h:26-111)
// with a single pass over HBM: f is read once and written once.
//
// Work decomposition: one CTA per tile of B_x * B_y * B_z lattice nodes (a
// whole number of cells per axis, so the node-class pattern is the same in
// every tile).  For each streamed direction alpha the CTA
//   1. loads the direction's source region (tile + the upwind window halo on
//      every axis where e_alpha has a component; periodic wrap through
//      per-axis index lists) from HBM/L2 into shared memory,
//   2. applies the 1-D Lagrange factors of the Kronecker-product operator
//      axis by axis (sum factorisation: z, then y in shared memory, x straight
//      into registers), so an output costs k (p+1) FMAs instead of (p+1)^k,
//   3. keeps the streamed value in registers.
// After the last direction every thread owns all Q streamed populations of
// its nodes and runs the collision epilogue in registers, then writes f once.
#pragma once

#include <cuda_runtime.h>

#include "collision.cuh"
#include "natgpu_common.h"
#include "stencils.cuh"

namespace natgpu {

constexpr int NT = 256;  // threads per CTA of the fused kernel


template <class Real>
struct SmemLayout {
  // offsets in bytes
  size_t w, wst, cls, j0, gidx, bufS, bufT1, bufT2, total;
};

template <class Real>
__host__ __device__ inline SmemLayout<Real> smem_layout(const int Rmax[3],
                                                        const int B[3]) {
  SmemLayout<Real> L;
  size_t o = 0;
  auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
  L.w = o;
  o = al(o + sizeof(Real) * 3 * ND_MAX * PER_MAX * PMAX1);
  L.wst = o;
  o = al(o + sizeof(int) * 3 * ND_MAX * BMAX);
  L.cls = o;
  o = al(o + sizeof(int) * 3 * BMAX);
  L.j0 = o;
  o = al(o + sizeof(int) * 3 * ND_MAX * PER_MAX);
  L.gidx = o;
  o = al(o + sizeof(int) * 3 * (ND_MAX + 1) * RMAX);
  L.bufS = o;
  o = al(o + sizeof(Real) * (size_t)Rmax[0] * Rmax[1] * Rmax[2]);
  L.bufT1 = o;
  o = al(o + sizeof(Real) * (size_t)Rmax[0] * Rmax[1] * B[2]);
  L.bufT2 = o;
  o = al(o + sizeof(Real) * (size_t)Rmax[0] * B[1] * B[2]);
  L.total = o;
  return L;
}

template <class Real>
__device__ __forceinline__ Real fma_r(Real a, Real b, Real c) {
  return fma(a, b, c);
}

// One window of a 1-D factor: sum_j w_j v_{j*stride}.  In the deviation
// mode it is evaluated as v_j0 + sum_{j != j0} w_j (v_j - v_j0) (j0: the
// dominant weight), which reproduces a constant field exactly whatever the
// float rounding of the weights.
template <bool DEV, class Real>
__device__ __forceinline__ Real window_sum(const Real* w, const Real* v, int stride, int p, int j0) {
  if constexpr (DEV) {
    const Real v0 = v[j0 * stride];
    Real acc = Real(0);
#pragma unroll
    for (int j = 0; j < PMAX1; ++j)
      if (j <= p && j != j0) acc = fma(w[j], v[j * stride] - v0, acc);
    return acc + v0;
  } else {
    Real acc = w[0] * v[0];
#pragma unroll
    for (int j = 1; j < PMAX1; ++j)
      if (j <= p) acc = fma(w[j], v[j * stride], acc);
    return acc;
  }
}

// Rest state subtracted in the deviation storage mode.
template <class S, int COLL>
__host__ __device__ constexpr double rest_state(int i) {
  if constexpr (COLL == COLL_BGK_INC) {
    return inc_rest(i);
  } else {
    return S::w(i);
  }
}

// Fused step kernel.  Real: arithmetic/storage type (double: plain FP64;
// float: deviation storage).  NPT: lattice nodes owned per thread.
// FORCE: the BGK form with the body-force term (bgk_collide)
template <class S, class Real, int COLL, int NPT, bool FORCE = false>
__global__ void __launch_bounds__(NT) k_sl_step(const StepParams P) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SLTables* __restrict__ T = P.tab;
  const int tid = threadIdx.x;

  const int Bx = T->ax[0].B, By = T->ax[1].B, Bz = T->ax[2].B;
  int Rmax[3] = {T->Rmax[0], T->Rmax[1], T->Rmax[2]};
  int Bv[3] = {Bx, By, Bz};
  const SmemLayout<Real> L = smem_layout<Real>(Rmax, Bv);
  Real* sW = reinterpret_cast<Real*>(smem_raw + L.w);
  int* sWst = reinterpret_cast<int*>(smem_raw + L.wst);
  int* sCls = reinterpret_cast<int*>(smem_raw + L.cls);
  int* sJ0 = reinterpret_cast<int*>(smem_raw + L.j0);
  int* sG = reinterpret_cast<int*>(smem_raw + L.gidx);
  Real* bS = reinterpret_cast<Real*>(smem_raw + L.bufS);
  Real* bT1 = reinterpret_cast<Real*>(smem_raw + L.bufT1);
  Real* bT2 = reinterpret_cast<Real*>(smem_raw + L.bufT2);

  // tile origin
  const int ntx = T->ax[0].ntiles, nty = T->ax[1].ntiles;
  const int bid = blockIdx.x;
  const int tx = bid % ntx, ty = (bid / ntx) % nty, tz = bid / (ntx * nty);
  const int g0[3] = {tx * Bx, ty * By, tz * Bz};
  const int p = T->p;

  // ---- tables -> shared memory --------------------------------------
  for (int i = tid; i < 3 * ND_MAX * PER_MAX * PMAX1; i += NT) {
    if constexpr (DEV)
      sW[i] = (&T->wf[0][0][0][0])[i];
    else
      sW[i] = (&T->w[0][0][0][0])[i];
  }
  for (int i = tid; i < 3 * ND_MAX * BMAX; i += NT) sWst[i] = (&T->wst[0][0][0])[i];
  for (int i = tid; i < 3 * ND_MAX * PER_MAX; i += NT) sJ0[i] = (&T->j0[0][0][0])[i];
  for (int i = tid; i < 3 * BMAX; i += NT) {
    const int a = i / BMAX, o = i % BMAX;
    sCls[i] = o % T->ax[a].period;
  }
  // periodic index lists: sG[a][0][k] = tile node k; sG[a][d+1][k] = source
  // region node k of displacement class d
  for (int i = tid; i < 3 * (ND_MAX + 1) * RMAX; i += NT) {
    const int a = i / ((ND_MAX + 1) * RMAX);
    const int r = i % ((ND_MAX + 1) * RMAX);
    const int d1 = r / RMAX, k = r % RMAX;
    const int n = T->ax[a].n;
    int g;
    if (d1 == 0) {
      g = g0[a] + k;
    } else {
      const int d = d1 - 1;
      g = g0[a] + (d < T->ax[a].nd ? T->ax[a].lo[d] : 0) + k;
    }
    g %= n;
    if (g < 0) g += n;
    sG[i] = g;
  }

  // ---- owned nodes ----------------------------------------------------
  const int TB = Bx * By * Bz;
  const long long n = P.n;
  const int nx = P.nx, nxy = P.nx * P.ny;
  int lx[NPT], ly[NPT], lz[NPT];
  long long node[NPT];
  bool own[NPT];
#pragma unroll
  for (int k = 0; k < NPT; ++k) {
    const int t = tid + k * NT;
    own[k] = t < TB;
    const int tt = own[k] ? t : 0;
    lx[k] = tt % Bx;
    ly[k] = (tt / Bx) % By;
    lz[k] = tt / (Bx * By);
    node[k] = (long long)(g0[2] + lz[k]) * nxy + (long long)(g0[1] + ly[k]) * nx +
              (g0[0] + lx[k]);
  }

  const Real* __restrict__ fin = static_cast<const Real*>(P.f_in);
  Real* __restrict__ fout = static_cast<Real*>(P.f_out);
  Real fs[NPT][Q];

  // rest population: not streamed
#pragma unroll
  for (int k = 0; k < NPT; ++k) fs[k][0] = own[k] ? fin[node[k]] : Real(0);

  const int* sGx = sG + 0 * (ND_MAX + 1) * RMAX;
  const int* sGy = sG + 1 * (ND_MAX + 1) * RMAX;
  const int* sGz = sG + 2 * (ND_MAX + 1) * RMAX;

  static_for<1, Q>([&](auto I) {
    constexpr int A = decltype(I)::value;
    constexpr int dx = S::dcls(A, 0);
    constexpr int dy = S::dcls(A, 1);
    constexpr int dz = (S::D == 3) ? S::dcls(A, 2) : -1;
    const int Rx = dx < 0 ? Bx : T->ax[0].R[dx < 0 ? 0 : dx];
    const int Ry = dy < 0 ? By : T->ax[1].R[dy < 0 ? 0 : dy];
    const int Rz = dz < 0 ? Bz : T->ax[2].R[dz < 0 ? 0 : dz];
    const int* gx = sGx + (dx + 1) * RMAX;
    const int* gy = sGy + (dy + 1) * RMAX;
    const int* gz = sGz + (dz + 1) * RMAX;
    const Real* __restrict__ src = fin + (long long)A * n;

    __syncthreads();  // previous direction done with the buffers (and tables ready)
    {
      const int tot = Rx * Ry * Rz;
      for (int i = tid; i < tot; i += NT) {
        const int x = i % Rx;
        const int t = i / Rx;
        const int y = t % Ry;
        const int z = t / Ry;
        bS[i] = __ldg(src + (long long)gz[z] * nxy + (long long)gy[y] * nx + gx[x]);
      }
    }
    __syncthreads();
    const Real* cur = bS;
    if constexpr (dz >= 0) {
      // z factor: (Rx, Ry, Rz) -> (Rx, Ry, Bz)
      const Real* wz = sW + ((2 * ND_MAX + dz) * PER_MAX) * PMAX1;
      const int* wstz = sWst + (2 * ND_MAX + dz) * BMAX;
      const int* clsz = sCls + 2 * BMAX;
      const int plane = Rx * Ry;
      const int tot = plane * Bz;
      for (int i = tid; i < tot; i += NT) {
        const int z = i / plane;
        const int xy = i - z * plane;
        const Real* s0 = cur + wstz[z] * plane + xy;
        const Real* wr = wz + clsz[z] * PMAX1;
        bT1[i] = window_sum<DEV>(wr, s0, plane, p, sJ0[(2 * ND_MAX + dz) * PER_MAX + clsz[z]]);
      }
      __syncthreads();
      cur = bT1;
    }
    if constexpr (dy >= 0) {
      // y factor: (Rx, Ry, Bz) -> (Rx, By, Bz)
      const Real* wy = sW + ((1 * ND_MAX + dy) * PER_MAX) * PMAX1;
      const int* wsty = sWst + (1 * ND_MAX + dy) * BMAX;
      const int* clsy = sCls + 1 * BMAX;
      const int tot = Rx * By * Bz;
      for (int i = tid; i < tot; i += NT) {
        const int x = i % Rx;
        const int t = i / Rx;
        const int y = t % By;
        const int z = t / By;
        const Real* s0 = cur + (z * Ry + wsty[y]) * Rx + x;
        const Real* wr = wy + clsy[y] * PMAX1;
        bT2[i] = window_sum<DEV>(wr, s0, Rx, p, sJ0[(1 * ND_MAX + dy) * PER_MAX + clsy[y]]);
      }
      __syncthreads();
      cur = bT2;
    }
    // x factor straight into registers: cur is (Rx, By, Bz)
    {
      const Real* wxx = sW + ((0 * ND_MAX + (dx < 0 ? 0 : dx)) * PER_MAX) * PMAX1;
      const int* wstx = sWst + (0 * ND_MAX + (dx < 0 ? 0 : dx)) * BMAX;
      const int* clsx = sCls;
#pragma unroll
      for (int k = 0; k < NPT; ++k) {
        const Real* row = cur + (lz[k] * By + ly[k]) * Rx;
        Real acc;
        if constexpr (dx >= 0) {
          const Real* s0 = row + wstx[lx[k]];
          const Real* wr = wxx + clsx[lx[k]] * PMAX1;
          acc = window_sum<DEV>(wr, s0, 1, p, sJ0[(0 * ND_MAX + dx) * PER_MAX + clsx[lx[k]]]);
        } else {
          acc = row[lx[k]];
        }
        fs[k][A] = own[k] ? acc : Real(0);
      }
    }
  });

  // ---- collision epilogue + single write --------------------------------
  int bad = 0;
#pragma unroll
  for (int k = 0; k < NPT; ++k) {
    if (!own[k]) continue;
    Real u[3] = {0, 0, 0};
    Real rho = Real(1);
    Real pre[Q];
    if constexpr (DEV) {
#pragma unroll
      for (int q = 0; q < Q; ++q) pre[q] = fs[k][q];
    }
    if constexpr (COLL == COLL_BGK) {
      rho = bgk_collide<S, DEV, DEV, FORCE>(P, fs[k], pre, u, false);
    } else if constexpr (COLL == COLL_BGK_INC) {
      rho = collide_bgk_inc<DEV, DEV>(fs[k], Real(1) / Real(P.tau), u, false);
    } else if constexpr (COLL == COLL_KBC) {
      rho = collide_kbc<S, DEV, DEV>(fs[k], Real(P.tau), u, false);
      if constexpr (DEV) conserve<S>(fs[k], pre);
    }
    (void)pre;
    if constexpr (COLL != COLL_NONE) {
      if (!(rho >= Real(1e-10))) bad |= (rho != rho) ? ST_NAN : ST_DENSITY;
      if (P.write_macro) {
        P.rho[node[k]] = (double)rho;
        P.u[node[k]] = (double)u[0] * P.scaling;
        P.u[n + node[k]] = (double)u[1] * P.scaling;
        if constexpr (S::D == 3) P.u[2 * n + node[k]] = (double)u[2] * P.scaling;
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) fout[(long long)q * n + node[k]] = fs[k][q];
  }
  if constexpr (COLL != COLL_NONE) {
    const unsigned any = __ballot_sync(0xffffffffu, bad != 0);
    if (any && bad) atomicOr(P.status, bad);
  }
}

// Rows of the streaming operator of the wall nodes (nodes with a departure
// path that meets a wall face), built on the host: Q - 1 rows per node,
// row k (Q - 1) + alpha - 1 holding sum_j w_j f_in[col_j] + cst[4 row + slot].
template <class Real>
struct WallNodes {
  int nbn;           // wall nodes
  const int* node;   // their lattice indices
};

// Collision of the wall nodes.  Their sparse rows have just been streamed
// into f_out by k_wall_rows (one thread per row); this takes the streamed
// values from there and the rest population from f_in, collides, and writes
// f (and rho/u on output steps).  Runs after the fused kernel of the whole
// lattice and overwrites the wall nodes, whose periodic-window values there
// are not the wall's.  (One thread walking all Q-1 rows of its node was
// latency-bound: a few thousand wall nodes are too few warps to hide ~300
// dependent loads each.)
template <class S, class Real, int COLL, bool FORCE = false>
__global__ void __launch_bounds__(128) k_wall_nodes(const StepParams P, const WallNodes<Real> W) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q;
  const long long n = P.n;
  const Real* __restrict__ fin = static_cast<const Real*>(P.f_in);
  Real* __restrict__ fout = static_cast<Real*>(P.f_out);
  int bad = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < W.nbn; k += gridDim.x * blockDim.x) {
    const int node = W.node[k];
    Real v[Q];
    v[0] = fin[node];
#pragma unroll
    for (int a = 1; a < Q; ++a) v[a] = fout[(long long)a * n + node];
    Real u[3] = {0, 0, 0};
    Real rho = Real(1);
    Real pre[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) pre[q] = v[q];
    if constexpr (COLL == COLL_BGK) {
      rho = bgk_collide<S, DEV, DEV, FORCE>(P, v, pre, u, false);
    } else if constexpr (COLL == COLL_BGK_INC) {
      rho = collide_bgk_inc<DEV, DEV>(v, Real(1) / Real(P.tau), u, false);
    } else if constexpr (COLL == COLL_KBC) {
      rho = collide_kbc<S, DEV, DEV>(v, Real(P.tau), u, false);
      if constexpr (DEV) conserve<S>(v, pre);
    }
    (void)pre;
    if (!(rho >= Real(1e-10))) bad |= (rho != rho) ? ST_NAN : ST_DENSITY;
    if (P.write_macro) {
      P.rho[node] = (double)rho;
      P.u[node] = (double)u[0] * P.scaling;
      P.u[n + node] = (double)u[1] * P.scaling;
      if constexpr (S::D == 3) P.u[2 * n + node] = (double)u[2] * P.scaling;
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) fout[(long long)q * n + node] = v[q];
  }
  if (bad) atomicOr(P.status, bad);
}

// Collision only (CollisionModel::collideAll on the device state), in place.
template <class S, class Real, int COLL, bool FORCE = false>
__global__ void __launch_bounds__(256) k_collide(const StepParams P) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q;
  const long long n = P.n;
  Real* f = static_cast<Real*>(P.f_out);
  int bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    Real v[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = f[q * n + i];
    Real u[3] = {0, 0, 0};
    const bool given = P.in_init != 0;
    if (given) {
      u[0] = Real(P.u[i] / P.scaling);
      u[1] = Real(P.u[n + i] / P.scaling);
      if constexpr (S::D == 3) u[2] = Real(P.u[2 * n + i] / P.scaling);
    }
    Real rho;
    Real pre[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) pre[q] = v[q];
    if constexpr (COLL == COLL_BGK_INC) {
      rho = collide_bgk_inc<DEV, DEV>(v, Real(1) / Real(P.tau), u, given);
    } else if constexpr (COLL == COLL_KBC) {
      rho = collide_kbc<S, DEV, DEV>(v, Real(P.tau), u, given);
      if constexpr (DEV) {
        if (!given) conserve<S>(v, pre);
      }
    } else {
      // with a prescribed velocity the momentum is not a collision invariant
      rho = bgk_collide<S, DEV, DEV, FORCE>(P, v, pre, u, given);
    }
    if (!(rho >= Real(1e-10))) bad |= (rho != rho) ? ST_NAN : ST_DENSITY;
    P.rho[i] = (double)rho;
    if (!given) {
      P.u[i] = (double)u[0] * P.scaling;
      P.u[n + i] = (double)u[1] * P.scaling;
      if constexpr (S::D == 3) P.u[2 * n + i] = (double)u[2] * P.scaling;
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q * n + i] = v[q];
  }
  if (bad) atomicOr(P.status, bad);
}

}  // namespace natgpu
