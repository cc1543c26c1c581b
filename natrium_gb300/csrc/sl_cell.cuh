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

// Shared memory per warp: Q * 32 * PER values (PER = p + 1 nodes per cell
// row in DG, p in FE_Q).
template <class S, class Real, int P, bool DG = true>
__host__ __device__ constexpr size_t cell_smem_per_warp() {
  return (size_t)S::Q * 32 * (DG ? P + 1 : P) * sizeof(Real);
}

// ---- tensor-core form of the corner directions (D3Q27, p = 3, FP32) --------
// For a corner direction (sx, sy, sz) the streamed values of one cell's 16
// nodes (cx, cy) at a fixed z class cz are a dense contraction over the
// 2 x 2 source cells in x and y (own and upwind) and the 4 rows of the z
// window: out[(cx, cy)] = sum_jz wz[jz] sum_k A[(cx, cy)][k] F_jz[k], k =
// (cx', ux, cy', uy), A = Wx (x) Wy with Wx[cx][(cx', ux)] = w_x[cx][cx'] when
// ux is the cell of cx's window (the upwind one for the class that leaves the
// cell) and 0 otherwise -- the per-cell (p+1)^2 x 4 (p+1)^2 block of the
// reference's assembled operator (SemiLagrangian.cpp:227-229, 483) restricted
// to one z row.  The CTA's 4 warps hold the 4 y rows (cy) of one y cell; warp
// w takes cells 8w .. 8w + 7 as the N = 8 columns of an m16n8k8 tile, M = the
// 16 (cx, cy) nodes, K = 8 (cx', ux) per step, 8 steps (cy', uy) per z row.
// Operands are split into two TF32 halves (a = a_hi + a_lo, both rounded to
// nearest) and the product taken as a_hi b_hi + a_hi b_lo + a_lo b_hi with
// FP32 accumulation; the z factor is applied to the four per-row partial sums
// at the end.  A's fragments are precomputed per CTA: [dx][dy][step][lane][8].
constexpr int CORNER_A_FLOATS = 4 * 8 * 32 * 8;

__device__ __forceinline__ unsigned tf32_rna(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// A fragments of the four (sx, sy) sign pairs; threads t0, t0 + stride, ...
template <int P>
__device__ __forceinline__ void fill_corner_table(float* sA, const float (&W)[3][2][PER_MAX][PMAX1], int t0,
                                                  int stride) {
  for (int i = t0; i < CORNER_A_FLOATS / 2; i += stride) {
    const int e = i & 3, lane = (i >> 2) & 31, st = (i >> 7) & 7, dxy = i >> 10;
    const int dx = dxy & 1, dy = dxy >> 1;
    const int g = lane >> 2, t = lane & 3;
    const int r = g + ((e & 1) ? 8 : 0);      // a0: (g, t), a1: (g+8, t), a2: (g, t+4), a3: (g+8, t+4)
    const int k = t + ((e & 2) ? 4 : 0);
    const int cx = r & 3, cy = r >> 2;
    const int cxs = k & 3, ux = k >> 2;       // source node and cell (0 own, 1 upwind) along x
    const int cys = st & 3, uy = st >> 2;     // along y
    const int ox = dx == 0 ? (cx == 0) : (cx == P);
    const int oy = dy == 0 ? (cy == 0) : (cy == P);
    const float a = (ux == ox && uy == oy) ? W[0][dx][cx][cxs] * W[1][dy][cy][cys] : 0.f;
    const unsigned hi = tf32_rna(a);
    const unsigned lo = tf32_rna(a - __uint_as_float(hi));
    float* q = sA + ((size_t)((dxy * 8 + st) * 32 + lane) * 8);
    q[e] = __uint_as_float(hi);
    q[4 + e] = __uint_as_float(lo);
  }
}

// ---- z sharing of the directions with y and z components -------------------
// A direction (sx, sy, sz) with sy, sz != 0 (yz-diagonal, or corner) needs,
// for each of the CTA's R rows, the y window of z-window sums (and then, for
// a corner, the x factor).  The z window is the same for the whole CTA (one
// z), so the z sums of the union of the R rows' y windows are computed once
// per CTA (U rows, each shared by up to P + 1 output rows) and every row then
// takes its y sum from them: about U / R + 1 window sums per node instead of
// P + 2.  The U x nx z sums live in the shared slots of the directions
// streamed last (the yz-diagonals go first), two buffers alternating between
// consecutive yz-diagonals, so one CTA barrier per direction suffices.

// directions with a y and a z component (the yz-diagonals, and the corners
// of D3Q27, whose x factor follows the shared y/z part)
template <class S>
__host__ __device__ constexpr bool is_yz(int a) {
  return S::D == 3 && S::e(a, 1) != 0 && S::e(a, 2) != 0;
}
template <class S>
__host__ __device__ constexpr int n_yz() {
  int k = 0;
  for (int a = 1; a < S::Q; ++a) k += is_yz<S>(a);
  return k;
}
// k-th streamed direction (k = 0 .. Q - 2): with ZS the y/z ones first
template <class S, bool ZS>
__host__ __device__ constexpr int cell_order(int k) {
  if (!ZS) return k + 1;
  int n = 0;
  for (int a = 1; a < S::Q; ++a)
    if (is_yz<S>(a) && n++ == k) return a;
  for (int a = 1; a < S::Q; ++a)
    if (!is_yz<S>(a) && n++ == k) return a;
  return -1;
}
// window start of row y along an axis with displacement sign SG (the node
// period PER = p + 1 in DG, p in FE_Q; the window spans p + 1 rows)
template <int P, bool DG, int SG>
__host__ __device__ constexpr int ws_row(int y) {
  constexpr int PER = DG ? P + 1 : P;
  return SG > 0 ? y - y % PER - (y % PER == 0 ? PER : 0)
                : y - y % PER + (DG && y % PER == P ? PER : 0);
}
// most union rows of R consecutive rows starting at a multiple of R
template <int P, bool DG, int R>
__host__ __device__ constexpr int zs_union_max() {
  constexpr int PER = DG ? P + 1 : P;
  int m = 0;
  for (int r = 0; r < PER * R; r += R) {
    const int y0 = r + 2 * PER * R;  // positive, same residue
    const int a = ws_row<P, DG, 1>(y0 + R - 1) - ws_row<P, DG, 1>(y0) + P + 1;
    const int b = ws_row<P, DG, -1>(y0 + R - 1) - ws_row<P, DG, -1>(y0) + P + 1;
    m = a > m ? a : m;
    m = b > m ? b : m;
  }
  return m;
}
// directions whose slots hold the two z-sum buffers: the last 2 SPB of the
// order, SPB = slots per buffer
template <class S, int P, int L, int WARPS, bool DG>
__host__ __device__ constexpr int zs_slots_per_buffer() {
  constexpr int RPW = L >= 32 ? 1 : 32 / L;
  constexpr int chunks = (zs_union_max<P, DG, WARPS * RPW>() + RPW - 1) / RPW;
  return (chunks + WARPS - 1) / WARPS;
}
template <class S, int P, int L, int WARPS, bool DG>
__device__ __forceinline__ int zs_slot(int buf, int s) {
  constexpr int SPB = zs_slots_per_buffer<S, P, L, WARPS, DG>();
  return cell_order<S, true>(S::Q - 2 - (buf * SPB + s));
}

// x factor of the lane's PER nodes from their y/z-factored values T and the
// neighbouring cells' values U (previous cell, the one upwind for sx > 0) and
// V (next cell).  DG: the classes whose departure point stays in the node's
// own cell take T; the one class that leaves it (0 for sx > 0, P for
// sx < 0) takes U or V, dominant its nearest node.  FE_Q (a lane owns nodes
// 0 .. P - 1 of its cell, node P being V[0]): for sx > 0 class 0 takes
// [U_0 .. U_{P-1}, T_0], the others [T_0 .. T_{P-1}, V_0]; for sx < 0 every
// class takes the latter.  The weights come straight from the kernel's
// constant bank (compile-time class and window).
template <bool DEV, int P, bool DG, int sx, class Real, int PER>
__device__ __forceinline__ void x_apply(const Real (&Wx)[PER_MAX][PMAX1], const Real (&T)[PER],
                                        const Real (&U)[PER], const Real (&V)[PER], Real (&out)[PER]) {
  static_for<0, PER>([&](auto C) {
    constexpr int c = decltype(C)::value;
    Real w[P + 1], v[P + 1];
#pragma unroll
    for (int j = 0; j <= P; ++j) w[j] = Wx[c][j];
    if constexpr (DG) {
      if constexpr (sx > 0 && c == 0) {
        out[c] = wsum_fixed<DEV, P, P>(w, U);
      } else if constexpr (sx < 0 && c == P) {
        out[c] = wsum_fixed<DEV, P, 0>(w, V);
      } else {
        out[c] = wsum_fixed<DEV, P, c>(w, T);
      }
    } else if constexpr (sx > 0 && c == 0) {
#pragma unroll
      for (int j = 0; j < P; ++j) v[j] = U[j];
      v[P] = T[0];
      out[c] = wsum_fixed<DEV, P, P>(w, v);  // dominant: the node itself, window slot P
    } else {
#pragma unroll
      for (int j = 0; j < P; ++j) v[j] = T[j];
      v[P] = V[0];
      out[c] = wsum_fixed<DEV, P, c>(w, v);
    }
  });
}

// which neighbouring values a direction's x factor needs
template <bool DG, int sx>
__host__ __device__ constexpr bool x_needs_prev() {
  return sx > 0;
}
template <bool DG, int sx>
__host__ __device__ constexpr bool x_needs_next() {
  return DG ? sx < 0 : sx != 0;
}

// x factor when the warp holds whole periodic rows of L <= 32 cells (lane
// r L + X holds cell X of the warp's row r): the neighbours by shuffles
template <bool DEV, int P, int L, bool DG, int sx, class Real, int PER>
__device__ __forceinline__ void x_factor(const Real (&Wx)[PER_MAX][PMAX1], const Real (&T)[PER], Real (&out)[PER],
                                         int X, int r) {
  Real U[PER], V[PER];
#pragma unroll
  for (int c = 0; c < PER; ++c) {
    U[c] = T[c];
    V[c] = T[c];
  }
  if constexpr (x_needs_prev<DG, sx>()) {
#pragma unroll
    for (int c = 0; c < PER; ++c) U[c] = __shfl_sync(0xffffffffu, T[c], r * L + (X + L - 1) % L);
  }
  if constexpr (x_needs_next<DG, sx>()) {
#pragma unroll
    for (int c = 0; c < (DG ? PER : 1); ++c) V[c] = __shfl_sync(0xffffffffu, T[c], r * L + (X + 1) % L);
  }
  x_apply<DEV, P, DG, sx>(Wx, T, U, V, out);
}

// x factor when GW warps share a periodic row of 32 GW cells (warp g of the
// row holds cells 32 g .. 32 g + 31): the neighbours by shuffles inside the
// warp, and across the warps through shared memory: every warp leaves its
// lanes 0 and 31's values in edge[warp][0 / 1], the row's warps meet at a
// named barrier (id 1 + row, 32 GW threads; at most four rows per CTA), and
// lane 0 / 31 take the
// previous / next warp's.  edge alternates between two buffers from one
// direction to the next, so one barrier per direction suffices.
template <bool DEV, int P, int GW, bool DG, int sx, class Real, int PER>
__device__ __forceinline__ void x_factor_mw(const Real (&Wx)[PER_MAX][PMAX1], const Real (&T)[PER],
                                            Real (&out)[PER], int lane, int warp, Real (*edge)[2][PER]) {
  const int g = warp % GW, row = warp / GW;
  const int wprev = warp - g + (g + GW - 1) % GW, wnext = warp - g + (g + 1) % GW;
  if (lane == 0 || lane == 31) {
#pragma unroll
    for (int c = 0; c < PER; ++c) edge[warp][lane == 0 ? 0 : 1][c] = T[c];
  }
  // a compile-time barrier id per row (a run-time id reserves all sixteen)
  switch (row) {
    case 0: asm volatile("bar.sync 1, %0;" ::"n"(32 * GW) : "memory"); break;
    case 1: asm volatile("bar.sync 2, %0;" ::"n"(32 * GW) : "memory"); break;
    case 2: asm volatile("bar.sync 3, %0;" ::"n"(32 * GW) : "memory"); break;
    default: asm volatile("bar.sync 4, %0;" ::"n"(32 * GW) : "memory"); break;
  }
  Real U[PER], V[PER];
#pragma unroll
  for (int c = 0; c < PER; ++c) {
    U[c] = T[c];
    V[c] = T[c];
  }
  if constexpr (x_needs_prev<DG, sx>()) {
#pragma unroll
    for (int c = 0; c < PER; ++c) {
      const Real sh = __shfl_sync(0xffffffffu, T[c], (lane + 31) & 31);
      U[c] = lane == 0 ? edge[wprev][1][c] : sh;
    }
  }
  if constexpr (x_needs_next<DG, sx>()) {
#pragma unroll
    for (int c = 0; c < (DG ? PER : 1); ++c) {
      const Real sh = __shfl_sync(0xffffffffu, T[c], (lane + 1) & 31);
      V[c] = lane == 31 ? edge[wnext][0][c] : sh;
    }
  }
  x_apply<DEV, P, DG, sx>(Wx, T, U, V, out);
}

// One corner direction A in the tensor-core form for the CTA's y cell `by`
// (rows 4 by .. 4 by + 3, warp cy owns row 4 by + cy) at row z (class cz):
// warp w computes cells 8w .. 8w + 7 for all 16 (cx, cy) nodes and stores
// them into the owning warps' arrays S (layout [warp][q][32 PER]).
template <class S, int P, int A>
__device__ __forceinline__ void corner_mma(const RowParams<float>& prm, const float* sA, float* S_all, int by, int z,
                                           int cz, int lane, int warp) {
  constexpr int Q = S::Q, PER = P + 1, NPW = 32 * PER;
  constexpr int sx = S::e(A, 0), sy = S::e(A, 1), sz = S::e(A, 2);
  constexpr int dx = sx > 0 ? 0 : 1, dy = sy > 0 ? 0 : 1, dz = sz > 0 ? 0 : 1;
  const int nx = prm.nx, ny = prm.ny, nz = prm.nz, nxy = nx * ny;
  const int g = lane >> 2, t = lane & 3;
  const int X = 8 * warp + g;                    // this thread's B column: cell X
  const int Xu = (X - sx + 32) & 31;             // its upwind cell along x (row of 32 cells)
  const int bo0 = 4 * X + t, bo1 = 4 * Xu + t;
  // z window: the upwind z cell for the class that leaves the cell
  const bool oz = dz == 0 ? (cz == 0) : (cz == P);
  const int zc = (z / PER) - (oz ? sz : 0);
  int zoff[PER];
#pragma unroll
  for (int j = 0; j < PER; ++j) zoff[j] = wrap(zc * PER + j, nz) * nxy;
  const float* __restrict__ src = prm.f_in + (size_t)A * prm.n;
  const float4* At = reinterpret_cast<const float4*>(sA + (size_t)((dx + 2 * dy) * 8 * 32 + lane) * 8);
  // Difference form: every row of A sums to 1, so per z row j and column
  // (cell) n the contraction is ref + A (F - ref) with ref = the source value
  // in the middle of the 2 x 2 cell window of that z row (the own cell's
  // corner node that faces the upwind cells), so that the differences take
  // both signs.  The tensor cores then accumulate only the small
  // differences: their FP32 accumulation truncates, which biases a sum of the
  // full values by about an ulp of it per step (measured on the 32^3 D3Q27
  // KBC Taylor-Green: 1.3e-5 relative error of u after 500 steps with the
  // full values, 9.9e-7 with the differences, 2.5e-7 for the scalar path).
  float ref[PER];
  const int gy_ref = wrap(by * PER + (sy > 0 ? 0 : P), ny);
  const int gx_ref = 4 * X + (sx > 0 ? 0 : P);
#pragma unroll
  for (int j = 0; j < PER; ++j) ref[j] = __ldg(src + (zoff[j] + gy_ref * nx + gx_ref));
  // The main products a_hi b_hi of each step go to a fresh accumulator and
  // are added in FP32 (round to nearest); only the two small correction
  // products accumulate on the tensor cores across steps.
  float acc[PER][4], cor[PER][4];
#pragma unroll
  for (int j = 0; j < PER; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[j][e] = cor[j][e] = 0.f;
#pragma unroll 2
  for (int st = 0; st < 8; ++st) {
    const int cys = st & 3, uy = st >> 2;
    const int gy = wrap((by - uy * sy) * PER + cys, ny);
    const float4 h = At[st * 32 * 2], l = At[st * 32 * 2 + 1];
    const unsigned ah[4] = {__float_as_uint(h.x), __float_as_uint(h.y), __float_as_uint(h.z), __float_as_uint(h.w)};
    const unsigned al[4] = {__float_as_uint(l.x), __float_as_uint(l.y), __float_as_uint(l.z), __float_as_uint(l.w)};
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const float* row = src + (zoff[j] + gy * nx);
      const float b0 = __ldg(row + bo0) - ref[j], b1 = __ldg(row + bo1) - ref[j];
      const unsigned b0h = tf32_rna(b0), b1h = tf32_rna(b1);
      const unsigned b0l = tf32_rna(b0 - __uint_as_float(b0h)), b1l = tf32_rna(b1 - __uint_as_float(b1h));
      float pm[4] = {0.f, 0.f, 0.f, 0.f};
      mma_tf32(pm, ah, b0h, b1h);
      mma_tf32(cor[j], al, b0h, b1h);
      mma_tf32(cor[j], ah, b0l, b1l);
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[j][e] += pm[e];
    }
  }
  // per z row T_j = ref_j + acc_j (the references of the thread's output
  // columns 2t, 2t + 1 come from lanes 8t, 8t + 4), then the z factor in the
  // difference form around the dominant row J0; the four values go to the
  // owning warps' arrays: c0 (g, 2t), c1 (g, 2t+1), c2 (g+8, 2t), c3 (g+8,
  // 2t+1); row r = cx + 4 cy, column = cell 8 warp + col
  float rc[PER][2];
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    rc[j][0] = __shfl_sync(0xffffffffu, ref[j], 8 * t);
    rc[j][1] = __shfl_sync(0xffffffffu, ref[j], 8 * t + 4);
  }
  const int J0 = win_j0<P, true, sz>(cz);
  float o[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    float T[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) T[j] = rc[j][e & 1] + (acc[j][e] + cor[j][e]);
    float tj0 = T[0];
#pragma unroll
    for (int j = 1; j < PER; ++j) tj0 = j == J0 ? T[j] : tj0;
    float v = 0.f;
#pragma unroll
    for (int j = 0; j < PER; ++j)
      if (j != J0) v = fma(prm.W.w[2][dz][cz][j], T[j] - tj0, v);
    o[e] = v + tj0;
  }
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int r = g + ((e & 2) ? 8 : 0);
    const int cx = r & 3, cy = r >> 2;
    const int cell = 8 * warp + 2 * t + (e & 1);
    S_all[((size_t)cy * Q + A) * NPW + cell * PER + cx] = o[e];
  }
}

// CTA: WARPS warps, each owning RPW = 32 / L consecutive x rows (y, z); the
// CTA covers WARPS * RPW rows of one z.  Requires nx = L (P + 1) (DG), ny a
// multiple of WARPS * RPW.
//
// MMA: the corner directions of D3Q27 in the tensor-core form above (p = 3,
// FP32, L = 32, 4 warps: the CTA is one y cell of one z row); the dynamic
// shared memory then ends with the A table.
//
// ZS: the directions with y and z components with z sharing (above).
// DGT = false: FE_Q (continuous) nodes.  A lane owns its cell's nodes
// 0 .. p - 1 (PER = p; node p is node 0 of the next cell), a window spans
// p + 1 nodes, and the x window's extra node comes from the next lane.
template <class S, class Real, int COLL, int P, int L, int WARPS, int MINB, bool MMA = false, bool ZS = false,
          bool DGT = true>
__global__ void __launch_bounds__(32 * WARPS, MINB) k_sl_cell(const __grid_constant__ RowParams<Real> prm) {
  constexpr bool DEV = sizeof(Real) == 4;
  constexpr int Q = S::Q;
  constexpr int PER = DGT ? P + 1 : P;  // nodes per cell row (the node period)
  constexpr int NW = P + 1;             // window length
  constexpr int GW = L > 32 ? L / 32 : 1;    // warps per x row
  constexpr int RPW = L >= 32 ? 1 : 32 / L;  // x rows per warp
  constexpr int NPW = 32 * PER;  // nodes per warp
  static_assert((L & (L - 1)) == 0 && L >= 8 && L <= 128, "L: a power of two, 8 .. 128 cells per x row");
  static_assert(GW == 1 || (WARPS % GW == 0 && WARPS / GW <= 4 && !ZS && !MMA),
                "several warps per row: whole rows per CTA, one named barrier per row, no z sharing");
  static_assert(!MMA || (Q == 27 && P == 3 && L == 32 && WARPS == 4 && DEV), "tensor-core corners: D3Q27, p=3, FP32");
  static_assert(!ZS || (S::D == 3 && !MMA && 2 * zs_slots_per_buffer<S, P, L, WARPS, DGT>() <= Q - 1 - n_yz<S>()),
                "z sharing: the two buffers must fit in the slots of the other directions");
  static_assert(!MMA || DGT, "tensor-core corners: DG");
  extern __shared__ __align__(16) unsigned char cell_smem[];
  __shared__ Real sw[row_table_size<P, DGT>()];
  fill_row_table<Real, P, DGT>(sw, prm.W.w, threadIdx.x, 32 * WARPS);
  float* sA = reinterpret_cast<float*>(cell_smem) + (size_t)WARPS * Q * NPW;
  if constexpr (MMA) fill_corner_table<P>(sA, prm.W.w, threadIdx.x, 32 * WARPS);
  __syncthreads();
  using Tab = const Real (*)[2][PER][P + 1];
  Tab tw = reinterpret_cast<Tab>(sw);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Real* Sw = reinterpret_cast<Real*>(cell_smem) + (size_t)warp * Q * NPW;
  // cell values at the warps' edges (several warps per row), two buffers
  __shared__ Real s_edge[2][GW > 1 ? WARPS : 1][2][PER];
  (void)s_edge;
  const int nx = prm.nx, ny = prm.ny, nz = prm.nz;
  const int nxy = nx * ny;
  const int rows_per_cta = GW > 1 ? WARPS / GW : WARPS * RPW;
  const int by = blockIdx.x % (ny / rows_per_cta);
  const int z = blockIdx.x / (ny / rows_per_cta);
  const int r = GW > 1 ? 0 : lane / L;                        // row of this lane within the warp
  const int X = GW > 1 ? (warp % GW) * 32 + lane : lane % L;  // cell along x
  const int y = by * rows_per_cta + (GW > 1 ? warp / GW : warp * RPW + r);
  const int cy = y % PER, cz = z % PER;
  const int x0 = X * PER;
  // the lane's y and z window rows per displacement sign (0: positive, 1:
  // negative) in the rotated order (slot 0 the dominant row), as element
  // offsets: computed once for all directions instead of per direction
  int yrow[2][NW], zrow[2][NW];
  {
    const int ws[4] = {win_start<P, DGT, 1>(y, cy), win_start<P, DGT, -1>(y, cy),
                       win_start<P, DGT, 1>(z, cz), win_start<P, DGT, -1>(z, cz)};
    const int j0[4] = {win_j0<P, DGT, 1>(cy), win_j0<P, DGT, -1>(cy), win_j0<P, DGT, 1>(cz),
                       win_j0<P, DGT, -1>(cz)};
#pragma unroll
    for (int j = 0; j < NW; ++j) {
#pragma unroll
      for (int d = 0; d < 2; ++d) {
        const int ry = j0[d] + j, rz = j0[2 + d] + j;
        yrow[d][j] = wrap(ws[d] + (ry > P ? ry - NW : ry), ny) * nx;
        zrow[d][j] = wrap(ws[2 + d] + (rz > P ? rz - NW : rz), nz) * nxy;
      }
    }
  }
  const int yself = y * nx, zself = z * nxy;

  // rest population: copied
  {
    Real v[PER];
    load_cell<PER>(prm.f_in + (size_t)z * nxy + (size_t)y * nx + x0, v);
    store_cell<PER>(Sw + lane * PER, v);
  }

  static_for<0, Q - 1>([&](auto K) {
    constexpr int A = cell_order<S, ZS>(decltype(K)::value);
    constexpr int sx = S::e(A, 0), sy = S::e(A, 1), sz = S::D == 3 ? S::e(A, 2) : 0;
    if constexpr (ZS && sy != 0 && sz != 0) {
      // z sums of the CTA's union rows into buffer K & 1, then this row's y sum
      constexpr int dy = sy > 0 ? 0 : 1, dz = sz > 0 ? 0 : 1;
      constexpr int R = WARPS * RPW;
      Real* S_all = reinterpret_cast<Real*>(cell_smem);
      const int y0 = by * R;
      const int ybase = ws_row<P, DGT, sy>(y0);
      const int U = ws_row<P, DGT, sy>(y0 + R - 1) - ybase + NW;
      const int* zo = zrow[dz];
      const Real* __restrict__ srcA = prm.f_in + (size_t)A * prm.n;
      auto zaddr = [&](int uu) {  // row uu of this direction's buffer
        const int ch = uu / RPW;
        const int q = zs_slot<S, P, L, WARPS, DGT>(decltype(K)::value & 1, ch / WARPS);
        return S_all + ((size_t)(ch % WARPS) * Q + q) * NPW + (uu % RPW) * nx;
      };
      for (int it = threadIdx.x; it < U * L; it += 32 * WARPS) {
        const int uu = it / L, xc = (it % L) * PER;
        const int gy = wrap(ybase + uu, ny);
        Real Z0[PER], acc[PER];
#pragma unroll
        for (int jz = 0; jz < NW; ++jz) {
          Real v[PER];
          load_cell<PER>(srcA + (zo[jz] + gy * nx + xc), v);
          const Real wz = tw[2][dz][cz][jz];
#pragma unroll
          for (int c = 0; c < PER; ++c) {
            if (jz == 0) {
              Z0[c] = v[c];
              acc[c] = DEV ? Real(0) : wz * v[c];
            } else {
              acc[c] = DEV ? fma(wz, v[c] - Z0[c], acc[c]) : fma(wz, v[c], acc[c]);
            }
          }
        }
        Real* zp = zaddr(uu) + xc;
#pragma unroll
        for (int c = 0; c < PER; ++c) zp[c] = DEV ? acc[c] + Z0[c] : acc[c];
      }
      __syncthreads();
      const int ys = win_start<P, DGT, sy>(y, cy), j0y = win_j0<P, DGT, sy>(cy);
      Real Y0[PER], acc[PER];
#pragma unroll
      for (int jy = 0; jy < NW; ++jy) {
        const int ry = j0y + jy;
        const Real* zp = zaddr(ys - ybase + (ry > P ? ry - NW : ry)) + x0;
        const Real wy = tw[1][dy][cy][jy];
#pragma unroll
        for (int c = 0; c < PER; ++c) {
          const Real v = zp[c];
          if (jy == 0) {
            Y0[c] = v;
            acc[c] = DEV ? Real(0) : wy * v;
          } else {
            acc[c] = DEV ? fma(wy, v - Y0[c], acc[c]) : fma(wy, v, acc[c]);
          }
        }
      }
      Real out[PER];
      if constexpr (sx == 0) {
#pragma unroll
        for (int c = 0; c < PER; ++c) out[c] = DEV ? acc[c] + Y0[c] : acc[c];
      } else {
        Real T[PER];
#pragma unroll
        for (int c = 0; c < PER; ++c) T[c] = DEV ? acc[c] + Y0[c] : acc[c];
        x_factor<DEV, P, L, DGT, sx>(prm.W.w[0][sx > 0 ? 0 : 1], T, out, X, r);
      }
      if constexpr (decltype(K)::value == n_yz<S>() - 1) {
        // the buffers' slots are written by their own directions later on
        __syncthreads();
      }
      store_cell<PER>(Sw + (size_t)A * NPW + lane * PER, out);
      return;
    } else if constexpr (MMA && sx != 0 && sy != 0 && sz != 0) {
      corner_mma<S, P, A>(prm, sA, reinterpret_cast<float*>(cell_smem), by, z, cz, lane, warp);
      return;
    } else {
    constexpr int NJY = sy != 0 ? P + 1 : 1;
    constexpr int NJZ = sz != 0 ? P + 1 : 1;
    constexpr int dy = sy > 0 ? 0 : 1, dz = sz > 0 ? 0 : 1, dx = sx > 0 ? 0 : 1;
    const Real* __restrict__ src = prm.f_in + ((size_t)A * prm.n + x0);  // + 32-bit row offsets
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
        const int zo = sz != 0 ? zrow[dz][jz] : zself;
        Real Y[PER];
        if constexpr (sy != 0) {
          Real y0v[PER], yacc[PER];
#pragma unroll
          for (int jy = 0; jy < NJY; ++jy) {
            Real v[PER];
            load_cell<PER>(src + (zo + yrow[dy][jy]), v);
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
          load_cell<PER>(src + (zo + yself), Y);
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
    } else if constexpr (GW > 1) {
      x_factor_mw<DEV, P, GW, DGT, sx>(prm.W.w[0][dx], T, out, lane, warp, s_edge[xorder<S>(A) & 1]);
    } else {
      x_factor<DEV, P, L, DGT, sx>(prm.W.w[0][dx], T, out, X, r);
    }
    store_cell<PER>(Sw + (size_t)A * NPW + lane * PER, out);
    }
  });
  if constexpr (MMA)
    __syncthreads();  // the corner values come from the CTA's other warps
  else
    __syncwarp();

  // phase 2: collide the warp's nodes, lane-strided
  const int row0 = GW > 1 ? y : by * rows_per_cta + warp * RPW;
  const int xw = GW > 1 ? (warp % GW) * NPW : 0;  // the warp's first node along x
  const Real inv_tau = Real(1) / Real(prm.tau);
#pragma unroll 1
  for (int k = 0; k < PER; ++k) {
    const int t = lane + 32 * k;  // node within the warp's rows (or row part)
    const int rr = GW > 1 ? 0 : t / nx, xx = GW > 1 ? xw + t : t % nx;
    const int node = z * nxy + (row0 + rr) * nx + xx;
    Real fs[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) fs[q] = Sw[(size_t)q * NPW + t];
    Real u[3] = {0, 0, 0};
    Real rho = Real(1);
    if constexpr (COLL == COLL_BGK) {
      rho = collide_bgk<S, DEV, false>(fs, inv_tau, u, false);
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
