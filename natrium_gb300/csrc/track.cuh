// Departure-path tracker shared by the host and the device (restates the
// tracker of SemiLagrangian::fillSparseObject, advection/SemiLagrangian.cpp:
// 145-522, with faceCrossedFirst :525-699, faceCrossedFirstWithoutMapping
// :702-757, the periodic translation of PeriodicBoundary.cpp:184-270 and the
// shape values of SemiLagrangianTools.cpp:15-64).
//
// Every function here is __host__ __device__ and works on a TrackGeom, a
// plain description of the mesh whose vertex pointer is host memory for the
// host tracker and device memory for the device one.  The translation unit
// that compiles this file turns floating-point contraction off on both sides
// (nvcc -fmad=false, host -ffp-contract=off), and the arithmetic uses only
// +, -, *, / and sqrt, which IEEE 754 rounds the same way on the CPU and the
// GPU: the two trackers produce the same rows bit for bit.
#pragma once

#include <math.h>

#include "natgpu_common.h"
#include "sl_mapped.cuh"

namespace natgpu {

struct TrackGeom {
  int D, Q, p, PER;
  int n_ax[3];       // device lattice per axis
  int N[3];          // cells per axis
  int periodic[3];
  int bc[6];         // NAT_BC_* per face (non-periodic axes)
  int mapped;        // MappingQ1 cells (vertices) or the Cartesian box (h)
  long long n;       // nodes per block
  double h[3], dt, cs2_scaled;
  double xi[PMAX1 + 1];
  double es[32][3];  // scaled velocities
  double w[32];
  double rest[32];   // rest state of f (w_i, or the incompressible rest state)
  double uw[6][3];   // wall velocities
  double pv[3][3];   // period vector of each axis
  int opp[32];
  const double* vtx;  // vertices (x fastest, 3 doubles each): host or device memory
};

struct TrackPath {
  int sdir, cell[3];
  double dep[3], c;
  double udep[3];  // unit coordinates of dep in cell (mapped meshes; valid when udep_ok)
  bool udep_ok;
};

__host__ __device__ inline const double* tg_vertex(const TrackGeom& g, int i, int j, int k) {
  const int n0 = g.N[0] + 1, n1 = g.D > 1 ? g.N[1] + 1 : 1;
  return g.vtx + 3 * (((long long)k * n1 + j) * n0 + i);
}

// the 2^D vertices of cell c, in the numbering bx + 2 by + 4 bz
__host__ __device__ inline void tg_cell_vertices(const TrackGeom& g, const int* c, double (*cv)[3]) {
  for (int k = 0; k < (1 << g.D); ++k) {
    const double* v = tg_vertex(g, c[0] + (k & 1), g.D > 1 ? c[1] + ((k >> 1) & 1) : 0,
                                g.D > 2 ? c[2] + ((k >> 2) & 1) : 0);
    for (int r = 0; r < 3; ++r) cv[k][r] = v[r];
  }
}

// The multilinear cell map in polynomial form, x(u) = c0 + u cu + v cv +
// w cw + uv cuv + uw cuw + vw cvw + uvw cuvw (2-D: the first, u, v, uv
// terms), coefficients from the vertices in the numbering bx + 2 by + 4 bz.
struct Q1Coef {
  double c[8][3];  // c0, cu, cv, cw, cuv, cuw, cvw, cuvw
};

__host__ __device__ inline void tg_q1_coef(int D, const double (*v)[3], Q1Coef& q) {
  for (int r = 0; r < 3; ++r) {
    q.c[0][r] = v[0][r];
    q.c[1][r] = v[1][r] - v[0][r];
    q.c[2][r] = v[2][r] - v[0][r];
    q.c[4][r] = (v[3][r] - v[2][r]) - (v[1][r] - v[0][r]);
    if (D == 3) {
      q.c[3][r] = v[4][r] - v[0][r];
      q.c[5][r] = (v[5][r] - v[4][r]) - (v[1][r] - v[0][r]);
      q.c[6][r] = (v[6][r] - v[4][r]) - (v[2][r] - v[0][r]);
      q.c[7][r] = ((v[7][r] - v[6][r]) - (v[5][r] - v[4][r])) - ((v[3][r] - v[2][r]) - (v[1][r] - v[0][r]));
    } else {
      q.c[3][r] = q.c[5][r] = q.c[6][r] = q.c[7][r] = 0.0;
    }
  }
}

// x(u), and the Jacobian dx_r/du_a when J is not null
__host__ __device__ inline void tg_q1_map_c(int D, const Q1Coef& q, const double* u, double* x, double (*J)[3]) {
  const double uu = u[0], vv = u[1], ww = D == 3 ? u[2] : 0.0;
  const double uv = uu * vv, uw = uu * ww, vw = vv * ww, uvw = uv * ww;
  for (int r = 0; r < 3; ++r) x[r] = 0.0;
  if (J)
    for (int r = 0; r < 3; ++r)
      for (int a = 0; a < 3; ++a) J[r][a] = 0.0;
  for (int r = 0; r < D; ++r) {
    if (D == 2) {
      x[r] = q.c[0][r] + uu * q.c[1][r] + vv * q.c[2][r] + uv * q.c[4][r];
      if (J) {
        J[r][0] = q.c[1][r] + vv * q.c[4][r];
        J[r][1] = q.c[2][r] + uu * q.c[4][r];
      }
    } else {
      x[r] = q.c[0][r] + uu * q.c[1][r] + vv * q.c[2][r] + ww * q.c[3][r] + uv * q.c[4][r] + uw * q.c[5][r] +
             vw * q.c[6][r] + uvw * q.c[7][r];
      if (J) {
        J[r][0] = q.c[1][r] + vv * q.c[4][r] + ww * q.c[5][r] + vw * q.c[7][r];
        J[r][1] = q.c[2][r] + uu * q.c[4][r] + ww * q.c[6][r] + uw * q.c[7][r];
        J[r][2] = q.c[3][r] + uu * q.c[5][r] + vv * q.c[6][r] + uv * q.c[7][r];
      }
    }
  }
}

// x(u) of cell c, and the Jacobian dx_r/du_a when J is not null
__host__ __device__ inline void tg_q1_map(const TrackGeom& g, const int* c, const double* u, double* x,
                                          double (*J)[3]) {
  double cv[8][3];
  tg_cell_vertices(g, c, cv);
  Q1Coef q;
  tg_q1_coef(g.D, cv, q);
  tg_q1_map_c(g.D, q, u, x, J);
}

__host__ __device__ inline double tg_det3(const double (*M)[3]) {
  return M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
         M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
}

__host__ __device__ inline double tg_det(int D, const double (*J)[3]) {
  return D == 2 ? J[0][0] * J[1][1] - J[0][1] * J[1][0] : tg_det3(J);
}

// J du = r (Cramer's rule); false for a singular J
__host__ __device__ inline bool tg_solve(int D, const double (*J)[3], const double* r, double* du) {
  const double det = tg_det(D, J);
  if (det == 0.0) return false;
  if (D == 2) {
    du[0] = (J[1][1] * r[0] - J[0][1] * r[1]) / det;
    du[1] = (-J[1][0] * r[0] + J[0][0] * r[1]) / det;
    return true;
  }
  for (int col = 0; col < 3; ++col) {
    double M[3][3];
    for (int row = 0; row < 3; ++row)
      for (int a = 0; a < 3; ++a) M[row][a] = a == col ? r[row] : J[row][a];
    du[col] = tg_det3(M) / det;
  }
  return true;
}

// Unit coordinates of x in cell c (the reference calls
// MappingQ1::transform_real_to_unit_cell): Newton's method from the cell
// centre, each step halved (up to 12 times) until the residual decreases;
// converged once a step is below 1e-14.  False when it cannot converge (the
// reference's ExcTransformationFailed).  The cell's map coefficients are
// computed once per inverse.
__host__ __device__ inline bool tg_q1_inverse(const TrackGeom& g, const int* c, const double* x, double* u) {
  const int D = g.D;
  Q1Coef q;
  {
    double cv[8][3];
    tg_cell_vertices(g, c, cv);
    tg_q1_coef(D, cv, q);
  }
  double y[3], J[3][3], r[3] = {0, 0, 0}, res = 0.0;
  for (int a = 0; a < 3; ++a) u[a] = a < D ? 0.5 : 0.0;
  tg_q1_map_c(D, q, u, y, J);
  for (int a = 0; a < D; ++a) {
    r[a] = y[a] - x[a];
    res += r[a] * r[a];
  }
  for (int it = 0; it < 100; ++it) {
    double du[3] = {0, 0, 0}, step = 1.0, stp = 0.0;
    bool ok = false;
    if (!tg_solve(D, J, r, du)) return false;
    for (int a = 0; a < D; ++a) stp += du[a] * du[a];
    for (int k = 0; k <= 12; ++k, step *= 0.5) {
      double un[3] = {u[0], u[1], u[2]}, yn[3], Jn[3][3], rn[3] = {0, 0, 0}, rs = 0.0;
      for (int a = 0; a < D; ++a) un[a] = u[a] - step * du[a];
      tg_q1_map_c(D, q, un, yn, Jn);
      for (int a = 0; a < D; ++a) {
        rn[a] = yn[a] - x[a];
        rs += rn[a] * rn[a];
      }
      if (rs < res || rs == 0.0) {
        for (int a = 0; a < D; ++a) {
          u[a] = un[a];
          r[a] = rn[a];
        }
        for (int row = 0; row < 3; ++row)
          for (int a = 0; a < 3; ++a) J[row][a] = Jn[row][a];
        res = rs;
        ok = true;
        break;
      }
    }
    if (!ok) return stp < 1e-24;  // stuck at round-off
    if (stp * step * step < 1e-28 || res == 0.0) return true;
  }
  return false;
}

__host__ __device__ inline double tg_snap(double v) {
  return fabs(v) < 1e-10 ? 0.0 : (fabs(v - 1.0) < 1e-10 ? 1.0 : v);
}

// First face of the axis-aligned cell [lo, lo + h] crossed by the segment
// p_in -> p_out (unit coordinates snapped at 1e-10; the x face is taken
// first, later faces only when strictly earlier); -1 if p_out lies in the
// closed cell.  Writes the crossing point.  Restates
// SemiLagrangian::faceCrossedFirst for MappingCartesian (SemiLagrangian.cpp:525-699).
__host__ __device__ inline int tg_face_cartesian(int D, const double* lo, const double* h, const double* p_in,
                                                 const double* p_out, double* p_b) {
  double pi[3], po[3], lambda = 100.0;
  int face = -1;
  for (int a = 0; a < D; ++a) {
    pi[a] = tg_snap((p_in[a] - lo[a]) / h[a]);
    po[a] = tg_snap((p_out[a] - lo[a]) / h[a]);
  }
  for (int a = 0; a < D; ++a) {
    double lam;
    int f;
    if (po[a] < 0) {
      lam = (0 - pi[a]) / (po[a] - pi[a]);
      f = 2 * a;
    } else if (po[a] > 1) {
      lam = (1 - pi[a]) / (po[a] - pi[a]);
      f = 2 * a + 1;
    } else {
      continue;
    }
    if (a == 0 || lam < lambda) {
      lambda = lam;
      face = f;
    }
  }
  if (face < 0) return -1;
  for (int a = 0; a < D; ++a) p_b[a] = lo[a] + tg_snap(pi[a] + (po[a] - pi[a]) * lambda) * h[a];
  return face;
}

// faceCrossedFirstWithoutMapping (SemiLagrangian.cpp:702-757), used when an
// inverse map fails: each face is the plane through its first vertex with
// the normal of its first two edges (SemiLagrangianTools.cpp:151-168); the
// smallest lambda in [0, 1) wins.  Face vertices in the cell numbering
// bx + 2 by + 4 bz.
__host__ __device__ inline int tg_face_planar(const TrackGeom& g, const int* c, const double* p_in,
                                              const double* p_out, double* p_b) {
  constexpr int FV2[4][2] = {{0, 2}, {1, 3}, {0, 1}, {2, 3}};
  constexpr int FV3[6][3] = {{0, 2, 4}, {1, 3, 5}, {0, 4, 1}, {2, 6, 3}, {0, 1, 2}, {4, 5, 6}};
  const int D = g.D;
  double lambda_min = 1.0;
  int index_min = 0;
  for (int i = 0; i < 2 * D; ++i) {
    const double* v[3];
    for (int k = 0; k < D; ++k) {
      const int cv = D == 2 ? FV2[i][k] : FV3[i][k];
      v[k] = tg_vertex(g, c[0] + (cv & 1), c[1] + ((cv >> 1) & 1), D > 2 ? c[2] + ((cv >> 2) & 1) : 0);
    }
    double n[3];
    if (D == 2) {
      n[0] = v[1][1] - v[0][1];
      n[1] = -(v[1][0] - v[0][0]);
    } else {
      double d1[3], d2[3];
      for (int a = 0; a < 3; ++a) {
        d1[a] = v[1][a] - v[0][a];
        d2[a] = v[2][a] - v[0][a];
      }
      n[0] = d1[1] * d2[2] - d1[2] * d2[1];
      n[1] = d1[2] * d2[0] - d1[0] * d2[2];
      n[2] = d1[0] * d2[1] - d1[1] * d2[0];
    }
    double num = 0.0, den = 0.0;
    for (int a = 0; a < D; ++a) {
      num += (p_in[a] - v[0][a]) * n[a];
      den += (p_in[a] - p_out[a]) * n[a];
    }
    const double lam = num / den;
    if (lam < 0) continue;
    if (lam < lambda_min) {
      lambda_min = lam;
      index_min = i;
    }
  }
  if (lambda_min == 1) return -1;
  for (int a = 0; a < D; ++a) p_b[a] = p_in[a] + (p_out[a] - p_in[a]) * lambda_min;
  return index_min;
}

// faceCrossedFirst with the mapping (SemiLagrangian.cpp:525-699): the face
// search of the unit cell on the inverse-mapped points, the crossing point
// mapped back; the planar search when an inverse map fails
// (SemiLagrangian.cpp:280-288).  po_out (when not null) receives the unit
// coordinates of p_out and *po_ok whether its inverse map succeeded.
__host__ __device__ inline int tg_face_q1(const TrackGeom& g, const int* c, const double* p_in, const double* p_out,
                                          double* p_b, double* po_out = nullptr, bool* po_ok = nullptr) {
  double pi[3] = {0, 0, 0}, po[3] = {0, 0, 0};
  const bool ok_in = tg_q1_inverse(g, c, p_in, pi);
  const bool ok_out = ok_in && tg_q1_inverse(g, c, p_out, po);
  if (po_ok) *po_ok = ok_out;
  if (po_out)
    for (int a = 0; a < 3; ++a) po_out[a] = po[a];
  if (!ok_in || !ok_out) return tg_face_planar(g, c, p_in, p_out, p_b);
  const double lo[3] = {0, 0, 0}, one[3] = {1, 1, 1};
  double hu[3] = {0, 0, 0};
  const int face = tg_face_cartesian(g.D, lo, one, pi, po, hu);
  if (face >= 0) tg_q1_map(g, c, hu, p_b, nullptr);
  return face;
}

// Position of the node at Gauss-Lobatto point (xi[l0], xi[l1], xi[l2]) of cell c.
__host__ __device__ inline void tg_node_point(const TrackGeom& g, const int* c, const int* l, double* x) {
  x[0] = x[1] = x[2] = 0.0;
  if (g.mapped) {
    double u[3] = {0, 0, 0};
    for (int a = 0; a < g.D; ++a) u[a] = g.xi[l[a]];
    tg_q1_map(g, c, u, x, nullptr);
    return;
  }
  for (int a = 0; a < g.D; ++a) x[a] = c[a] * g.h[a] + g.xi[l[a]] * g.h[a];
}

// The departure path of one (node at x in cell own, direction alpha): source
// direction, cell and point where it ends, wall term; returns the number of
// wall hits (-1: the lifetime cap was reached, identity row).
__host__ __device__ inline int tg_trace(const TrackGeom& g, const double* x, const int* own, int alpha,
                                        TrackPath& P) {
  const int D = g.D;
  // defaults (also what an identity row of the lifetime cap uses)
  P.sdir = alpha;
  P.c = 0.0;
  P.udep_ok = false;
  for (int a = 0; a < 3; ++a) {
    P.cell[a] = own[a];
    P.dep[a] = x[a];
    P.udep[a] = 0.0;
  }
  double udep[3] = {0, 0, 0};
  bool udep_ok = false;
  int cdir = alpha, hit_dn = 0, hits = 0, life = 0;
  int cell[3] = {own[0], own[1], own[2]};
  double cur[3] = {x[0], x[1], x[2]}, dep[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) dep[a] = x[a] - g.dt * g.es[alpha][a];
  double c = 0.0;
  for (;;) {
    if (++life > 50) {  // lifetime cap (SemiLagrangian.cpp:252-271): identity row; the
      P.c = c;          // wall terms of the hits before it stay registered
      return -1;
    }
    double lo[3], pb[3];
    for (int a = 0; a < D; ++a) lo[a] = cell[a] * g.h[a];
    const int face = g.mapped ? tg_face_q1(g, cell, cur, dep, pb, udep, &udep_ok)
                              : tg_face_cartesian(D, lo, g.h, cur, dep, pb);
    if (face < 0) break;
    const int ax = face / 2, upper = face % 2;
    const bool at_boundary = upper ? (cell[ax] == g.N[ax] - 1) : (cell[ax] == 0);
    if (at_boundary && !g.periodic[ax] && g.bc[face] == 1 /* NAT_BC_VELOCITY_BOUNCE_BACK */) {
      double dist = 0.0, ve = 0.0, exu = 0.0;
      cdir = g.opp[cdir];
      for (int a = 0; a < D; ++a) {
        dist += (dep[a] - pb[a]) * (dep[a] - pb[a]);
        ve += g.es[cdir][a] * g.es[cdir][a];
      }
      dist = sqrt(dist);
      ve = sqrt(ve);
      for (int a = 0; a < D; ++a) {
        cur[a] = pb[a];
        dep[a] = cur[a] - g.es[cdir][a] * dist / ve;
      }
      for (int a = 0; a < D; ++a) exu += g.uw[face][a] * g.es[alpha][a];
      c += 2.0 * g.w[alpha] * 1.0 * exu / g.cs2_scaled;
      ++hits;
      continue;
    }
    if (at_boundary && !g.periodic[ax]) {  // do-nothing
      for (int a = 0; a < D; ++a) {
        cur[a] = dep[a] + g.dt * g.es[cdir][a];
        dep[a] = cur[a] + g.dt * g.es[cdir][a];
      }
      cdir = g.opp[cdir];
      hit_dn = 1;
      ++hits;
      continue;
    }
    for (int a = 0; a < D; ++a) cur[a] = pb[a];
    if (at_boundary) {  // periodic: translate by the axis' period vector
      for (int a = 0; a < D; ++a) {
        const double shift = upper ? -g.pv[ax][a] : g.pv[ax][a];
        cur[a] += shift;
        dep[a] += shift;
      }
      cell[ax] = upper ? 0 : g.N[ax] - 1;
    } else {
      cell[ax] += upper ? 1 : -1;
    }
  }
  if (hit_dn) cdir = g.opp[cdir];  // SemiLagrangian.cpp:312-316
  P.sdir = cdir;
  P.c = c;
  // the last face check ran on (cell, dep): its inverse map of dep is the
  // departure point's unit coordinates
  P.udep_ok = g.mapped && udep_ok;
  for (int a = 0; a < 3; ++a) {
    P.cell[a] = cell[a];
    P.dep[a] = dep[a];
    P.udep[a] = udep[a];
  }
  return hits;
}

// Lagrange basis l_j(x) on the Gauss-Lobatto points xi[0..p]
__host__ __device__ inline double tg_lagrange(int p, const double* xi, int j, double x) {
  double v = 1.0;
  for (int k = 0; k <= p; ++k)
    if (k != j) v *= (x - xi[k]) / (xi[j] - xi[k]);
  return v;
}

// One departure-point row of a mapped mesh (sl_mapped.cuh): direction alpha
// (1..Q-1) of node `node`: the first source node of the departure cell
// (sdir * n + node index), the unit point, the 1-D Lagrange values, the
// constants of the plain and the deviation storage, and the flags.
struct TrackRow {
  long long base;
  double uu[3];
  double l1[3][PMAX1];
  double c_plain, c_dev;
  unsigned char flags;
  int cell[3];
};

// Returns 0, or 1 when the inverse map of the departure cell fails at the
// departure point (the reference throws there).
__host__ __device__ inline int tg_row(const TrackGeom& g, long long node, int alpha, TrackRow& R) {
  const int D = g.D, p = g.p, PER = g.PER;
  const int idx[3] = {(int)(node % g.n_ax[0]), (int)((node / g.n_ax[0]) % g.n_ax[1]),
                      (int)(node / ((long long)g.n_ax[0] * g.n_ax[1]))};
  int own[3] = {0, 0, 0}, loc[3] = {0, 0, 0};
  for (int a = 0; a < D; ++a) {
    own[a] = idx[a] / PER;
    loc[a] = idx[a] % PER;
  }
  double x[3];
  tg_node_point(g, own, loc, x);
  TrackPath P;
  const int hits = tg_trace(g, x, own, alpha, P);
  const bool identity = hits < 0;
  const int sdir = identity ? alpha : P.sdir;
  int cell[3] = {own[0], own[1], own[2]};
  if (!identity)
    for (int a = 0; a < D; ++a) cell[a] = P.cell[a];
  for (int a = 0; a < 3; ++a) R.cell[a] = cell[a];
  for (int a = 0; a < 3; ++a)
    for (int j = 0; j < PMAX1; ++j) R.l1[a][j] = (a >= D && j == 0) ? 1.0 : 0.0;
  double ud[3] = {0, 0, 0};
  if (!identity && g.mapped) {
    if (P.udep_ok) {
      for (int a = 0; a < 3; ++a) ud[a] = P.udep[a];
    } else if (!tg_q1_inverse(g, cell, P.dep, ud)) {
      return 1;
    }
  }
  for (int a = 0; a < 3; ++a) R.uu[a] = 0.0;
  for (int a = 0; a < D; ++a) {
    if (identity) {
      cell[a] = own[a];
      R.uu[a] = g.xi[idx[a] % PER];
      for (int j = 0; j <= p; ++j) R.l1[a][j] = (j == idx[a] % PER) ? 1.0 : 0.0;
      continue;
    }
    double ul = g.mapped ? ud[a] : (P.dep[a] - cell[a] * g.h[a]) / g.h[a];
    if (fabs(ul) < 1e-10) ul = 0.0;
    if (fabs(ul - 1.0) < 1e-10) ul = 1.0;
    R.uu[a] = ul;
    for (int j = 0; j <= p; ++j) R.l1[a][j] = tg_lagrange(p, g.xi, j, ul);
  }
  const int np1 = p + 1;
  const int nloc = D == 3 ? np1 * np1 * np1 : np1 * np1;
  double wrest = 0.0;
  bool tiny = false;
  for (int li = 0; li < nloc; ++li) {
    const int lx = li % np1, ly = (li / np1) % np1, lz = D == 3 ? li / (np1 * np1) : 0;
    const double v = R.l1[0][lx] * R.l1[1][ly] * (D == 3 ? R.l1[2][lz] : 1.0);
    if (fabs(v) < 1e-10) {  // SemiLagrangian.cpp:483
      if (v != 0.0) tiny = true;
      continue;
    }
    wrest += v * g.rest[sdir];
  }
  const long long first = ((long long)(cell[2] * PER) * g.n_ax[1] + cell[1] * PER) * g.n_ax[0] + cell[0] * PER;
  R.base = sdir * g.n + first;
  R.c_plain = P.c;
  R.c_dev = P.c + wrest - g.rest[alpha];
  unsigned char fl = tiny ? (unsigned char)MAP_TINY : 0;
  for (int a = 0; a < D; ++a)
    if (PER == p && cell[a] == g.N[a] - 1) fl |= (unsigned char)(1u << a);  // FE_Q wrap
  R.flags = fl;
  for (int a = 0; a < 3; ++a) R.cell[a] = cell[a];
  return 0;
}

}  // namespace natgpu
