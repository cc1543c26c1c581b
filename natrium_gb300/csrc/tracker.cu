// Host departure-path tracker of libnatgpu.so (restates the tracker of
// SemiLagrangian::fillSparseObject, advection/SemiLagrangian.cpp:145-522):
//  - the face search on Cartesian and on MappingQ1 cells
//    (SemiLagrangian.cpp:525-757), wall hits and periodic translations;
//  - the sparse rows of the wall nodes (k_wall_rows streams them);
//  - the departure-point rows of mapped meshes (sl_mapped.cuh) and the mapped
//    mesh's setup (period vectors, Jacobian quadrature weights).
// Runs once per time step size, on all host threads.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "sl_mapped.cuh"
#include "solver.h"

namespace natgpu {
namespace api {

// ---- wall boundaries ----------------------------------------------------------
// Rows of the streaming operator whose departure path meets a wall face,
// evaluated as sparse rows after the interior streaming (the interior kernel
// computes those rows with the periodic window; this overwrites them):
//   f_out[dst] = sum_k w_k f_in[col_k] + c
// (SemiLagrangian.cpp:354-399 for the rows, SemiLagrangianBoundaryHandler::apply
// and VelocityNeqBounceBack.cpp:137-194 for the wall-velocity term c).
template <class Real>
__global__ void k_wall_rows(int nbr, const int* __restrict__ dst, const int* __restrict__ ptr,
                            const int* __restrict__ col, const Real* __restrict__ w, const double* __restrict__ cst,
                            int cst_slot, const Real* __restrict__ f_in, Real* __restrict__ f_out) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nbr; r += gridDim.x * blockDim.x) {
    Real acc = Real(cst[4 * r + cst_slot]);
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) acc = fma(w[k], f_in[col[k]], acc);
    f_out[dst[r]] = acc;
  }
}

// First face of the axis-aligned cell [lo, lo + h] crossed by the segment
// p_in -> p_out (unit coordinates snapped at 1e-10; the x face is taken
// first, later faces only when strictly earlier); -1 if p_out lies in the
// closed cell.  Writes the crossing point.  Restates
// SemiLagrangian::faceCrossedFirst for MappingCartesian (SemiLagrangian.cpp:525-699).
int face_crossed_first(int D, const double* lo, const double* h, const double* p_in, const double* p_out,
                       double* p_b) {
  double pi[3], po[3], lambda = 100.0;
  int face = -1;
  auto snap = [](double v) { return fabs(v) < 1e-10 ? 0.0 : (fabs(v - 1.0) < 1e-10 ? 1.0 : v); };
  for (int a = 0; a < D; ++a) {
    pi[a] = snap((p_in[a] - lo[a]) / h[a]);
    po[a] = snap((p_out[a] - lo[a]) / h[a]);
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
  for (int a = 0; a < D; ++a) p_b[a] = lo[a] + snap(pi[a] + (po[a] - pi[a]) * lambda) * h[a];
  return face;
}

// ---- MappingQ1: multilinear image of the unit cell from its 2^D vertices ----
const double* grid_vertex(const nat_solver* s, int i, int j, int k) {
  const int n0 = s->spec.cells[0] + 1, n1 = s->D > 1 ? s->spec.cells[1] + 1 : 1;
  return s->vtx.data() + 3 * (((long long)k * n1 + j) * n0 + i);
}

// x(u) of cell c, and the Jacobian dx_r/du_a when J is not null
void q1_map(const nat_solver* s, const int* c, const double* u, double* x, double (*J)[3]) {
  const int D = s->D;
  for (int r = 0; r < 3; ++r) {
    x[r] = 0.0;
    if (J)
      for (int a = 0; a < 3; ++a) J[r][a] = 0.0;
  }
  for (int k = 0; k < (1 << D); ++k) {
    const int b[3] = {k & 1, (k >> 1) & 1, (k >> 2) & 1};
    double phi = 1.0, dphi[3];
    for (int a = 0; a < D; ++a) phi *= b[a] ? u[a] : 1.0 - u[a];
    for (int a = 0; a < D; ++a) {
      dphi[a] = b[a] ? 1.0 : -1.0;
      for (int q = 0; q < D; ++q)
        if (q != a) dphi[a] *= b[q] ? u[q] : 1.0 - u[q];
    }
    const double* v = grid_vertex(s, c[0] + b[0], D > 1 ? c[1] + b[1] : 0, D > 2 ? c[2] + b[2] : 0);
    for (int r = 0; r < D; ++r) {
      x[r] += phi * v[r];
      if (J)
        for (int a = 0; a < D; ++a) J[r][a] += dphi[a] * v[r];
    }
  }
}

double det3(const double (*M)[3]) {
  return M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
         M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
}

double q1_det(int D, const double (*J)[3]) { return D == 2 ? J[0][0] * J[1][1] - J[0][1] * J[1][0] : det3(J); }

// J du = r (Cramer's rule); false for a singular J
bool q1_solve(int D, const double (*J)[3], const double* r, double* du) {
  const double det = q1_det(D, J);
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
    du[col] = det3(M) / det;
  }
  return true;
}

// Unit coordinates of x in cell c (the reference calls
// MappingQ1::transform_real_to_unit_cell): Newton's method from the cell
// centre, each step halved (up to 12 times) until the residual decreases;
// converged once a step is below 1e-14.  False when it cannot converge (the
// reference's ExcTransformationFailed).
bool q1_inverse(const nat_solver* s, const int* c, const double* x, double* u) {
  const int D = s->D;
  double y[3], J[3][3], r[3] = {0, 0, 0}, res = 0.0;
  for (int a = 0; a < 3; ++a) u[a] = a < D ? 0.5 : 0.0;
  q1_map(s, c, u, y, J);
  for (int a = 0; a < D; ++a) {
    r[a] = y[a] - x[a];
    res += r[a] * r[a];
  }
  for (int it = 0; it < 100; ++it) {
    double du[3] = {0, 0, 0}, step = 1.0, stp = 0.0;
    bool ok = false;
    if (!q1_solve(D, J, r, du)) return false;
    for (int a = 0; a < D; ++a) stp += du[a] * du[a];
    for (int k = 0; k <= 12; ++k, step *= 0.5) {
      double un[3] = {u[0], u[1], u[2]}, yn[3], Jn[3][3], rn[3] = {0, 0, 0}, rs = 0.0;
      for (int a = 0; a < D; ++a) un[a] = u[a] - step * du[a];
      q1_map(s, c, un, yn, Jn);
      for (int a = 0; a < D; ++a) {
        rn[a] = yn[a] - x[a];
        rs += rn[a] * rn[a];
      }
      if (rs < res || rs == 0.0) {
        for (int a = 0; a < D; ++a) {
          u[a] = un[a];
          r[a] = rn[a];
        }
        memcpy(J, Jn, sizeof(Jn));
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

// faceCrossedFirstWithoutMapping (SemiLagrangian.cpp:702-757), used when an
// inverse map fails: each face is the plane through its first vertex with
// the normal of its first two edges (SemiLagrangianTools.cpp:151-168); the
// smallest lambda in [0, 1) wins.  Face vertices in the cell numbering
// bx + 2 by + 4 bz.
int face_crossed_first_planar(const nat_solver* s, const int* c, const double* p_in, const double* p_out,
                              double* p_b) {
  static const int FV2[4][2] = {{0, 2}, {1, 3}, {0, 1}, {2, 3}};
  static const int FV3[6][3] = {{0, 2, 4}, {1, 3, 5}, {0, 4, 1}, {2, 6, 3}, {0, 1, 2}, {4, 5, 6}};
  const int D = s->D;
  double lambda_min = 1.0;
  int index_min = 0;
  for (int i = 0; i < 2 * D; ++i) {
    const double* v[3];
    for (int k = 0; k < D; ++k) {
      const int cv = D == 2 ? FV2[i][k] : FV3[i][k];
      v[k] = grid_vertex(s, c[0] + (cv & 1), c[1] + ((cv >> 1) & 1), D > 2 ? c[2] + ((cv >> 2) & 1) : 0);
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
// (SemiLagrangian.cpp:280-288).
int face_crossed_first_q1(const nat_solver* s, const int* c, const double* p_in, const double* p_out,
                          double* p_b) {
  double pi[3] = {0, 0, 0}, po[3] = {0, 0, 0};
  if (!q1_inverse(s, c, p_in, pi) || !q1_inverse(s, c, p_out, po))
    return face_crossed_first_planar(s, c, p_in, p_out, p_b);
  static const double lo[3] = {0, 0, 0}, one[3] = {1, 1, 1};
  double hu[3] = {0, 0, 0};
  const int face = face_crossed_first(s->D, lo, one, pi, po, hu);
  if (face >= 0) q1_map(s, c, hu, p_b, nullptr);
  return face;
}

// Position of the node at Gauss-Lobatto point (xi[l0], xi[l1], xi[l2]) of cell c.
void node_point(const nat_solver* s, const int* c, const int* l, const double* xi, double* x) {
  x[0] = x[1] = x[2] = 0.0;
  if (s->mapped) {
    double u[3] = {0, 0, 0};
    for (int a = 0; a < s->D; ++a) u[a] = xi[l[a]];
    q1_map(s, c, u, x, nullptr);
    return;
  }
  for (int a = 0; a < s->D; ++a) x[a] = c[a] * s->h[a] + xi[l[a]] * s->h[a];
}

void free_mapped_rows(nat_solver* s) {
  cudaFree(s->d_mp_base);
  cudaFree(s->d_mp_u);
  cudaFree(s->d_mp_c);
  cudaFree(s->d_mp_flags);
  s->d_mp_base = nullptr;
  s->d_mp_u = s->d_mp_c = nullptr;
  s->d_mp_flags = nullptr;
}

// Departure-point rows to the device in the solve's arithmetic type.
int upload_mapped_rows(nat_solver* s, const std::vector<int>& base, const std::vector<double>& u,
                       const std::vector<double>& c2, const std::vector<unsigned char>& flags) {
  const bool f64 = s->spec.precision == NAT_FP64;
  const size_t es = f64 ? 8 : 4, nr = base.size();
  // every gathered index must address the Q x n_dev state
  const int P = s->spec.order;
  const long long qn = (long long)s->Q * s->n_dev;
  const long long st[3] = {1, s->n_ax[0], (long long)s->n_ax[0] * s->n_ax[1]};
  for (size_t r = 0; r < nr; ++r) {
    long long lo = base[r], hi = base[r];
    for (int a = 0; a < s->D; ++a) {
      if (flags[r] & (1u << a)) {
        lo += (long long)(P - s->n_ax[a]) * st[a];
        hi += (long long)(P - 1) * st[a];
      } else {
        hi += (long long)P * st[a];
      }
    }
    if (lo < 0 || hi >= qn)
      return fail(s, NAT_ERR_CUDA, "internal error: departure-point row %zu addresses %lld..%lld", r, lo, hi);
  }
  std::vector<unsigned char> ub(u.size() * es), cb(nr * es);
  for (size_t i = 0; i < u.size(); ++i) {
    if (f64)
      memcpy(&ub[i * 8], &u[i], 8);
    else {
      const float v = (float)u[i];
      memcpy(&ub[i * 4], &v, 4);
    }
  }
  for (size_t r = 0; r < nr; ++r) {
    const double c = c2[2 * r + (f64 ? 0 : 1)];
    if (f64)
      memcpy(&cb[r * 8], &c, 8);
    else {
      const float v = (float)c;
      memcpy(&cb[r * 4], &v, 4);
    }
  }
  auto alloc = [&](void** p, size_t bytes) -> bool {
    if (cudaMalloc(p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return true;
  };
  if (!alloc((void**)&s->d_mp_base, sizeof(int) * nr) || !alloc(&s->d_mp_u, ub.size()) ||
      !alloc(&s->d_mp_c, cb.size()) || !alloc((void**)&s->d_mp_flags, nr))
    return fail(s, NAT_ERR_OOM, "cudaMalloc of the departure-point rows failed");
  CK(cudaMemcpy(s->d_mp_base, base.data(), sizeof(int) * nr, cudaMemcpyHostToDevice), "mapped rows");
  CK(cudaMemcpy(s->d_mp_u, ub.data(), ub.size(), cudaMemcpyHostToDevice), "mapped rows");
  CK(cudaMemcpy(s->d_mp_c, cb.data(), cb.size(), cudaMemcpyHostToDevice), "mapped rows");
  CK(cudaMemcpy(s->d_mp_flags, flags.data(), nr, cudaMemcpyHostToDevice), "mapped rows");
  return NAT_OK;
}

int build_wall_rows(nat_solver* s) {
  cudaFree(s->d_br_dst);
  cudaFree(s->d_br_ptr);
  cudaFree(s->d_br_col);
  cudaFree(s->d_br_w);
  cudaFree(s->d_br_wf);
  cudaFree(s->d_br_c);
  cudaFree(s->d_bn_node);
  s->d_br_dst = s->d_br_ptr = s->d_br_col = s->d_bn_node = nullptr;
  s->d_br_w = s->d_br_c = nullptr;
  s->d_br_wf = nullptr;
  s->nbr = 0;
  s->nbn = 0;
  free_mapped_rows(s);
  if (!s->walls && !s->mapped) return NAT_OK;
  HostStencil hs;
  get_host_stencil(s->spec.stencil, &hs, s->spec.scaling);
  const int D = s->D, Q = s->Q, p = s->spec.order, PER = s->period;
  double xi[PMAX1 + 1];
  gl_points(p, xi);
  double es[32][3];
  int opp[32];
  for (int i = 0; i < Q; ++i)
    for (int a = 0; a < 3; ++a) es[i][a] = a < D ? hs.e[i][a] * s->spec.scaling : 0.0;
  for (int i = 0; i < Q; ++i) {
    opp[i] = 0;
    for (int j = 0; j < Q; ++j)
      if (es[j][0] == -es[i][0] && es[j][1] == -es[i][1] && es[j][2] == -es[i][2]) opp[i] = j;
  }
  double grest[32];
  for (int q = 0; q < Q; ++q) grest[q] = s->rest[q] * s->gref;
  const long long n = s->n_dev;
  const int* N = s->spec.cells;
  // the departure path of one (node, direction): source direction, cell and
  // point where it ends, wall term; returns the number of wall hits (-1: the
  // lifetime cap was reached, identity row)
  struct Path {
    int sdir, cell[3];
    double dep[3], c;
  };
  auto trace = [&](const double* x, const int* own, int alpha, Path& P) -> int {
    // defaults (also what an identity row of the lifetime cap uses)
    P.sdir = alpha;
    P.c = 0.0;
    for (int a = 0; a < 3; ++a) {
      P.cell[a] = own[a];
      P.dep[a] = x[a];
    }
    int cdir = alpha, hit_dn = 0, hits = 0, life = 0;
    int cell[3] = {own[0], own[1], own[2]};
    double cur[3] = {x[0], x[1], x[2]}, dep[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) dep[a] = x[a] - s->dt * es[alpha][a];
    double c = 0.0;
    for (;;) {
      if (++life > 50) {  // lifetime cap (SemiLagrangian.cpp:252-271): identity row; the
        P.c = c;          // wall terms of the hits before it stay registered
        return -1;
      }
      double lo[3], pb[3];
      for (int a = 0; a < D; ++a) lo[a] = cell[a] * s->h[a];
      const int face = s->mapped ? face_crossed_first_q1(s, cell, cur, dep, pb)
                                 : face_crossed_first(D, lo, s->h, cur, dep, pb);
      if (face < 0) break;
      const int ax = face / 2, upper = face % 2;
      const bool at_boundary = upper ? (cell[ax] == N[ax] - 1) : (cell[ax] == 0);
      if (at_boundary && !s->spec.periodic[ax] && s->bc[face] == NAT_BC_VELOCITY_BOUNCE_BACK) {
        double dist = 0.0, ve = 0.0, exu = 0.0;
        cdir = opp[cdir];
        for (int a = 0; a < D; ++a) {
          dist += (dep[a] - pb[a]) * (dep[a] - pb[a]);
          ve += es[cdir][a] * es[cdir][a];
        }
        dist = sqrt(dist);
        ve = sqrt(ve);
        for (int a = 0; a < D; ++a) {
          cur[a] = pb[a];
          dep[a] = cur[a] - es[cdir][a] * dist / ve;
        }
        for (int a = 0; a < D; ++a) exu += s->uw[face][a] * es[alpha][a];
        c += 2.0 * hs.w[alpha] * 1.0 * exu / s->cs2_scaled;
        ++hits;
        continue;
      }
      if (at_boundary && !s->spec.periodic[ax]) {  // do-nothing
        for (int a = 0; a < D; ++a) {
          cur[a] = dep[a] + s->dt * es[cdir][a];
          dep[a] = cur[a] + s->dt * es[cdir][a];
        }
        cdir = opp[cdir];
        hit_dn = 1;
        ++hits;
        continue;
      }
      for (int a = 0; a < D; ++a) cur[a] = pb[a];
      if (at_boundary) {  // periodic: translate by the axis' period vector
        for (int a = 0; a < D; ++a) {
          const double shift = upper ? -s->pv[ax][a] : s->pv[ax][a];
          cur[a] += shift;
          dep[a] += shift;
        }
        cell[ax] = upper ? 0 : N[ax] - 1;
      } else {
        cell[ax] += upper ? 1 : -1;
      }
    }
    if (hit_dn) cdir = opp[cdir];  // SemiLagrangian.cpp:312-316
    P.sdir = cdir;
    P.c = c;
    for (int a = 0; a < 3; ++a) {
      P.cell[a] = cell[a];
      P.dep[a] = dep[a];
    }
    return hits;
  };
  // mapped meshes (one population): departure-point rows of every node
  // (sl_mapped.cuh) instead of sparse matrix rows
  const bool dp = s->mapped && !s->thermal;
  std::vector<int> mp_base;
  std::vector<double> mp_u, mp_c;
  std::vector<unsigned char> mp_flags;
  if (dp) {
    if ((long long)Q * n > INT32_MAX) return fail(s, NAT_ERR_UNSUPPORTED, "Q x nodes exceeds 2^31");
    mp_base.assign((size_t)(Q - 1) * n, 0);
    // FP32: unit coordinates; FP64: the 1-D Lagrange values (sl_mapped.cuh)
    mp_u.assign((size_t)(Q - 1) * D * n * (s->spec.precision == NAT_FP64 ? p + 1 : 1), 0.0);
    mp_c.assign((size_t)2 * (Q - 1) * n, 0.0);
    mp_flags.assign((size_t)(Q - 1) * n, 0);
  }
  // rows of the nodes [n0, n1) into one chunk (the chunks run on host
  // threads; departure-point rows go straight to their slots)
  struct Chunk {
    std::vector<int> dst, ptr, col, bnodes;
    std::vector<double> w, cst;
    int rc = NAT_OK;
    char err[256] = {0};
  };
  auto work = [&](long long n0, long long n1, Chunk& C) {
  std::vector<int>& dst = C.dst;
  std::vector<int>& ptr = C.ptr;
  std::vector<int>& col = C.col;
  std::vector<int>& bnodes = C.bnodes;
  std::vector<double>& w = C.w;
  std::vector<double>& cst = C.cst;
  for (long long node = n0; node < n1; ++node) {
    int idx[3] = {(int)(node % s->n_ax[0]), (int)((node / s->n_ax[0]) % s->n_ax[1]),
                  (int)(node / ((long long)s->n_ax[0] * s->n_ax[1]))};
    double x[3] = {0, 0, 0};
    int own[3] = {0, 0, 0}, loc[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) {
      own[a] = idx[a] / PER;
      loc[a] = idx[a] % PER;
    }
    node_point(s, own, loc, xi, x);
    // a node is a wall node when one of its paths meets a wall; all its rows
    // are then evaluated as sparse rows
    Path paths[32];
    int hits[32];
    bool wall_node = false;
    for (int alpha = 1; alpha < Q; ++alpha) {
      hits[alpha] = trace(x, own, alpha, paths[alpha]);
      if (hits[alpha] != 0) wall_node = true;
    }
    if (!wall_node && !s->mapped) continue;
    if (!dp) bnodes.push_back((int)node);
    for (int alpha = 1; alpha < Q; ++alpha) {
      const Path& P = paths[alpha];
      const bool identity = hits[alpha] < 0;
      const int sdir = identity ? alpha : P.sdir;
      int cell[3] = {own[0], own[1], own[2]};
      if (!identity)
        for (int a = 0; a < D; ++a) cell[a] = P.cell[a];
      double l1[3][PMAX1];
      for (int a = 0; a < 3; ++a)
        for (int j = 0; j < PMAX1; ++j) l1[a][j] = (a >= D && j == 0) ? 1.0 : 0.0;
      double ud[3] = {0, 0, 0};
      if (!identity && s->mapped && !q1_inverse(s, cell, P.dep, ud)) {
        C.rc = NAT_ERR_UNSUPPORTED;
        snprintf(C.err, sizeof(C.err),
                 "the inverse map of cell (%d %d %d) failed at a departure point; the mesh is too distorted "
                 "for this time step",
                 cell[0], cell[1], cell[2]);
        return;
      }
      double uu[3] = {0, 0, 0};  // unit coordinates of the departure point
      for (int a = 0; a < D; ++a) {
        if (identity) {
          cell[a] = own[a];
          uu[a] = xi[idx[a] % PER];
          for (int j = 0; j <= p; ++j) l1[a][j] = (j == idx[a] % PER) ? 1.0 : 0.0;
          continue;
        }
        double ul = s->mapped ? ud[a] : (P.dep[a] - cell[a] * s->h[a]) / s->h[a];
        if (fabs(ul) < 1e-10) ul = 0.0;
        if (fabs(ul - 1.0) < 1e-10) ul = 1.0;
        uu[a] = ul;
        for (int j = 0; j <= p; ++j) l1[a][j] = lagrange(p, xi, j, ul);
      }
      const double c = P.c;
      const int np1 = p + 1;
      const int nloc = D == 3 ? np1 * np1 * np1 : np1 * np1;
      double wrest = 0.0, wgrest = 0.0;
      bool tiny = false;
      for (int li = 0; li < nloc; ++li) {
        const int lx = li % np1, ly = (li / np1) % np1, lz = D == 3 ? li / (np1 * np1) : 0;
        const double v = l1[0][lx] * l1[1][ly] * (D == 3 ? l1[2][lz] : 1.0);
        if (fabs(v) < 1e-10) {  // SemiLagrangian.cpp:483
          if (v != 0.0) tiny = true;
          continue;
        }
        wrest += v * s->rest[sdir];
        wgrest += v * grest[sdir];
        if (dp) continue;
        // the FE_Q node p of the last cell of a periodic axis is node 0
        const int ix = (cell[0] * PER + lx) % s->n_ax[0], iy = (cell[1] * PER + ly) % s->n_ax[1],
                  iz = (cell[2] * PER + lz) % s->n_ax[2];
        const long long src = ((long long)iz * s->n_ax[1] + iy) * s->n_ax[0] + ix;
        col.push_back((int)(sdir * n + src));
        w.push_back(v);
      }
      if (dp) {
        // departure-point row: first node of the cell, unit point, constants, flags
        const long long r = (long long)(alpha - 1) * n + node;
        const long long first =
            ((long long)(cell[2] * PER) * s->n_ax[1] + cell[1] * PER) * s->n_ax[0] + cell[0] * PER;
        mp_base[r] = (int)(sdir * n + first);
        if (s->spec.precision == NAT_FP64) {
          for (int a = 0; a < D; ++a)
            for (int j = 0; j <= p; ++j)
              mp_u[(((long long)(alpha - 1) * D + a) * (p + 1) + j) * n + node] = l1[a][j];
        } else {
          for (int a = 0; a < D; ++a) mp_u[((long long)(alpha - 1) * D + a) * n + node] = uu[a];
        }
        mp_c[2 * r] = c;                                // plain f
        mp_c[2 * r + 1] = c + wrest - s->rest[alpha];  // f - w_i storage
        unsigned char fl = tiny ? MAP_TINY : 0;
        for (int a = 0; a < D; ++a)
          if (PER == p && cell[a] == N[a] - 1) fl |= (unsigned char)(1u << a);  // FE_Q wrap
        mp_flags[r] = fl;
        continue;
      }
      if (col.size() > (size_t)INT32_MAX) {
        C.rc = NAT_ERR_UNSUPPORTED;
        snprintf(C.err, sizeof(C.err), "sparse rows exceed 2^31 entries; use fewer nodes");
        return;
      }
      dst.push_back((int)(alpha * n + node));
      ptr.push_back((int)col.size());
      cst.push_back(c);                           // plain f
      cst.push_back(c + wrest - s->rest[alpha]);  // f - w_i storage
      cst.push_back(0.0);                         // plain g: no wall term
      cst.push_back(wgrest - grest[alpha]);       // g - w_i g_ref storage
    }
  }
  };
  const int nthr = (int)std::max<long long>(1, std::min<long long>(std::thread::hardware_concurrency(), n / 256));
  std::vector<Chunk> chunks(nthr);
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nthr; ++t)
      th.emplace_back(work, n * t / nthr, n * (t + 1) / nthr, std::ref(chunks[t]));
    for (auto& t : th) t.join();
  }
  for (const Chunk& C : chunks)
    if (C.rc) return fail(s, C.rc, "%s", C.err);
  std::vector<int> dst, ptr(1, 0), col, bnodes;
  std::vector<double> w, cst;
  for (Chunk& C : chunks) {
    const size_t off = col.size();
    if (off + C.col.size() > (size_t)INT32_MAX)
      return fail(s, NAT_ERR_UNSUPPORTED, "sparse rows exceed 2^31 entries; use fewer nodes");
    for (int v : C.ptr) ptr.push_back((int)(v + off));
    dst.insert(dst.end(), C.dst.begin(), C.dst.end());
    col.insert(col.end(), C.col.begin(), C.col.end());
    bnodes.insert(bnodes.end(), C.bnodes.begin(), C.bnodes.end());
    w.insert(w.end(), C.w.begin(), C.w.end());
    cst.insert(cst.end(), C.cst.begin(), C.cst.end());
    C = Chunk();
  }
  if (dp) return upload_mapped_rows(s, mp_base, mp_u, mp_c, mp_flags);
  s->nbn = (int)bnodes.size();
  s->nbr = (int)dst.size();
  if (s->nbr == 0) return NAT_OK;
  // every index must address the Q x n_dev state (checked before any launch)
  const long long qn = (long long)Q * n;
  for (int v : col)
    if (v < 0 || v >= qn) return fail(s, NAT_ERR_CUDA, "internal error: wall row column %d out of range", v);
  for (int v : dst)
    if (v < 0 || v >= qn) return fail(s, NAT_ERR_CUDA, "internal error: wall row destination %d out of range", v);
  std::vector<float> wf(w.begin(), w.end());
#define WALLOC(ptr_, bytes_)                                                  \
  do {                                                                        \
    if (cudaMalloc((void**)&(ptr_), (bytes_)) != cudaSuccess) {               \
      cudaGetLastError();                                                     \
      return fail(s, NAT_ERR_OOM, "cudaMalloc(%zu) failed", (size_t)(bytes_)); \
    }                                                                         \
  } while (0)
  WALLOC(s->d_br_dst, sizeof(int) * dst.size());
  WALLOC(s->d_br_ptr, sizeof(int) * ptr.size());
  WALLOC(s->d_br_col, sizeof(int) * std::max<size_t>(col.size(), 1));
  WALLOC(s->d_br_w, sizeof(double) * std::max<size_t>(w.size(), 1));
  WALLOC(s->d_br_wf, sizeof(float) * std::max<size_t>(w.size(), 1));
  WALLOC(s->d_br_c, sizeof(double) * cst.size());
  WALLOC(s->d_bn_node, sizeof(int) * bnodes.size());
#undef WALLOC
  CK(cudaMemcpy(s->d_br_dst, dst.data(), sizeof(int) * dst.size(), cudaMemcpyHostToDevice), "wall rows");
  CK(cudaMemcpy(s->d_br_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice), "wall rows");
  if (!col.empty()) {
    CK(cudaMemcpy(s->d_br_col, col.data(), sizeof(int) * col.size(), cudaMemcpyHostToDevice), "wall rows");
    CK(cudaMemcpy(s->d_br_w, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice), "wall rows");
    CK(cudaMemcpy(s->d_br_wf, wf.data(), sizeof(float) * wf.size(), cudaMemcpyHostToDevice), "wall rows");
  }
  CK(cudaMemcpy(s->d_br_c, cst.data(), sizeof(double) * cst.size(), cudaMemcpyHostToDevice), "wall rows");
  CK(cudaMemcpy(s->d_bn_node, bnodes.data(), sizeof(int) * bnodes.size(), cudaMemcpyHostToDevice), "wall nodes");
  return NAT_OK;
}

// Overwrite the wall rows of a streamed buffer (f: slot 0/1, g: slot 2 or none).
int launch_wall_rows(nat_solver* s, const void* in, void* out, bool g_pop) {
  if ((!s->walls && !s->mapped) || s->nbr == 0) return NAT_OK;
  const int grid = std::min((s->nbr + 255) / 256, 152 * 8);
  if (s->spec.precision == NAT_FP64) {
    k_wall_rows<double><<<grid, 256, 0, s->stream>>>(s->nbr, s->d_br_dst, s->d_br_ptr, s->d_br_col, s->d_br_w,
                                                     s->d_br_c, g_pop ? 2 : 0, (const double*)in, (double*)out);
  } else {
    k_wall_rows<float><<<grid, 256, 0, s->stream>>>(s->nbr, s->d_br_dst, s->d_br_ptr, s->d_br_col, s->d_br_wf,
                                                    s->d_br_c, g_pop ? 3 : 1, (const float*)in, (float*)out);
  }
  CK(cudaGetLastError(), "wall rows kernel");
  s->launches++;
  return NAT_OK;
}

// MappingQ1 mesh of nat_spec::vertices: copy, check, period vectors, the
// smallest vertex distance of a cell (utilities/CFDSolverUtilities.cpp:69-84)
// and the per-node quadrature weights (Gauss-Lobatto weight times det J of
// every cell holding the node).  The box lengths become the grid's extents.
int setup_mapping(nat_solver* s, const double* vertices, double* hmin) {
  const int D = s->D;
  const int* N = s->spec.cells;
  const long long nv = (long long)(N[0] + 1) * (N[1] + 1) * (D == 3 ? N[2] + 1 : 1);
  s->vtx.assign(vertices, vertices + 3 * nv);
  for (double v : s->vtx)
    if (!std::isfinite(v)) return fail(s, NAT_ERR_INVALID_ARG, "vertices must be finite");
  s->mapped = true;
  // period vectors: the offset between the vertices of the two faces of an
  // axis, one vector for all of them on a periodic axis
  for (int a = 0; a < D; ++a) {
    const int nb = a == 0 ? 1 : 0, nc = a == 2 ? 1 : 2;
    const int mb = N[nb] + 1, mc = D > 2 ? N[nc] + 1 : 1;
    double lo = 1e300, hi = -1e300;
    for (int ic = 0; ic < mc; ++ic)
      for (int ib = 0; ib < mb; ++ib) {
        int i0[3] = {0, 0, 0}, i1[3] = {0, 0, 0};
        i0[nb] = i1[nb] = ib;
        if (D > 2) i0[nc] = i1[nc] = ic;
        i1[a] = N[a];
        const double* v0 = grid_vertex(s, i0[0], i0[1], i0[2]);
        const double* v1 = grid_vertex(s, i1[0], i1[1], i1[2]);
        for (int b = 0; b < D; ++b) {
          const double d = v1[b] - v0[b];
          if (ib == 0 && ic == 0)
            s->pv[a][b] = d;
          else if (s->spec.periodic[a] && fabs(d - s->pv[a][b]) > 1e-12 * (fabs(d) + 1.0))
            return fail(s, NAT_ERR_INVALID_ARG, "periodic axis %d: the two faces' vertices differ by more than one "
                        "translation", a);
        }
      }
    for (long long k = 0; k < nv; ++k) {
      lo = std::min(lo, s->vtx[3 * k + a]);
      hi = std::max(hi, s->vtx[3 * k + a]);
    }
    s->spec.length[a] = s->spec.periodic[a] ? fabs(s->pv[a][a]) : hi - lo;
    if (!(s->spec.length[a] > 0)) return fail(s, NAT_ERR_INVALID_ARG, "degenerate vertex grid along axis %d", a);
    s->h[a] = s->spec.length[a] / N[a];
  }
  // cells: positive det J at the corners, smallest vertex distance
  const int p = s->spec.order, PER = s->period, np1 = p + 1;
  double xi[PMAX1 + 1], wq[PMAX1 + 1];
  gl_points(p, xi);
  gl_weights(p, xi, wq);
  std::vector<double> mw((size_t)s->n_dev, 0.0);
  *hmin = 1e300;
  const int ncz = D == 3 ? N[2] : 1;
  for (int cz = 0; cz < ncz; ++cz)
    for (int cy = 0; cy < N[1]; ++cy)
      for (int cx = 0; cx < N[0]; ++cx) {
        const int c[3] = {cx, cy, cz};
        const double* cv[8];
        for (int k = 0; k < (1 << D); ++k)
          cv[k] = grid_vertex(s, cx + (k & 1), cy + ((k >> 1) & 1), D > 2 ? cz + ((k >> 2) & 1) : 0);
        for (int i = 0; i < (1 << D); ++i) {
          for (int j = i + 1; j < (1 << D); ++j) {
            double d2 = 0.0;
            for (int a = 0; a < D; ++a) d2 += (cv[i][a] - cv[j][a]) * (cv[i][a] - cv[j][a]);
            *hmin = std::min(*hmin, sqrt(d2));
          }
          const double u[3] = {(double)(i & 1), (double)((i >> 1) & 1), (double)((i >> 2) & 1)};
          double x[3], J[3][3];
          q1_map(s, c, u, x, J);
          if (!(q1_det(D, J) > 0))
            return fail(s, NAT_ERR_INVALID_ARG, "cell (%d %d %d) is inverted or degenerate", cx, cy, cz);
        }
        const int nloc = D == 3 ? np1 * np1 * np1 : np1 * np1;
        for (int li = 0; li < nloc; ++li) {
          const int l[3] = {li % np1, (li / np1) % np1, D == 3 ? li / (np1 * np1) : 0};
          const double u[3] = {xi[l[0]], xi[l[1]], D == 3 ? xi[l[2]] : 0.0};
          double x[3], J[3][3];
          q1_map(s, c, u, x, J);
          double w = q1_det(D, J);
          for (int a = 0; a < D; ++a) w *= wq[l[a]];
          const int ix = (cx * PER + l[0]) % s->n_ax[0], iy = (cy * PER + l[1]) % s->n_ax[1],
                    iz = (cz * PER + l[2]) % s->n_ax[2];
          mw[((size_t)iz * s->n_ax[1] + iy) * s->n_ax[0] + ix] += w;
        }
      }
  if (cudaMalloc((void**)&s->d_mw, sizeof(double) * mw.size()) != cudaSuccess) {
    cudaGetLastError();
    return fail(s, NAT_ERR_OOM, "cudaMalloc(%zu) failed", sizeof(double) * mw.size());
  }
  CK(cudaMemcpy(s->d_mw, mw.data(), sizeof(double) * mw.size(), cudaMemcpyHostToDevice), "node weights");
  return NAT_OK;
}

}  // namespace api
}  // namespace natgpu
