/*
 * natoracle.c -- CPU oracle for the semi-Lagrangian stream + collide path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C (FP64) restatement of
 * NATriuM's reference algorithm for the hot path.  It is used by the tests,
 * by __graft_entry__.smoke() and by bench.py's CPU-baseline leg and reference
 * arm: to check results and as the timed CPU baseline, never as the product
 * path that is measured or shipped.  The product path (natrium_gb300/,
 * libnatgpu.so) never links, loads or calls it.
 *
 * Parity status: the reference (deal.II 9.3.3 + Trilinos 13.0.1 + p4est +
 * Boost + MPI) cannot be compiled or run here, so there are no outputs of the
 * reference itself.  This restatement is pinned against the known answers and
 * invariants that the reference's own unit / integration tests state
 * (faceCrossedFirst lambdas and boundary points, A*1 = 1, BGK collision
 * invariants and fixed point, collideAll == collideSinglePoint, KBC mass ==
 * BGK mass, Taylor-Green kinetic-energy decay); see tests/test_oracle_*.py.
 *
 * What is restated (file:line are paths inside the reference's src/library/natrium):
 *   - stencils:  stencils/D2Q9.cpp:40-61, D3Q19.cpp:37-67, D3Q27.cpp:36-112,
 *                D2Q25H.cpp:37-84; c_s^2 = scaling^2/3; |e|_max = sqrt(2)*scaling
 *                (D2Q9.h:101-103, D3Q19.h:154-156, D3Q27.h:187-189, D2Q25H.h:149-151)
 *   - time step: utilities/CFDSolverUtilities.cpp:92-100
 *   - FE support points: advection/AdvectionTools.cpp:48-95 (Gauss-Lobatto,
 *                FE_Q for semi-Lagrangian, FE_DGQArbitraryNodes for DG)
 *   - departure-point trace + assembly: advection/SemiLagrangian.cpp:145-522
 *                (tracker queue, 50-crossing lifetime cap :252-271, periodic
 *                wrap :336-353, drop |w| < 1e-10 :483, add into block (alpha,alpha))
 *   - faceCrossedFirst with MappingCartesian: SemiLagrangian.cpp:525-699
 *                (1e-10 snapping :557-570 and :676-684)
 *   - shape values: advection/SemiLagrangianTools.cpp:15-64 (snap to [0,1])
 *   - stream: advection/SemiLagrangian.h:150-161 (f_old = f; A.vmult)
 *   - BGK collide (the time loop's path): collision_advanced/CollisionOperator.h:26-111,
 *                CollisionSchemes.h:28-41, Equilibria.h:33-83,
 *                AuxiliaryCollisionFunctions.h:45-68,151-268
 *   - legacy BGK single point / equilibrium: collision/BGK.cpp:24-45,
 *                collision/BGKStandard.cpp:23-41
 *   - BGK incompressible D2Q9: collision/BGKIncompressible.cpp:62-190
 *   - KBC D2Q9: collision/KBCStandard.cpp:88-497 (without the statistics file)
 *   - compressible two-population BGK on D2Q25H: CollisionOperator.h:113-224,
 *                CollisionSchemes.h:43-118 (relaxWithG), Equilibria.h:88-267
 *                (quartic equilibrium), AuxiliaryCollisionFunctions.h:289-307,
 *                420-566 (temperature, g^eq, Prandtl terms, Knudsen estimate,
 *                H3/H4), CompressibleCFDSolver.h:181-314, 739-899 (stream,
 *                gStream, collide, equilibrium initialisation)
 *   - KBC D3Q27: no reference implementation exists; the D2Q9 construction
 *                (trace kept in the shear part, product-form equilibrium of
 *                KBCStandard.cpp:26-63) is extended to D3Q27.  Parity unpinned.
 *
 * The Lagrange basis is evaluated in product form from the definition
 * L_j(x) = prod_{k != j} (x - x_k) / (x_j - x_k); Gauss-Lobatto points are the
 * end points plus the roots of P_p', found by Newton iteration on the
 * Legendre ODE.  Neither is taken from deal.II.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_D2Q9 0
#define ORC_D3Q19 1
#define ORC_D3Q27 2
#define ORC_D2Q25H 3

#define ORC_OK 0
#define ORC_ERR_ARG -1
#define ORC_ERR_DENSITY -2
#define ORC_ERR_OOM -3

/* ------------------------------------------------------------------------ */
/* stencils                                                                  */
/* ------------------------------------------------------------------------ */

/* Unit directions (unscaled) and weights.  Orderings follow the reference's
 * tables exactly (D3Q19 and D3Q27 orderings differ from each other). */
static const double D2Q9_E[9][3] = {{0, 0, 0},  {1, 0, 0},  {0, 1, 0},
                                    {-1, 0, 0}, {0, -1, 0}, {1, 1, 0},
                                    {-1, 1, 0}, {-1, -1, 0}, {1, -1, 0}};
static const double D3Q19_E[19][3] = {
    {0, 0, 0},  {1, 0, 0},  {0, 0, 1},  {-1, 0, 0}, {0, 0, -1},
    {0, -1, 0}, {0, 1, 0},  {1, 0, 1},  {-1, 0, 1}, {-1, 0, -1},
    {1, 0, -1}, {1, -1, 0}, {1, 1, 0},  {-1, 1, 0}, {-1, -1, 0},
    {0, -1, 1}, {0, 1, 1},  {0, 1, -1}, {0, -1, -1}};
static const double D3Q27_E[27][3] = {
    {0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0},
    {0, 0, 1},   {0, 0, -1},  {0, 1, 1},   {0, -1, -1}, {0, 1, -1},
    {0, -1, 1},  {1, 0, 1},   {-1, 0, -1}, {1, 0, -1},  {-1, 0, 1},
    {1, 1, 0},   {-1, -1, 0}, {1, -1, 0},  {-1, 1, 0},  {1, 1, 1},
    {-1, -1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1},  {-1, 1, -1},
    {1, -1, -1}, {-1, 1, 1}};

int orc_stencil(int id, double scaling, int* D, int* Q, double* e_scaled,
                double* w, double* cs2_scaled, double* max_speed) {
  int i, a;
  if (id == ORC_D2Q9) {
    static const double W[9] = {4. / 9.,  1. / 9.,  1. / 9.,  1. / 9., 1. / 9.,
                                1. / 36., 1. / 36., 1. / 36., 1. / 36.};
    *D = 2;
    *Q = 9;
    for (i = 0; i < 9; i++) {
      w[i] = W[i];
      for (a = 0; a < 3; a++) e_scaled[3 * i + a] = D2Q9_E[i][a] * scaling;
    }
  } else if (id == ORC_D3Q19) {
    *D = 3;
    *Q = 19;
    for (i = 0; i < 19; i++) {
      w[i] = (i == 0) ? 1. / 3. : (i <= 6 ? 1. / 18. : 1. / 36.);
      for (a = 0; a < 3; a++) e_scaled[3 * i + a] = D3Q19_E[i][a] * scaling;
    }
  } else if (id == ORC_D3Q27) {
    *D = 3;
    *Q = 27;
    for (i = 0; i < 27; i++) {
      w[i] = (i == 0) ? 8. / 27.
                      : (i <= 6 ? 2. / 27. : (i <= 18 ? 1. / 54. : 1. / 216.));
      for (a = 0; a < 3; a++) e_scaled[3 * i + a] = D3Q27_E[i][a] * scaling;
    }
  } else if (id == ORC_D2Q25H) {
    /* D2Q25H.cpp:37-84: two speeds c_m, c_n; weights are products of 1-D
     * weights w_0, w_m, w_n. */
    double r = (sqrt(5.) - sqrt(2.)) / sqrt(3.);
    double w0 = (-3 - 3 * r * r * r * r + 54 * r * r) / (75 * r * r);
    double wm = (9 * r * r * r * r - 6 - 27 * r * r) / (300 * r * r * (r * r - 1));
    double wn = (9 - 6 * r * r * r * r - 27 * r * r) / (300 * (1 - r * r));
    double cm = scaling * sqrt(5. - sqrt(10.)) / sqrt(3.);
    double cn = sqrt(5. + sqrt(10.)) * scaling / sqrt(3.);
    const double E[25][2] = {
        {0.0, 0.0}, {cm, 0.0}, {0.0, cm}, {-cm, 0.0}, {0.0, -cm},
        {cm, cm},   {-cm, cm}, {-cm, -cm}, {cm, -cm}, {cn, 0.0},
        {0.0, cn},  {-cn, 0.0}, {0.0, -cn}, {cn, cn}, {-cn, cn},
        {-cn, -cn}, {cn, -cn}, {cm, cn},  {cm, -cn}, {-cm, -cn},
        {-cm, cn},  {cn, cm},  {cn, -cm}, {-cn, -cm}, {-cn, cm}};
    const double Wt[25] = {w0 * w0, w0 * wm, w0 * wm, w0 * wm, w0 * wm,
                           wm * wm, wm * wm, wm * wm, wm * wm, w0 * wn,
                           w0 * wn, w0 * wn, w0 * wn, wn * wn, wn * wn,
                           wn * wn, wn * wn, wm * wn, wm * wn, wm * wn,
                           wm * wn, wm * wn, wm * wn, wm * wn, wm * wn};
    *D = 2;
    *Q = 25;
    for (i = 0; i < 25; i++) {
      w[i] = Wt[i];
      e_scaled[3 * i + 0] = E[i][0];
      e_scaled[3 * i + 1] = E[i][1];
      e_scaled[3 * i + 2] = 0.0;
    }
  } else {
    return ORC_ERR_ARG;
  }
  *cs2_scaled = scaling * scaling / 3.;
  *max_speed = scaling * sqrt(2.);
  return ORC_OK;
}

/* CFDSolverUtilities.cpp:92-100: dt = CFL * dx_min / (|e|_max * p^2) */
double orc_time_step(double dx_min, int p, double max_speed, double cfl) {
  return cfl * dx_min / (max_speed * p * p);
}

/* ------------------------------------------------------------------------ */
/* 1-D Gauss-Lobatto points and Lagrange basis                               */
/* ------------------------------------------------------------------------ */

/* Legendre P_n and P_n' at x by the three-term recurrence. */
static void legendre(int n, long double x, long double* P, long double* dP) {
  long double p0 = 1.0L, p1 = x, d0 = 0.0L, d1 = 1.0L;
  int k;
  if (n == 0) {
    *P = 1.0L;
    *dP = 0.0L;
    return;
  }
  for (k = 2; k <= n; k++) {
    long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
    long double d2 = d0 + (2 * k - 1) * p1;
    p0 = p1;
    p1 = p2;
    d0 = d1;
    d1 = d2;
  }
  *P = p1;
  *dP = d1;
}

/* p+1 Gauss-Lobatto points on [0,1] (QGaussLobatto(p+1) mapped to the unit
 * interval).  Interior points: roots of P_p', Newton on
 * (1-x^2) P'' = 2x P' - p(p+1) P. */
void orc_gl_points(int p, double* xi) {
  int j, it;
  xi[0] = 0.0;
  xi[p] = 1.0;
  for (j = 1; j < p; j++) {
    long double x = -cosl(3.14159265358979323846264338327950288L * j / p);
    for (it = 0; it < 100; it++) {
      long double P, dP;
      legendre(p, x, &P, &dP);
      long double d2P = (2 * x * dP - p * (p + 1) * P) / (1 - x * x);
      long double dx = dP / d2P;
      x -= dx;
      if (fabsl(dx) < 1e-22L) break;
    }
    xi[j] = (double)((x + 1.0L) / 2.0L);
  }
  /* symmetric by construction of the family; enforce it exactly */
  for (j = 1; j < p - j; j++) {
    double a = 0.5 * (xi[j] + (1.0 - xi[p - j]));
    xi[j] = a;
    xi[p - j] = 1.0 - a;
  }
  if (p % 2 == 0) xi[p / 2] = 0.5;
}

/* L_j(x) on the points xi[0..p], product form. */
double orc_lagrange(int p, const double* xi, int j, double x) {
  double v = 1.0;
  int k;
  for (k = 0; k <= p; k++) {
    if (k == j) continue;
    v *= (x - xi[k]) / (xi[j] - xi[k]);
  }
  return v;
}

/* ------------------------------------------------------------------------ */
/* Cartesian mesh, reference node numbering                                 */
/* ------------------------------------------------------------------------ */

/* Boundary kinds of the six box faces (x-, x+, y-, y+, z-, z+). */
#define ORC_BC_PERIODIC 0
#define ORC_BC_VELOCITY_BOUNCE_BACK 1 /* boundaries/VelocityNeqBounceBack */
#define ORC_BC_DO_NOTHING 2           /* boundaries/DoNothingBoundary */

typedef struct {
  int dim;
  int N[3];
  int p;
  int dg; /* 0: FE_Q (the reference's semi-Lagrangian element), 1: FE_DGQ */
  double L[3];
  int bc[6];       /* per face: ORC_BC_*; both faces of an axis periodic or neither */
  double uw[6][3]; /* wall velocity of a bounce-back face (scaled units) */
  /* MappingQ1 cells (NULL: the Cartesian box, MappingCartesian): the grid
   * vertices, x fastest, (N0+1)(N1+1)(N2+1) points of 3 doubles; a periodic
   * axis needs vertex N_a = vertex 0 + L_a e_a */
  const double* vtx;
} orc_mesh;

static int nodes_per_axis(const orc_mesh* m, int a) {
  if (a >= m->dim) return 1;
  return m->dg ? m->N[a] * (m->p + 1) : m->N[a] * m->p + 1;
}

int64_t orc_n_nodes(const orc_mesh* m) {
  return (int64_t)nodes_per_axis(m, 0) * nodes_per_axis(m, 1) *
         nodes_per_axis(m, 2);
}

/* Node layout (both topologies): lexicographic over the node lattice,
 * x fastest.  FE_Q lattice index i along an axis: cell i/p, local i%p (the
 * last node i = N p is local p of the last cell).  DG: cell i/(p+1), local
 * i%(p+1). */
static void axis_cell_local(const orc_mesh* m, int a, int i, int* c, int* l) {
  if (a >= m->dim) {
    *c = 0;
    *l = 0;
    return;
  }
  if (m->dg) {
    *c = i / (m->p + 1);
    *l = i % (m->p + 1);
  } else {
    if (i == m->N[a] * m->p) {
      *c = m->N[a] - 1;
      *l = m->p;
    } else {
      *c = i / m->p;
      *l = i % m->p;
    }
  }
}

/* global node index of local node (lx,ly,lz) of cell (cx,cy,cz) */
static int64_t cell_node_index(const orc_mesh* m, const int* c, const int* l) {
  int64_t idx = 0, stride = 1;
  int a;
  for (a = 0; a < m->dim; a++) {
    int i = m->dg ? c[a] * (m->p + 1) + l[a] : c[a] * m->p + l[a];
    idx += stride * i;
    stride *= nodes_per_axis(m, a);
  }
  return idx;
}

/* ---- MappingQ1 (multilinear map of a cell from its 2^D vertices) -------- */
static const double* grid_vertex(const orc_mesh* m, int i, int j, int k) {
  const int n0 = m->N[0] + 1, n1 = m->dim > 1 ? m->N[1] + 1 : 1;
  return m->vtx + 3 * (((int64_t)k * n1 + j) * n0 + i);
}

/* x = sum over corners of prod_a (b_a ? u_a : 1 - u_a) V_corner; also the
 * Jacobian J[r][a] = dx_r / du_a when J != NULL */
static void q1_map(const orc_mesh* m, const int* c, const double* u, double* x, double J[3][3]) {
  const int D = m->dim, nc = 1 << D;
  int k, a, r;
  for (r = 0; r < 3; r++) {
    x[r] = 0.0;
    if (J)
      for (a = 0; a < 3; a++) J[r][a] = 0.0;
  }
  for (k = 0; k < nc; k++) {
    int b[3] = {k & 1, (k >> 1) & 1, (k >> 2) & 1};
    double phi = 1.0, dphi[3];
    for (a = 0; a < D; a++) phi *= b[a] ? u[a] : 1.0 - u[a];
    for (a = 0; a < D; a++) {
      dphi[a] = b[a] ? 1.0 : -1.0;
      int q;
      for (q = 0; q < D; q++)
        if (q != a) dphi[a] *= b[q] ? u[q] : 1.0 - u[q];
    }
    const double* v = grid_vertex(m, c[0] + b[0], D > 1 ? c[1] + b[1] : 0, D > 2 ? c[2] + b[2] : 0);
    for (r = 0; r < D; r++) {
      x[r] += phi * v[r];
      if (J)
        for (a = 0; a < D; a++) J[r][a] += dphi[a] * v[r];
    }
  }
}

/* J du = r for D = 2 or 3 (Cramer's rule); -1 for a singular J */
static int q1_solve(int D, double J[3][3], const double* r, double* du) {
  if (D == 2) {
    const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    if (det == 0.0) return -1;
    du[0] = (J[1][1] * r[0] - J[0][1] * r[1]) / det;
    du[1] = (-J[1][0] * r[0] + J[0][0] * r[1]) / det;
    return 0;
  }
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  if (det == 0.0) return -1;
  int col, row, a;
  for (col = 0; col < 3; col++) {
    double M[3][3];
    for (row = 0; row < 3; row++)
      for (a = 0; a < 3; a++) M[row][a] = a == col ? r[row] : J[row][a];
    du[col] = (M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
               M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
               M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0])) / det;
  }
  return 0;
}

/* Inverse of the cell map (the reference calls
 * MappingQ1::transform_real_to_unit_cell): Newton's method from the cell
 * centre, each step halved (up to 12 times) until the residual decreases.
 * Converged when a step is below 1e-14 in unit coordinates; -1 when the
 * residual cannot be decreased before that (the reference's
 * ExcTransformationFailed), or after 100 steps. */
static int q1_inverse(const orc_mesh* m, const int* c, const double* x, double* u) {
  const int D = m->dim;
  int it, a;
  double y[3], J[3][3], r[3], res = 0.0;
  for (a = 0; a < 3; a++) u[a] = a < D ? 0.5 : 0.0;
  q1_map(m, c, u, y, J);
  for (a = 0; a < D; a++) {
    r[a] = y[a] - x[a];
    res += r[a] * r[a];
  }
  for (it = 0; it < 100; it++) {
    double du[3] = {0, 0, 0}, step = 1.0, stp = 0.0;
    int k, ok = 0;
    if (q1_solve(D, J, r, du)) return -1;
    for (a = 0; a < D; a++) stp += du[a] * du[a];
    for (k = 0; k <= 12; k++, step *= 0.5) {
      double un[3] = {u[0], u[1], u[2]}, yn[3], Jn[3][3], rn[3], rs = 0.0;
      for (a = 0; a < D; a++) un[a] = u[a] - step * du[a];
      q1_map(m, c, un, yn, Jn);
      for (a = 0; a < D; a++) {
        rn[a] = yn[a] - x[a];
        rs += rn[a] * rn[a];
      }
      if (rs < res || rs == 0.0) {
        for (a = 0; a < D; a++) {
          u[a] = un[a];
          r[a] = rn[a];
        }
        memcpy(J, Jn, sizeof(Jn));
        res = rs;
        ok = 1;
        break;
      }
    }
    if (!ok) return stp < 1e-24 ? 0 : -1; /* stuck at round-off */
    if (stp * step * step < 1e-28 || res == 0.0) return 0;
  }
  return -1;
}

void orc_node_coords(const orc_mesh* m, double* X) {
  double xi[16];
  int64_t n = orc_n_nodes(m), g;
  int nx = nodes_per_axis(m, 0), ny = nodes_per_axis(m, 1);
  orc_gl_points(m->p, xi);
  for (g = 0; g < n; g++) {
    int ii[3] = {(int)(g % nx), (int)((g / nx) % ny), (int)(g / ((int64_t)nx * ny))};
    int a;
    for (a = 0; a < 3; a++) {
      if (a >= m->dim) {
        X[3 * g + a] = 0.0;
        continue;
      }
      int c, l;
      double h = m->L[a] / m->N[a];
      axis_cell_local(m, a, ii[a], &c, &l);
      X[3 * g + a] = c * h + xi[l] * h;
    }
    if (m->vtx) {
      /* mapped node: the cell's map at the Gauss-Lobatto unit point */
      int c[3] = {0, 0, 0}, l[3] = {0, 0, 0};
      double u[3] = {0, 0, 0}, x[3];
      for (a = 0; a < m->dim; a++) {
        axis_cell_local(m, a, ii[a], &c[a], &l[a]);
        u[a] = xi[l[a]];
      }
      q1_map(m, c, u, x, NULL);
      for (a = 0; a < 3; a++) X[3 * g + a] = a < m->dim ? x[a] : 0.0;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* faceCrossedFirst for an axis-aligned cell (MappingCartesian)              */
/* ------------------------------------------------------------------------ */

/* SemiLagrangian.cpp:525-699.  Returns the face id (0:x-,1:x+,2:y-,3:y+,
 * 4:z-,5:z+) crossed first on the way from p_in (inside the cell) to p_out,
 * or -1 if p_out lies in the closed cell.  Writes the boundary point and
 * lambda when a face is crossed. */
int orc_face_crossed_first(int dim, const double* lo, const double* h,
                           const double* p_in, const double* p_out,
                           double* p_boundary, double* lambda) {
  double pi[3], po[3], hh[3];
  int a, face = -1;
  *lambda = 100;
  for (a = 0; a < dim; a++) {
    pi[a] = (p_in[a] - lo[a]) / h[a];
    po[a] = (p_out[a] - lo[a]) / h[a];
    if (fabs(pi[a]) < 1e-10) pi[a] = 0;
    if (fabs(pi[a] - 1) < 1e-10) pi[a] = 1;
    if (fabs(po[a]) < 1e-10) po[a] = 0;
    if (fabs(po[a] - 1) < 1e-10) po[a] = 1;
  }
  for (a = 0; a < dim; a++) {
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
    /* the reference takes the x face unconditionally and later faces only
     * when strictly smaller */
    if (a == 0 || lam < *lambda) {
      *lambda = lam;
      face = f;
    }
  }
  if (face == -1) return -1;
  for (a = 0; a < dim; a++) {
    hh[a] = pi[a] + (po[a] - pi[a]) * (*lambda);
    if (fabs(hh[a]) < 1e-10) hh[a] = 0;
    if (fabs(hh[a] - 1) < 1e-10) hh[a] = 1;
    p_boundary[a] = lo[a] + hh[a] * h[a];
  }
  return face;
}

/* faceCrossedFirst with the mapping (SemiLagrangian.cpp:525-699): both points
 * to unit coordinates of the cell, the face with the smallest lambda in unit
 * space, the crossing point mapped back to real space. */
/* faceCrossedFirstWithoutMapping (SemiLagrangian.cpp:702-757), taken when
 * an inverse map fails: every face is treated as the plane through its first
 * vertex with the normal of its first edges (SemiLagrangianTools.cpp:151-168);
 * the smallest non-negative lambda below 1 wins, faces in order 0..2D-1.
 * Face vertices in the cell numbering bx + 2 by + 4 bz. */
static int face_crossed_first_planar(const orc_mesh* m, const int* c, const double* p_in, const double* p_out,
                                     double* p_boundary) {
  static const int FV2[4][2] = {{0, 2}, {1, 3}, {0, 1}, {2, 3}};
  static const int FV3[6][3] = {{0, 2, 4}, {1, 3, 5}, {0, 4, 1}, {2, 6, 3}, {0, 1, 2}, {4, 5, 6}};
  const int D = m->dim;
  double lambda_min = 1.0;
  int i, a, index_min = 0;
  for (i = 0; i < 2 * D; i++) {
    const double* v[3];
    int k;
    for (k = 0; k < D; k++) {
      const int cv = D == 2 ? FV2[i][k] : FV3[i][k];
      v[k] = grid_vertex(m, c[0] + (cv & 1), c[1] + ((cv >> 1) & 1), D > 2 ? c[2] + ((cv >> 2) & 1) : 0);
    }
    double n[3];
    if (D == 2) {
      n[0] = v[1][1] - v[0][1]; /* cross_product_2d(d) = (d_y, -d_x) */
      n[1] = -(v[1][0] - v[0][0]);
    } else {
      double d1[3], d2[3];
      for (a = 0; a < 3; a++) {
        d1[a] = v[1][a] - v[0][a];
        d2[a] = v[2][a] - v[0][a];
      }
      n[0] = d1[1] * d2[2] - d1[2] * d2[1];
      n[1] = d1[2] * d2[0] - d1[0] * d2[2];
      n[2] = d1[0] * d2[1] - d1[1] * d2[0];
    }
    double num = 0.0, den = 0.0;
    for (a = 0; a < D; a++) {
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
  for (a = 0; a < D; a++) p_boundary[a] = p_in[a] + (p_out[a] - p_in[a]) * lambda_min;
  return index_min;
}

static int face_crossed_first_q1(const orc_mesh* m, const int* c, const double* p_in, const double* p_out,
                                 double* p_boundary) {
  const int D = m->dim;
  double pi[3] = {0, 0, 0}, po[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, one[3] = {1, 1, 1}, hu[3] = {0, 0, 0}, lam;
  if (q1_inverse(m, c, p_in, pi) || q1_inverse(m, c, p_out, po))
    return face_crossed_first_planar(m, c, p_in, p_out, p_boundary); /* SemiLagrangian.cpp:283-287 */
  const int face = orc_face_crossed_first(D, lo, one, pi, po, hu, &lam);
  if (face >= 0) q1_map(m, c, hu, p_boundary, NULL);
  return face;
}

/* ------------------------------------------------------------------------ */
/* semi-Lagrangian assembly (tracker algorithm) -> per-direction CSR         */
/* ------------------------------------------------------------------------ */

typedef struct {
  int Q, D;
  int64_t n;
  int64_t* rowptr[32]; /* per streamed direction alpha = 1..Q-1 */
  int32_t* col[32];    /* source node */
  int32_t* sdir[32];   /* source direction (alpha itself unless a wall reversed the path) */
  double* val[32];
  double* bconst[32];  /* per row: wall-velocity term of bounce-back hits (NULL: none) */
  int64_t nnz[32];
  int n_lifetime_hits;
  int n_wall_hits;
} orc_sl;

/* LagrangianPathTracker: destination (dest, alpha), the direction whose
 * population is currently followed (cdir), and the do-nothing flag. */
typedef struct {
  int64_t dest;
  int alpha;
  int cdir;
  int hit_dn;
  int cell[3];
  double cur[3], dep[3];
  int life;
} tracker;

/* dynamic COO buffer per direction, converted to CSR at the end */
typedef struct {
  int64_t* row;
  int32_t* col;
  int32_t* sdir;
  double* val;
  int64_t size, cap;
} coo;

static int coo_push(coo* c, int64_t r, int32_t col, int32_t sdir, double v) {
  if (c->size == c->cap) {
    int64_t nc = c->cap ? 2 * c->cap : 1024;
    int64_t* nr = (int64_t*)realloc(c->row, nc * sizeof(int64_t));
    if (!nr) return ORC_ERR_OOM;
    c->row = nr;
    int32_t* ncol = (int32_t*)realloc(c->col, nc * sizeof(int32_t));
    if (!ncol) return ORC_ERR_OOM;
    c->col = ncol;
    int32_t* nsd = (int32_t*)realloc(c->sdir, nc * sizeof(int32_t));
    if (!nsd) return ORC_ERR_OOM;
    c->sdir = nsd;
    double* nv = (double*)realloc(c->val, nc * sizeof(double));
    if (!nv) return ORC_ERR_OOM;
    c->val = nv;
    c->cap = nc;
  }
  c->row[c->size] = r;
  c->col[c->size] = col;
  c->sdir[c->size] = sdir;
  c->val[c->size] = v;
  c->size++;
  return ORC_OK;
}

void orc_sl_free(orc_sl* s) {
  int a;
  if (!s) return;
  for (a = 0; a < 32; a++) {
    free(s->rowptr[a]);
    free(s->col[a]);
    free(s->sdir[a]);
    free(s->val[a]);
    free(s->bconst[a]);
  }
  free(s);
}

/* Periodic translation per axis: L_a e_a on the box; with mapped cells the
 * offset between the two faces' vertices, which must be the same vector for
 * all of them on a periodic axis (PeriodicBoundary.cpp:184-270, the offset of
 * face 1 to face 0).  -1 when a periodic axis has no common offset. */
static int periodic_offsets(const orc_mesh* m, double pv[3][3]) {
  const int D = m->dim;
  int a, b;
  for (a = 0; a < D; a++) {
    for (b = 0; b < 3; b++) pv[a][b] = a == b ? m->L[a] : 0.0;
    if (!m->vtx) continue;
    /* the vertex lattice of face a-, walked over the other axes */
    const int nb = a == 0 ? 1 : 0, nc = a == 2 ? 1 : 2;
    const int mb = m->N[nb] + 1, mc = D > 2 ? m->N[nc] + 1 : 1;
    int ib, ic;
    for (ic = 0; ic < mc; ic++)
      for (ib = 0; ib < mb; ib++) {
        int lo_i[3] = {0, 0, 0}, hi_i[3] = {0, 0, 0};
        lo_i[nb] = hi_i[nb] = ib;
        if (D > 2) lo_i[nc] = hi_i[nc] = ic;
        hi_i[a] = m->N[a];
        const double* v0 = grid_vertex(m, lo_i[0], lo_i[1], lo_i[2]);
        const double* v1 = grid_vertex(m, hi_i[0], hi_i[1], hi_i[2]);
        for (b = 0; b < D; b++) {
          const double d = v1[b] - v0[b];
          if (ib == 0 && ic == 0)
            pv[a][b] = d;
          else if (m->bc[2 * a] == ORC_BC_PERIODIC && fabs(d - pv[a][b]) > 1e-12 * (fabs(d) + 1.0))
            return -1;
        }
      }
  }
  return 0;
}

/* Assemble the streaming operator for all streamed directions.
 * Restates SemiLagrangian::fillSparseObject (SemiLagrangian.cpp:145-522) for
 * an axis-aligned periodic box: every node is traced once (the first cell in
 * cell order that holds it), its departure points x - dt e_alpha are followed
 * across faces (periodic faces shift the points by the box length), and the
 * FE shape values of the cell that holds the departure point become the row.
 * Non-periodic faces (SemiLagrangian.cpp:354-399):
 *   VelocityNeqBounceBack: the followed direction is reversed, the path
 *     continues from the wall point for the remaining length, and the hit adds
 *     2 w_alpha rho_w (e_alpha . u_w) / c_s^2 (rho_w = 1) to the destination
 *     (boundaries/VelocityNeqBounceBack.cpp:137-194);
 *   DoNothingBoundary: the path restarts at the destination and runs the
 *     other way (x + dt e_alpha); the population stays alpha. */
orc_sl* orc_sl_assemble(const orc_mesh* m, int stencil, double scaling,
                        double dt) {
  int D, Q, a, alpha;
  double e[3 * 32], w[32], cs2, vmax, xi[16];
  int p = m->p, dpc = 1;
  int64_t n = orc_n_nodes(m);
  char* tracked;
  orc_sl* s;
  coo buf[32];
  int cells_total = 1;
  int c_iter;
  double* vals = NULL;
  double h[3] = {1, 1, 1};
  double pv[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  int opp[32];

  if (orc_stencil(stencil, scaling, &D, &Q, e, w, &cs2, &vmax) != ORC_OK)
    return NULL;
  if (D != m->dim || Q > 32 || p < 1 || p > 15) return NULL;
  for (a = 0; a < D; a++) {
    dpc *= (p + 1);
    cells_total *= m->N[a];
    h[a] = m->L[a] / m->N[a];
  }
  orc_gl_points(p, xi);
  if (periodic_offsets(m, pv)) return NULL;
  for (alpha = 0; alpha < Q; alpha++) {
    int j, k;
    opp[alpha] = 0;
    for (j = 0; j < Q; j++) {
      int same = 1;
      for (k = 0; k < 3; k++)
        if (e[3 * j + k] != -e[3 * alpha + k]) same = 0;
      if (same) opp[alpha] = j;
    }
  }
  s = (orc_sl*)calloc(1, sizeof(orc_sl));
  if (!s) return NULL;
  s->Q = Q;
  s->D = D;
  s->n = n;
  memset(buf, 0, sizeof(buf));
  tracked = (char*)calloc((size_t)n, 1);
  if (!tracked) {
    free(s);
    return NULL;
  }

  vals = (double*)malloc(sizeof(double) * dpc);
  if (!vals) goto fail;

  for (c_iter = 0; c_iter < cells_total; c_iter++) {
    int cc[3] = {0, 0, 0};
    int tmp = c_iter, li;
    for (a = 0; a < D; a++) {
      cc[a] = tmp % m->N[a];
      tmp /= m->N[a];
    }
    /* every not-yet-seen node of the cell gets one tracker per direction;
     * each tracker is followed until its departure point is found (the
     * reference keeps them in a queue; the order does not change the rows) */
    for (li = 0; li < dpc; li++) {
      int l[3] = {0, 0, 0}, t = li;
      for (a = 0; a < D; a++) {
        l[a] = t % (p + 1);
        t /= (p + 1);
      }
      int64_t g = cell_node_index(m, cc, l);
      if (tracked[g]) continue;
      tracked[g] = 1;
      double x[3] = {0, 0, 0};
      for (a = 0; a < D; a++) x[a] = cc[a] * h[a] + xi[l[a]] * h[a];
      if (m->vtx) {
        double ul[3] = {0, 0, 0};
        for (a = 0; a < D; a++) ul[a] = xi[l[a]];
        q1_map(m, cc, ul, x, NULL);
      }
      for (alpha = 1; alpha < Q; alpha++) {
        tracker el;
        el.dest = g;
        el.alpha = alpha;
        el.cdir = alpha;
        el.hit_dn = 0;
        el.life = 0;
        for (a = 0; a < 3; a++) {
          el.cell[a] = cc[a];
          el.cur[a] = x[a];
          el.dep[a] = (a < D) ? x[a] + e[3 * alpha + a] * (-dt) : 0.0;
        }
        for (;;) {
          el.life++;
          if (el.life > 50) {
            /* SemiLagrangian.cpp:252-271: identity entry */
            if (coo_push(&buf[alpha], g, (int32_t)g, alpha, 1.0)) goto fail;
            s->n_lifetime_hits++;
            break;
          }
          double lo[3], pb[3], lam, ud[3] = {0, 0, 0};
          for (a = 0; a < D; a++) lo[a] = el.cell[a] * h[a];
          int face = m->vtx ? face_crossed_first_q1(m, el.cell, el.cur, el.dep, pb)
                            : orc_face_crossed_first(D, lo, h, el.cur, el.dep, pb, &lam);
          if (face == -1) {
            if (el.hit_dn) el.cdir = opp[el.cdir]; /* SemiLagrangian.cpp:312-316 */
            /* found: shape values of the cell at the departure point
             * (SemiLagrangianTools.cpp:15-64, snap to [0,1] at 1e-10) */
            double l1[3][16];
            int k, lj;
            if (m->vtx && q1_inverse(m, el.cell, el.dep, ud)) goto fail;
            for (a = 0; a < D; a++) {
              double uu = m->vtx ? ud[a] : (el.dep[a] - lo[a]) / h[a];
              if (fabs(uu) < 1e-10) uu = 0;
              if (fabs(uu - 1) < 1e-10) uu = 1;
              for (k = 0; k <= p; k++) l1[a][k] = orc_lagrange(p, xi, k, uu);
            }
            for (lj = 0; lj < dpc; lj++) {
              int ll[3] = {0, 0, 0}, tt = lj;
              double v = 1.0;
              for (a = 0; a < D; a++) {
                ll[a] = tt % (p + 1);
                tt /= (p + 1);
                v *= l1[a][ll[a]];
              }
              vals[lj] = v;
            }
            for (lj = 0; lj < dpc; lj++) {
              int ll[3] = {0, 0, 0}, tt = lj;
              if (fabs(vals[lj]) < 1e-10) continue; /* SemiLagrangian.cpp:483 */
              for (a = 0; a < D; a++) {
                ll[a] = tt % (p + 1);
                tt /= (p + 1);
              }
              int64_t src = cell_node_index(m, el.cell, ll);
              if (coo_push(&buf[alpha], g, (int32_t)src, el.cdir, vals[lj])) goto fail;
            }
            break;
          }
          int ax = face / 2;
          int upper = face % 2;
          int at_boundary =
              upper ? (el.cell[ax] == m->N[ax] - 1) : (el.cell[ax] == 0);
          if (at_boundary && m->bc[face] == ORC_BC_VELOCITY_BOUNCE_BACK) {
            /* SemiLagrangian.cpp:357-386: reverse the followed direction,
             * continue from the wall point for the remaining length */
            double dist = 0.0, ve = 0.0, exu = 0.0;
            el.cdir = opp[el.cdir];
            for (a = 0; a < D; a++) {
              dist += (el.dep[a] - pb[a]) * (el.dep[a] - pb[a]);
              ve += e[3 * el.cdir + a] * e[3 * el.cdir + a];
            }
            dist = sqrt(dist);
            ve = sqrt(ve);
            for (a = 0; a < D; a++) {
              el.cur[a] = pb[a];
              el.dep[a] = el.cur[a] - e[3 * el.cdir + a] * dist / ve;
            }
            /* VelocityNeqBounceBack.cpp:168-192, rho = 1, scaled e and c_s^2 */
            for (a = 0; a < D; a++) exu += m->uw[face][a] * e[3 * alpha + a];
            if (!s->bconst[alpha]) {
              s->bconst[alpha] = (double*)calloc((size_t)n, sizeof(double));
              if (!s->bconst[alpha]) goto fail;
            }
            s->bconst[alpha][g] += 2 * w[alpha] * 1.0 * exu / cs2;
            s->n_wall_hits++;
            continue;
          }
          if (at_boundary && m->bc[face] == ORC_BC_DO_NOTHING) {
            /* SemiLagrangian.cpp:388-399: restart at the destination and
             * follow the opposite direction */
            for (a = 0; a < D; a++) {
              el.cur[a] = el.dep[a] + dt * e[3 * el.cdir + a];
              el.dep[a] = el.cur[a] + dt * e[3 * el.cdir + a];
            }
            el.cdir = opp[el.cdir];
            el.hit_dn = 1;
            s->n_wall_hits++;
            continue;
          }
          for (a = 0; a < D; a++) el.cur[a] = pb[a];
          if (at_boundary) {
            /* periodic face (SemiLagrangian.cpp:336-353): translate the
             * boundary point and the departure point by the box length */
            for (a = 0; a < D; a++) {
              const double shift = upper ? -pv[ax][a] : pv[ax][a];
              el.cur[a] += shift;
              el.dep[a] += shift;
            }
            el.cell[ax] = upper ? 0 : m->N[ax] - 1;
          } else {
            el.cell[ax] += upper ? 1 : -1;
          }
        }
      }
    }
  }

  /* COO -> CSR per direction, rows in order, entries of a row in insertion
   * order; duplicate (row, col) pairs are summed like the matrix's add(). */
  for (alpha = 1; alpha < Q; alpha++) {
    coo* c = &buf[alpha];
    int64_t* cnt = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    int64_t k;
    if (!cnt) goto fail;
    for (k = 0; k < c->size; k++) cnt[c->row[k] + 1]++;
    for (k = 0; k < n; k++) cnt[k + 1] += cnt[k];
    s->rowptr[alpha] = cnt;
    s->col[alpha] = (int32_t*)malloc(sizeof(int32_t) * (c->size + 1));
    s->sdir[alpha] = (int32_t*)malloc(sizeof(int32_t) * (c->size + 1));
    s->val[alpha] = (double*)malloc(sizeof(double) * (c->size + 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (n + 1));
    if (!s->col[alpha] || !s->sdir[alpha] || !s->val[alpha] || !fill) {
      free(fill);
      goto fail;
    }
    memcpy(fill, cnt, sizeof(int64_t) * (n + 1));
    for (k = 0; k < c->size; k++) {
      int64_t r = c->row[k];
      int64_t pos = fill[r]++;
      s->col[alpha][pos] = c->col[k];
      s->sdir[alpha][pos] = c->sdir[k];
      s->val[alpha][pos] = c->val[k];
    }
    free(fill);
    s->nnz[alpha] = c->size;
    free(c->row);
    free(c->col);
    free(c->sdir);
    free(c->val);
    memset(c, 0, sizeof(coo));
  }
  free(vals);
  free(tracked);
  return s;
fail:
  for (a = 0; a < 32; a++) {
    free(buf[a].row);
    free(buf[a].col);
    free(buf[a].sdir);
    free(buf[a].val);
  }
  free(vals);
  free(tracked);
  orc_sl_free(s);
  return NULL;
}

int64_t orc_sl_nnz(const orc_sl* s, int alpha) {
  if (!s || alpha < 1 || alpha >= s->Q) return -1;
  return s->nnz[alpha];
}

int orc_sl_lifetime_hits(const orc_sl* s) { return s ? s->n_lifetime_hits : -1; }

int orc_sl_csr(const orc_sl* s, int alpha, int64_t* rowptr, int32_t* col,
               double* val) {
  if (!s || alpha < 1 || alpha >= s->Q) return ORC_ERR_ARG;
  memcpy(rowptr, s->rowptr[alpha], sizeof(int64_t) * (s->n + 1));
  memcpy(col, s->col[alpha], sizeof(int32_t) * s->nnz[alpha]);
  memcpy(val, s->val[alpha], sizeof(double) * s->nnz[alpha]);
  return ORC_OK;
}

/* SemiLagrangian::stream (SemiLagrangian.h:150-161): f_old = f, then
 * fStream <- A * f_old.fStream (block diagonal for periodic boxes); f_0 is
 * not streamed.  f_old / f_new: Q blocks of n doubles. */
static int sl_stream(const orc_sl* s, const double* f_old, double* f_new, int nthreads, int wall_terms);

int orc_sl_stream(const orc_sl* s, const double* f_old, double* f_new,
                  int nthreads) {
  return sl_stream(s, f_old, f_new, nthreads, 1);
}

/* The second population of the compressible model goes through the same
 * matrix (CompressibleCFDSolver::gStream, CompressibleCFDSolver.h:279-314)
 * without the wall-velocity terms: SemiLagrangianBoundaryHandler::apply only
 * changes f (SemiLagrangianBoundaryHandler.cpp:27-32, VelocityNeqBounceBack.cpp:190-193). */
int orc_sl_stream_g(const orc_sl* s, const double* g_old, double* g_new, int nthreads) {
  return sl_stream(s, g_old, g_new, nthreads, 0);
}

static int sl_stream(const orc_sl* s, const double* f_old, double* f_new, int nthreads, int wall_terms) {
  int alpha;
  int64_t n = s->n;
  (void)nthreads;
  memcpy(f_new, f_old, sizeof(double) * n); /* f_0 */
  for (alpha = 1; alpha < s->Q; alpha++) {
    const int64_t* rp = s->rowptr[alpha];
    const int32_t* cl = s->col[alpha];
    const int32_t* sd = s->sdir[alpha];
    const double* vl = s->val[alpha];
    const double* bc = wall_terms ? s->bconst[alpha] : NULL;
    double* y = f_new + (int64_t)alpha * n;
    int64_t r;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (r = 0; r < n; r++) {
      double acc = 0.0;
      int64_t k;
      for (k = rp[r]; k < rp[r + 1]; k++) acc += vl[k] * f_old[(int64_t)sd[k] * n + cl[k]];
      /* SemiLagrangianBoundaryHandler::apply after the vmult: wall terms */
      y[r] = bc ? acc + bc[r] : acc;
    }
  }
  return ORC_OK;
}

/* Source directions of the entries of direction alpha (CSR order). */
int orc_sl_csr_dirs(const orc_sl* s, int alpha, int32_t* sdir) {
  if (!s || alpha < 1 || alpha >= s->Q) return ORC_ERR_ARG;
  memcpy(sdir, s->sdir[alpha], sizeof(int32_t) * s->nnz[alpha]);
  return ORC_OK;
}

/* Wall-velocity terms of direction alpha (n values; zeros when none). */
int orc_sl_bconst(const orc_sl* s, int alpha, double* b) {
  if (!s || alpha < 1 || alpha >= s->Q) return ORC_ERR_ARG;
  if (s->bconst[alpha])
    memcpy(b, s->bconst[alpha], sizeof(double) * s->n);
  else
    memset(b, 0, sizeof(double) * s->n);
  return ORC_OK;
}

int orc_sl_wall_hits(const orc_sl* s) { return s ? s->n_wall_hits : -1; }

/* ------------------------------------------------------------------------ */
/* collisions                                                                */
/* ------------------------------------------------------------------------ */

/* collision_advanced: CollisionOperator<D,Q,BGKEquilibrium,BGKCollision>
 * ::collideAll (CollisionOperator.h:26-111).  tau = nu/(dt cs2_scaled) + 1/2
 * (AuxiliaryCollisionFunctions.h:63-68,177).  u arrays hold the scaled
 * velocity (u_unscaled * scaling).  Returns ORC_ERR_DENSITY if any density
 * is below 1e-10 (AuxiliaryCollisionFunctions.h:45-59). */
/* Advanced BGK (CollisionOperator.h:26-111 with BGKCollision::relax and
 * BGKEquilibrium).  With a constant body force (scheme 1 SHIFTING_VELOCITY,
 * 2 EXACT_DIFFERENCE; force in scaled units, dt the time step), as
 * CollisionOperator.h:76-90 applies it when the problem has an external
 * force (AuxiliaryCollisionFunctions.h:332-414):
 *   u_raw += dt F / (2 rho)                     (SHIFTING: before relax;
 *                                                EXACT: after it)
 *   SHIFTING: velocity += tau dt F / (rho scaling) before the equilibrium;
 *   EXACT: after relax, velocity += dt F / (rho scaling) and
 *          f += feq(shifted velocity) - feq.
 * The force is left out with a prescribed velocity (in_init). */
static void advanced_bgk_feq(int stencil, int D, int Q, const double e[32][3], const double* w, double cs2, double dens,
                    const double* vel, double* feq) {
  int pq, j;
  if (stencil == ORC_D2Q9) {
    /* Equilibria.h:33-63 */
    double prefactor = 1. / cs2, sp, usq, mixed, wt;
    sp = vel[0] * vel[0] + vel[1] * vel[1];
    usq = -sp / (2 * cs2);
    wt = 4. / 9. * dens;
    feq[0] = wt * (1 + usq);
    wt = 1. / 9. * dens;
    mixed = prefactor * (vel[0]);
    feq[1] = wt * (1 + mixed * (1 + 0.5 * mixed) + usq);
    feq[3] = wt * (1 - mixed * (1 - 0.5 * mixed) + usq);
    mixed = prefactor * (vel[1]);
    feq[2] = wt * (1 + mixed * (1 + 0.5 * mixed) + usq);
    feq[4] = wt * (1 - mixed * (1 - 0.5 * mixed) + usq);
    wt = 1. / 36. * dens;
    mixed = prefactor * (vel[0] + vel[1]);
    feq[5] = wt * (1 + mixed * (1 + 0.5 * mixed) + usq);
    feq[7] = wt * (1 - mixed * (1 - 0.5 * mixed) + usq);
    mixed = prefactor * (-vel[0] + vel[1]);
    feq[6] = wt * (1 + mixed * (1 + 0.5 * mixed) + usq);
    feq[8] = wt * (1 - mixed * (1 - 0.5 * mixed) + usq);
  } else {
    /* Equilibria.h:66-83 */
    double uu = 0.0;
    for (j = 0; j < D; j++) uu += -(vel[j] * vel[j]) / (2.0 * cs2);
    for (pq = 0; pq < Q; pq++) {
      double ue = 0.0;
      for (j = 0; j < D; j++) ue += (vel[j] * e[pq][j]) / cs2;
      feq[pq] = w[pq] * dens * (1 + ue * (1 + 0.5 * (ue)) + uu);
    }
  }
}

static int collide_bgk_legacy_guo(int stencil, double scaling, double tau, double dt, int64_t n, double* f,
                                  double* rho, double* u, int in_init, const double* force);

int orc_collide_bgk_force(int stencil, double scaling, double tau, double dt, int64_t n, double* f, double* rho,
                          double* u, int in_init, int scheme, const double* force, int nthreads) {
  int D, Q, bad = 0;
  double es[3 * 32], w[32], cs2s, vmax;
  double e[32][3];
  int64_t ii;
  if (orc_stencil(stencil, scaling, &D, &Q, es, w, &cs2s, &vmax) != ORC_OK)
    return ORC_ERR_ARG;
  {
    int i, a;
    for (i = 0; i < Q; i++)
      for (a = 0; a < 3; a++) e[i][a] = es[3 * i + a] / scaling;
  }
  const double cs2 = cs2s / (scaling * scaling);
  if (scheme == 3) return collide_bgk_legacy_guo(stencil, scaling, tau, dt, n, f, rho, u, in_init, force);
  (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (ii = 0; ii < n; ii++) {
    double fl[32], feq[32], vel[3] = {0, 0, 0}, dens = 0.0;
    int pq, j;
    for (pq = 0; pq < Q; pq++) fl[pq] = f[(int64_t)pq * n + ii];
    for (pq = 0; pq < Q; pq++) dens += fl[pq];
    if (dens < 1e-10 || dens != dens) bad = 1;
    rho[ii] = dens;
    if (stencil == ORC_D2Q9) {
      /* AuxiliaryCollisionFunctions.h:258-268 */
      vel[0] = 1.0 / dens * (fl[1] + fl[5] + fl[8] - fl[3] - fl[6] - fl[7]);
      vel[1] = 1.0 / dens * (fl[2] + fl[5] + fl[6] - fl[4] - fl[7] - fl[8]);
    } else {
      for (j = 0; j < D; j++) {
        vel[j] = 0.0;
        for (pq = 0; pq < Q; pq++) vel[j] += e[pq][j] * fl[pq];
        vel[j] = vel[j] * 1.0 / dens;
      }
    }
    const int forced = scheme != 0 && !in_init;
    if (!in_init) {
      for (j = 0; j < D; j++) u[(int64_t)j * n + ii] = vel[j] * scaling;
      if (forced && scheme == 1) {
        /* applyMacroscopicForces, applyForces */
        for (j = 0; j < D; j++) u[(int64_t)j * n + ii] += 0.5 * dt * force[j] / dens;
        for (j = 0; j < D; j++) vel[j] += tau * dt * force[j] / dens / scaling;
      }
    } else {
      for (j = 0; j < D; j++) vel[j] = u[(int64_t)j * n + ii] / scaling;
    }
    advanced_bgk_feq(stencil, D, Q, e, w, cs2, dens, vel, feq);
    /* CollisionSchemes.h:38-40 */
    for (pq = 0; pq < Q; pq++) fl[pq] -= 1. / tau * (fl[pq] - feq[pq]);
    if (forced && scheme == 2) {
      /* postCollisionApplyForces (EXACT_DIFFERENCE) */
      double shifted[32];
      for (j = 0; j < D; j++) {
        vel[j] += dt * force[j] / dens / scaling;
        u[(int64_t)j * n + ii] += 0.5 * dt * force[j] / dens;
      }
      advanced_bgk_feq(stencil, D, Q, e, w, cs2, dens, vel, shifted);
      for (pq = 0; pq < Q; pq++) fl[pq] += shifted[pq] - feq[pq];
    }
    for (pq = 0; pq < Q; pq++) f[(int64_t)pq * n + ii] = fl[pq];
  }
  return bad ? ORC_ERR_DENSITY : ORC_OK;
}

/* The legacy BGKStandard collision with the GUO forcing scheme, in the
 * reference's scaled variables: collideAllD2Q9 (collision/BGKStandard.cpp:
 * 64-239; velocity :128-133, equilibrium :142-175, relaxation :177-186,
 * source :222-225) with applyGuoForcingD2Q9 (collision/
 * ExternalForceFunctions.h:119-200), and collideAllD3Q19 (BGKStandard.cpp:
 * 241-477; velocity :374-380).  In collideAllD3Q19 the relaxed values are
 * written to the global vectors (:441-459) and the source term then goes to
 * the local copy f_i, which is not stored again (:466-473): only the shifted
 * equilibrium acts.  Restated as written.  force: scaled units. */
static int collide_bgk_legacy_guo(int stencil, double scaling, double tau, double dt, int64_t n, double* f,
                                  double* rho, double* u, int in_init, const double* force) {
  int D, Q, bad = 0;
  double es[3 * 32], w[32], cs2, vmax;
  int64_t ii;
  if (orc_stencil(stencil, scaling, &D, &Q, es, w, &cs2, &vmax) != ORC_OK) return ORC_ERR_ARG;
  if (stencil != ORC_D2Q9 && stencil != ORC_D3Q19) return ORC_ERR_ARG;
  const double prefactor = scaling / cs2;
  const double relax_factor = -1.0 / tau; /* BGK.cpp:13-16 with the legacy tau - 1/2 */
  const double omega = -relax_factor;
  for (ii = 0; ii < n; ii++) {
    double fl[32], feq[32], vel[3] = {0, 0, 0}, dens = 0.0;
    int i, a;
    for (i = 0; i < Q; i++) fl[i] = f[(int64_t)i * n + ii];
    for (i = 0; i < Q; i++) dens += fl[i];
    rho[ii] = dens;
    if (dens < 1e-10 || dens != dens) {
      bad = 1;
      continue;
    }
    if (!in_init) {
      for (a = 0; a < D; a++) {
        double m = 0.0;
        for (i = 0; i < Q; i++) m += fl[i] * (es[3 * i + a] / scaling);
        vel[a] = scaling / dens * m;
      }
      for (a = 0; a < D; a++) {
        vel[a] += 0.5 * dt * force[a] / dens;
        u[(int64_t)a * n + ii] = vel[a];
      }
    } else {
      for (a = 0; a < D; a++) vel[a] = u[(int64_t)a * n + ii];
    }
    double sp = 0.0;
    for (a = 0; a < D; a++) sp += vel[a] * vel[a];
    const double usq = -sp / (2 * cs2);
    for (i = 0; i < Q; i++) {
      double eu = 0.0;
      for (a = 0; a < D; a++) eu += (es[3 * i + a] / scaling) * vel[a];
      const double mixed = prefactor * eu;
      feq[i] = w[i] * dens * (1 + mixed * (1 + 0.5 * mixed) + usq);
    }
    for (i = 0; i < Q; i++) fl[i] += relax_factor * (fl[i] - feq[i]);
    if (stencil == ORC_D2Q9 && !in_init) {
      double ug_fg = 0.0;
      for (a = 0; a < D; a++) ug_fg += vel[a] * force[a];
      const double one_min_omega_half = 1 - 0.5 * omega;
      for (i = 0; i < Q; i++) {
        double eia_ua = 0.0, eig_fg = 0.0;
        for (a = 0; a < D; a++) {
          eia_ua += (es[3 * i + a] / scaling) * vel[a];
          eig_fg += (es[3 * i + a] / scaling) * force[a];
        }
        const double s_i = w[i] * one_min_omega_half *
                           (prefactor * (eig_fg - ug_fg) + prefactor * prefactor * (eia_ua * eig_fg));
        fl[i] += dt * s_i;
      }
    }
    for (i = 0; i < Q; i++) f[(int64_t)i * n + ii] = fl[i];
  }
  return bad ? ORC_ERR_DENSITY : ORC_OK;
}

int orc_collide_bgk(int stencil, double scaling, double tau, int64_t n, double* f, double* rho, double* u,
                    int in_init, int nthreads) {
  return orc_collide_bgk_force(stencil, scaling, tau, 0.0, n, f, rho, u, in_init, 0, NULL, nthreads);
}

/* Legacy equilibrium, BGKStandard::getEquilibriumDistribution
 * (BGKStandard.cpp:23-41), scaled u and e, scaled c_s^2.  Used for the
 * equilibrium initialisation (CFDSolver.cpp:1103-1130). */
int orc_equilibrium(int stencil, double scaling, int64_t n, const double* rho,
                    const double* u, double* f) {
  int D, Q;
  double es[3 * 32], w[32], cs2s, vmax;
  int64_t ii;
  if (orc_stencil(stencil, scaling, &D, &Q, es, w, &cs2s, &vmax) != ORC_OK)
    return ORC_ERR_ARG;
  for (ii = 0; ii < n; ii++) {
    double uu = 0.0;
    int a, i;
    for (a = 0; a < D; a++) uu += u[(int64_t)a * n + ii] * u[(int64_t)a * n + ii];
    double usq = -uu / (2 * cs2s);
    for (i = 0; i < Q; i++) {
      double pre = w[i] * rho[ii];
      if (i == 0) {
        f[(int64_t)i * n + ii] = pre * (1 + usq);
        continue;
      }
      double ue = 0.0;
      for (a = 0; a < D; a++) ue += u[(int64_t)a * n + ii] * es[3 * i + a];
      double mixed = ue / cs2s;
      f[(int64_t)i * n + ii] = pre * (1 + mixed * (1 + 0.5 * (mixed)) + usq);
    }
  }
  return ORC_OK;
}

/* Legacy BGK::collideSinglePoint (BGK.cpp:24-45) with the BGKStandard
 * equilibrium; relax_param = nu/(dt cs2_scaled) (the legacy convention,
 * CollisionModel.h:152-157), prefactor -1/(relax_param + 1/2) (BGK.cpp:13-16). */
int orc_bgk_collide_single_point(int stencil, double scaling,
                                 double relax_param, double* fq) {
  int D, Q, i, a;
  double es[3 * 32], w[32], cs2s, vmax, u[3] = {0, 0, 0}, rho = 0, feq[32];
  if (orc_stencil(stencil, scaling, &D, &Q, es, w, &cs2s, &vmax) != ORC_OK)
    return ORC_ERR_ARG;
  for (i = 0; i < Q; i++) rho += fq[i];
  for (i = 0; i < Q; i++)
    for (a = 0; a < D; a++) u[a] += fq[i] * es[3 * i + a];
  for (a = 0; a < D; a++) u[a] *= 1. / rho;
  {
    double uu = 0;
    for (a = 0; a < D; a++) uu += u[a] * u[a];
    double usq = -uu / (2 * cs2s);
    for (i = 0; i < Q; i++) {
      double pre = w[i] * rho;
      if (i == 0) {
        feq[i] = pre * (1 + usq);
        continue;
      }
      double ue = 0;
      for (a = 0; a < D; a++) ue += u[a] * es[3 * i + a];
      double mixed = ue / cs2s;
      feq[i] = pre * (1 + mixed * (1 + 0.5 * mixed) + usq);
    }
  }
  double pf = -1. / (relax_param + 0.5);
  for (i = 0; i < Q; i++) fq[i] = fq[i] + pf * (fq[i] - feq[i]);
  return ORC_OK;
}

/* BGKIncompressible::collideAllD2Q9 (BGKIncompressible.cpp:62-190), lambda
 * = 1/3, gamma = 1/12 (BGKIncompressible.h:22-23).  Velocities are scaled.
 * Note the reference's weighting of directions 5-8 carries the density while
 * 0-4 do not (BGKIncompressible.cpp:133,137,157); restated as written. */
int orc_collide_bgk_incompressible_d2q9(double scaling, double tau, int64_t n,
                                        double* f, double* rho, double* u,
                                        int in_init) {
  const double lam = 1.0 / 3.0, gam = 1.0 / 12.0;
  double cs2 = scaling * scaling / 3.;
  double prefactor = scaling / cs2;
  double relax = -1. / tau;
  int64_t i;
  int bad = 0;
  double* F[9];
  int k;
  for (k = 0; k < 9; k++) F[k] = f + (int64_t)k * n;
  for (i = 0; i < n; i++) {
    double feq[9];
    rho[i] = F[0][i] + F[1][i] + F[2][i] + F[3][i] + F[4][i] + F[5][i] +
             F[6][i] + F[7][i] + F[8][i];
    if (rho[i] < 1e-10 || rho[i] != rho[i]) bad = 1;
    if (!in_init) {
      u[i] = scaling / rho[i] *
             (F[1][i] + F[5][i] + F[8][i] - F[3][i] - F[6][i] - F[7][i]);
      u[n + i] = scaling / rho[i] *
                 (F[2][i] + F[5][i] + F[6][i] - F[4][i] - F[7][i] - F[8][i]);
    }
    double ux = u[i], uy = u[n + i];
    double sigma = lam + gam;
    double sp = ux * ux + uy * uy;
    double usq = -sp / (2 * cs2);
    double wt = 4. / 9.;
    feq[0] = -4 * sigma * rho[i] + wt * (1 + usq);
    wt = 1. / 9.;
    double mixed = prefactor * (ux);
    feq[1] = lam * rho[i] + wt * (1 + mixed * (1 + 0.5 * mixed) + usq);
    feq[3] = lam * rho[i] + wt * (1 - mixed * (1 - 0.5 * mixed) + usq);
    mixed = prefactor * (uy);
    feq[2] = lam * rho[i] + wt * (1 + mixed * (1 + 0.5 * mixed) + usq);
    feq[4] = lam * rho[i] + wt * (1 - mixed * (1 - 0.5 * mixed) + usq);
    wt = 1. / 36. * rho[i];
    mixed = prefactor * (ux + uy);
    feq[5] = gam * rho[i] + wt * (1 + mixed * (1 + 0.5 * mixed) + usq);
    feq[7] = gam * rho[i] + wt * (1 - mixed * (1 - 0.5 * mixed) + usq);
    mixed = prefactor * (-ux + uy);
    feq[6] = gam * rho[i] + wt * (1 + mixed * (1 + 0.5 * mixed) + usq);
    feq[8] = gam * rho[i] + wt * (1 - mixed * (1 - 0.5 * mixed) + usq);
    for (k = 0; k < 9; k++) F[k][i] += relax * (F[k][i] - feq[k]);
  }
  return bad ? ORC_ERR_DENSITY : ORC_OK;
}

/* KBCStandard::collideAllD2Q9 (KBCStandard.cpp:88-497), KBC_C variant,
 * without the gamma / entropy statistics file.  beta = 1/(2 tau) with
 * tau = relax_param + 1/2 (KBCStandard.cpp:424).  If gamma_out is not NULL
 * the stabiliser of each node is written there. */
int orc_collide_kbc_d2q9(double scaling, double tau, int64_t n, double* f,
                         double* rho_out, double* u, int in_init,
                         double* gamma_out) {
  int64_t i;
  int bad = 0, k;
  double* F[9];
  const double s3 = sqrt(3);
  for (k = 0; k < 9; k++) F[k] = f + (int64_t)k * n;
  for (i = 0; i < n; i++) {
    double rho = F[0][i] + F[1][i] + F[2][i] + F[3][i] + F[4][i] + F[5][i] +
                 F[6][i] + F[7][i] + F[8][i];
    rho_out[i] = rho;
    if (rho < 1e-10 || rho != rho) bad = 1;
    if (!in_init) {
      u[i] = scaling / rho *
             (F[1][i] + F[5][i] + F[8][i] - F[3][i] - F[6][i] - F[7][i]);
      u[n + i] = scaling / rho *
                 (F[2][i] + F[5][i] + F[6][i] - F[4][i] - F[7][i] - F[8][i]);
    }
    double ux = u[i] / scaling, uy = u[n + i] / scaling;
    double T, N, Pi, A, Qxyy, Qyxx;
    double kk[9], s[9], h[9], seq[9], heq[9], feq[9], ds[9], dh[9];
    T = F[1][i] + F[2][i] + F[3][i] + F[4][i] +
        2 * (F[5][i] + F[6][i] + F[7][i] + F[8][i]);
    T = T / rho;
    N = F[1][i] - F[2][i] + F[3][i] - F[4][i];
    N = N / rho;
    Pi = F[5][i] - F[6][i] + F[7][i] - F[8][i];
    Pi = Pi / rho;
    kk[0] = rho;
    kk[1] = 0.5 * rho * ux;
    kk[3] = 0.5 * rho * -ux;
    kk[2] = 0.5 * rho * uy;
    kk[4] = 0.5 * rho * -uy;
    kk[5] = kk[6] = kk[7] = kk[8] = 0;
    s[0] = -rho * T;
    s[1] = 0.5 * rho * 0.5 * (T + N);
    s[2] = 0.5 * rho * 0.5 * (T - N);
    s[3] = 0.5 * rho * 0.5 * (T + N);
    s[4] = 0.5 * rho * 0.5 * (T - N);
    s[5] = 0.25 * rho * Pi;
    s[6] = 0.25 * rho * -Pi;
    s[7] = 0.25 * rho * Pi;
    s[8] = 0.25 * rho * -Pi;
    for (k = 0; k < 9; k++) h[k] = F[k][i] - kk[k] - s[k];
    double uxi = ux * s3, uyi = uy * s3;
    double sqx = sqrt(1 + uxi * uxi), sqy = sqrt(1 + uyi * uyi);
    double pre = rho * (2 - sqx) * (2 - sqy);
    double px = (2 * uxi / s3 + sqx) / (1 - uxi / s3);
    double py = (2 * uyi / s3 + sqy) / (1 - uyi / s3);
    feq[0] = 4. / 9. * pre;
    feq[1] = 1. / 9. * pre * px;
    feq[2] = 1. / 9. * pre * py;
    feq[3] = 1. / 9. * pre / px;
    feq[4] = 1. / 9. * pre / py;
    feq[5] = 1. / 36. * pre * px * py;
    feq[6] = 1. / 36. * pre / px * py;
    feq[7] = 1. / 36. * pre / px / py;
    feq[8] = 1. / 36. * pre * px / py;
    T = feq[1] + feq[2] + feq[3] + feq[4] + 2 * (feq[5] + feq[6] + feq[7] + feq[8]);
    T = T / rho;
    N = feq[1] - feq[2] + feq[3] - feq[4];
    N = N / rho;
    Pi = feq[5] - feq[6] + feq[7] - feq[8];
    Pi = Pi / rho;
    Qxyy = Qyxx = A = 0;
    (void)Qxyy;
    (void)Qyxx;
    (void)A;
    seq[0] = -rho * T;
    seq[1] = 0.5 * rho * 0.5 * (T + N);
    seq[3] = 0.5 * rho * 0.5 * (T + N);
    seq[2] = 0.5 * rho * 0.5 * (T - N);
    seq[4] = 0.5 * rho * 0.5 * (T - N);
    seq[5] = 0.25 * rho * Pi;
    seq[6] = 0.25 * rho * -Pi;
    seq[7] = 0.25 * rho * Pi;
    seq[8] = 0.25 * rho * -Pi;
    for (k = 0; k < 9; k++) heq[k] = feq[k] - kk[k] - seq[k];
    double sum_s = 0, sum_h = 0;
    for (k = 0; k < 9; k++) {
      ds[k] = s[k] - seq[k];
      dh[k] = h[k] - heq[k];
    }
    for (k = 0; k < 9; k++) sum_s += ds[k] * dh[k] / feq[k];
    for (k = 0; k < 9; k++) sum_h += dh[k] * dh[k] / feq[k];
    double beta = 1. / (tau) / 2;
    double gamma = 1. / beta - (2 - 1. / beta) * (sum_s / sum_h);
    if (sum_h < 1e-16) gamma = 2;
    if (gamma_out) gamma_out[i] = gamma;
    for (k = 0; k < 9; k++) F[k][i] = F[k][i] - beta * (2 * ds[k] + gamma * dh[k]);
  }
  return bad ? ORC_ERR_DENSITY : ORC_OK;
}

/* KBC for D3Q27 -- no reference implementation (KBCStandard.cpp:65-86 throws
 * for every stencil but D2Q9 / D3Q15).  Extension of the D2Q9 KBC_C
 * construction above: the shear part s carries the full second moment at
 * unit density (rest: -rho T; axis +-a: rho M_aa / 2; face diagonal in the
 * (a,b) plane: rho M_ab c_a c_b / 4), the equilibrium is the product form of
 * KBCStandard::getEquilibriumDistribution (KBCStandard.cpp:26-63), and
 * dh = (f - feq) - ds because the kinematic part cancels.  Parity unpinned. */
static void kbc27_shear(const double* fl, double rho, const double e[27][3],
                        double* s) {
  double M[3][3] = {{0}};
  int i, a, b;
  for (i = 0; i < 27; i++)
    for (a = 0; a < 3; a++)
      for (b = 0; b < 3; b++) M[a][b] += fl[i] * e[i][a] * e[i][b];
  for (a = 0; a < 3; a++)
    for (b = 0; b < 3; b++) M[a][b] /= rho;
  double T = M[0][0] + M[1][1] + M[2][2];
  for (i = 0; i < 27; i++) {
    int nz = (e[i][0] != 0) + (e[i][1] != 0) + (e[i][2] != 0);
    if (nz == 0) {
      s[i] = -rho * T;
    } else if (nz == 1) {
      for (a = 0; a < 3; a++)
        if (e[i][a] != 0) s[i] = 0.5 * rho * M[a][a];
    } else if (nz == 2) {
      int ia = -1, ib = -1;
      for (a = 0; a < 3; a++)
        if (e[i][a] != 0) {
          if (ia < 0)
            ia = a;
          else
            ib = a;
        }
      s[i] = 0.25 * rho * M[ia][ib] * e[i][ia] * e[i][ib];
    } else {
      s[i] = 0.0;
    }
  }
}

int orc_collide_kbc_d3q27(double scaling, double tau, int64_t n, double* f,
                          double* rho_out, double* u, int in_init,
                          double* gamma_out) {
  int64_t ii;
  int bad = 0;
  double e[27][3], w[27];
  {
    int i, a;
    for (i = 0; i < 27; i++) {
      w[i] = (i == 0) ? 8. / 27.
                      : (i <= 6 ? 2. / 27. : (i <= 18 ? 1. / 54. : 1. / 216.));
      for (a = 0; a < 3; a++) e[i][a] = D3Q27_E[i][a];
    }
  }
  for (ii = 0; ii < n; ii++) {
    double fl[27], feq[27], s[27], seq[27], ds[27], dh[27], vel[3] = {0, 0, 0};
    double rho = 0;
    int i, a;
    for (i = 0; i < 27; i++) fl[i] = f[(int64_t)i * n + ii];
    for (i = 0; i < 27; i++) rho += fl[i];
    rho_out[ii] = rho;
    if (rho < 1e-10 || rho != rho) bad = 1;
    if (!in_init) {
      for (a = 0; a < 3; a++) {
        double m = 0;
        for (i = 0; i < 27; i++) m += e[i][a] * fl[i];
        vel[a] = m / rho;
        u[(int64_t)a * n + ii] = vel[a] * scaling;
      }
    } else {
      for (a = 0; a < 3; a++) vel[a] = u[(int64_t)a * n + ii] / scaling;
    }
    double fac[3][3]; /* per axis: [c=-1], [c=0], [c=+1] factors */
    for (a = 0; a < 3; a++) {
      double v = vel[a] * sqrt(3.);
      double sq = sqrt(1 + v * v);
      double base = 2 - sq;
      double post = (2 * v / sqrt(3.) + sq) / (1 - v / sqrt(3.));
      fac[a][0] = base / post;
      fac[a][1] = base;
      fac[a][2] = base * post;
    }
    for (i = 0; i < 27; i++) {
      double val = w[i] * rho;
      for (a = 0; a < 3; a++) val *= fac[a][(int)e[i][a] + 1];
      feq[i] = val;
    }
    kbc27_shear(fl, rho, e, s);
    kbc27_shear(feq, rho, e, seq);
    double sum_s = 0, sum_h = 0;
    for (i = 0; i < 27; i++) {
      ds[i] = s[i] - seq[i];
      dh[i] = (fl[i] - feq[i]) - ds[i];
    }
    for (i = 0; i < 27; i++) sum_s += ds[i] * dh[i] / feq[i];
    for (i = 0; i < 27; i++) sum_h += dh[i] * dh[i] / feq[i];
    double beta = 1. / tau / 2;
    double gamma = 1. / beta - (2 - 1. / beta) * (sum_s / sum_h);
    if (sum_h < 1e-16) gamma = 2;
    if (gamma_out) gamma_out[ii] = gamma;
    for (i = 0; i < 27; i++)
      f[(int64_t)i * n + ii] = fl[i] - beta * (2 * ds[i] + gamma * dh[i]);
  }
  return bad ? ORC_ERR_DENSITY : ORC_OK;
}

/* One time step of the reference loop in its own algorithmic form: copy f,
 * per-direction CSR SpMV, separate BGK collide sweep (CFDSolver.cpp:658-843).
 * f and work are Q*n; after the call f holds the new state. */
int orc_step_bgk(const orc_sl* s, int stencil, double scaling, double tau,
                 double* f, double* work, double* rho, double* u, int nsteps,
                 int nthreads) {
  int k, rc = ORC_OK;
  for (k = 0; k < nsteps; k++) {
    orc_sl_stream(s, f, work, nthreads);
    memcpy(f, work, sizeof(double) * (size_t)s->Q * s->n);
    rc = orc_collide_bgk(stencil, scaling, tau, s->n, f, rho, u, 0, nthreads);
    if (rc != ORC_OK) return rc;
  }
  return rc;
}

/* ------------------------------------------------------------------------ */
/* compressible two-population model (D2Q25H)                                */
/* ------------------------------------------------------------------------ */

/* Per-call constants of the compressible collision: unscaled directions
 * e = direction / scaling, weights and unscaled c_s^2 = scaled c_s^2 /
 * scaling^2 (GeneralCollisionData, AuxiliaryCollisionFunctions.h:151-178),
 * and the Hermite tensors computed once per collideAll call
 * (CollisionOperator.h:151-152; calculateH3 / calculateH4,
 * AuxiliaryCollisionFunctions.h:520-566). */
typedef struct {
  int D, Q;
  double e[32][3], w[32], cs2;
  double H3[32][2][2][2];
  double H4[32][2][2][2][2];
} orc_thermal_k;

static int thermal_consts(int stencil, double scaling, orc_thermal_k* k) {
  double es[3 * 32], cs2s, vmax;
  int i, a, b, c, d;
  if (stencil != ORC_D2Q25H) return ORC_ERR_ARG;
  if (orc_stencil(stencil, scaling, &k->D, &k->Q, es, k->w, &cs2s, &vmax) != ORC_OK) return ORC_ERR_ARG;
  for (i = 0; i < k->Q; i++)
    for (a = 0; a < 3; a++) k->e[i][a] = es[3 * i + a] / scaling;
  k->cs2 = cs2s / (scaling * scaling);
  for (i = 0; i < k->Q; i++) {
    const double* e = k->e[i];
    const double cs2 = k->cs2;
    for (a = 0; a < 2; a++)
      for (b = 0; b < 2; b++)
        for (c = 0; c < 2; c++) {
          const double dbc = b == c, dac = a == c, dab = a == b;
          k->H3[i][a][b][c] = e[a] * e[b] * e[c] - cs2 * (e[a] * dbc + e[b] * dac + e[c] * dab);
          for (d = 0; d < 2; d++) {
            const double dcd = c == d, dbd = b == d, dad = a == d;
            const double power4 = e[a] * e[b] * e[c] * e[d];
            const double power2 = e[a] * e[b] * dcd + e[a] * e[c] * dbd + e[a] * e[d] * dbc +
                                  e[b] * e[c] * dad + e[b] * e[d] * dac + e[c] * e[d] * dab;
            const double power0 = dab * dcd + dac * dbd + dad * dbc;
            k->H4[i][a][b][c][d] = (power4 - cs2 * power2 + cs2 * cs2 * power0);
          }
        }
  }
  return ORC_OK;
}

/* QuarticEquilibrium::polynomial for T_D = 2 (Equilibria.h:130-267), in the
 * reference's order of operations.  u unscaled. */
static void quartic_feq(const orc_thermal_k* k, double rho, const double* u, double T, double* feq) {
  const double cs2 = k->cs2;
  double uu_term = 0.0;
  int i, j, alp, bet;
  for (j = 0; j < 2; j++) uu_term += -(u[j] * u[j]) / (2.0 * cs2);
  const double T1 = cs2 * (T - 1);
  const double a_xxx = u[0] * u[0] * u[0] + T1 * (u[0] + u[0] + u[0]);
  const double a_xxy = u[0] * u[0] * u[1] + T1 * (u[1]);
  const double a_xyy = u[0] * u[1] * u[1] + T1 * (u[0]);
  const double a_yyy = u[1] * u[1] * u[1] + T1 * (u[1] + u[1] + u[1]);
  const double a_xxxx = u[0] * u[0] * u[0] * u[0] + T1 * u[0] * u[0] * 6.0 + T1 * T1 * 3.0;
  const double a_yyyy = u[1] * u[1] * u[1] * u[1] + T1 * u[1] * u[1] * 6.0 + T1 * T1 * 3.0;
  const double a_xxxy = u[0] * u[0] * u[0] * u[1] + T1 * (u[0] * u[1] * 3.0);
  const double a_xyyy = u[0] * u[1] * u[1] * u[1] + T1 * (u[0] * u[1] * 3.0);
  const double a_xxyy = u[0] * u[0] * u[1] * u[1] + T1 * (u[0] * u[0] + u[1] * u[1]) + T1 * T1;
  for (i = 0; i < k->Q; i++) {
    const double* e = k->e[i];
    const double w = k->w[i];
    double ue_term = 0.0;
    for (j = 0; j < 2; j++) ue_term += (u[j] * e[j]) / cs2;
    feq[i] = w * rho * (1 + ue_term * (1 + 0.5 * (ue_term)) + uu_term);
    for (alp = 0; alp < 2; alp++)
      for (bet = 0; bet < 2; bet++) {
        const double eye = alp == bet;
        feq[i] += rho * w / (2.0 * cs2) * ((T - 1) * eye * e[alp] * e[bet] - cs2 * eye * (T - 1));
      }
    feq[i] += w * rho / (6. * cs2 * cs2 * cs2) *
              (a_xxx * k->H3[i][0][0][0] + 3 * (a_xxy * k->H3[i][0][0][1] + a_xyy * k->H3[i][0][1][1]) +
               a_yyy * k->H3[i][1][1][1]);
    feq[i] += w * rho / (24. * cs2 * cs2 * cs2 * cs2) *
              (k->H4[i][0][0][0][0] * a_xxxx + k->H4[i][1][1][1][1] * a_yyyy + 6.0 * k->H4[i][0][0][1][1] * a_xxyy +
               4.0 * k->H4[i][0][1][1][1] * a_xyyy + 4.0 * k->H4[i][0][0][0][1] * a_xxxy);
  }
}

/* BGKEquilibrium, generic form (Equilibria.h:66-83); u unscaled. */
static void bgk_feq(const orc_thermal_k* k, double rho, const double* u, double* feq) {
  double uu = 0.0;
  int i, j;
  for (j = 0; j < k->D; j++) uu += -(u[j] * u[j]) / (2.0 * k->cs2);
  for (i = 0; i < k->Q; i++) {
    double ue = 0.0;
    for (j = 0; j < k->D; j++) ue += (u[j] * k->e[i][j]) / k->cs2;
    feq[i] = k->w[i] * rho * (1 + ue * (1 + 0.5 * (ue)) + uu);
  }
}

/* CompressibleCFDSolver::calcQuarticEquilibrium (CompressibleCFDSolver.h:790-840):
 * the same quartic equilibrium written as full tensor contractions; the
 * initialisation uses this form. */
static void quartic_feq_tensor(const orc_thermal_k* k, double density, const double* velocity,
                               double temperature, double* feq) {
  const int dim = 2;
  const double cs2 = k->cs2;
  double uu_term = 0.0;
  int i, j, alp, bet, gam, det;
  for (j = 0; j < dim; j++) uu_term += -(velocity[j] * velocity[j]) / (2.0 * cs2);
  for (i = 0; i < k->Q; i++) {
    const double* e = k->e[i];
    const double weight = k->w[i];
    const double T1 = cs2 * (temperature - 1);
    double ue_term = 0.0;
    for (j = 0; j < dim; j++) ue_term += (velocity[j] * e[j]) / cs2;
    feq[i] = weight * density * (1 + ue_term * (1 + 0.5 * (ue_term)) + uu_term);
    for (alp = 0; alp < dim; alp++)
      for (bet = 0; bet < dim; bet++) {
        const double dab = alp == bet;
        feq[i] += density * weight / (2.0 * cs2) * ((temperature - 1) * dab * e[alp] * e[bet] - cs2 * dab * (temperature - 1));
        for (gam = 0; gam < dim; gam++) {
          const double dbg = bet == gam, dag = alp == gam;
          feq[i] += weight * density / (6. * cs2 * cs2 * cs2) *
                    (velocity[alp] * velocity[bet] * velocity[gam] +
                     T1 * (dab * velocity[gam] + dbg * velocity[alp] + dag * velocity[bet])) *
                    (e[alp] * e[bet] * e[gam] - cs2 * (e[gam] * dab + e[bet] * dag + e[alp] * dbg));
          for (det = 0; det < dim; det++) {
            const double dgd = gam == det, dbd = bet == det, dad = alp == det;
            const double power4 = e[alp] * e[bet] * e[gam] * e[det];
            const double power2 = e[alp] * e[bet] * dgd + e[alp] * e[gam] * dbd + e[alp] * e[det] * dbg +
                                  e[bet] * e[gam] * dad + e[bet] * e[det] * dag + e[gam] * e[det] * dab;
            const double power0 = dab * dgd + dag * dbd + dad * dbg;
            const double u4 = velocity[alp] * velocity[bet] * velocity[gam] * velocity[det];
            const double u2 = velocity[alp] * velocity[bet] * dgd + velocity[alp] * velocity[gam] * dbd +
                              velocity[alp] * velocity[det] * dbg + velocity[bet] * velocity[gam] * dad +
                              velocity[bet] * velocity[det] * dag + velocity[gam] * velocity[det] * dab;
            const double multieye = dab * dgd + dag * dbd + dad * dbg;
            feq[i] += weight * density / (24. * cs2 * cs2 * cs2 * cs2) * (power4 - cs2 * power2 + cs2 * cs2 * power0) *
                      (u4 + T1 * (u2 + T1 * multieye));
          }
        }
      }
  }
}

/* Equilibrium initialisation of both populations
 * (CompressibleCFDSolver::initializeDistributions, CompressibleCFDSolver.h:849-899):
 * f = f^eq(rho, u, T) (tensor form above), g = f^eq T (2 C_v - D),
 * C_v = 1 / (gamma - 1).  u holds the scaled velocity. */
int orc_thermal_init(int stencil, double scaling, double gamma, int64_t n, const double* rho,
                     const double* u, const double* T, double* f, double* g) {
  orc_thermal_k k;
  int64_t ii;
  if (thermal_consts(stencil, scaling, &k) != ORC_OK) return ORC_ERR_ARG;
  const double C_v = 1. / (gamma - 1.0);
  for (ii = 0; ii < n; ii++) {
    double vel[2], feq[32];
    int j;
    for (j = 0; j < 2; j++) vel[j] = u[(int64_t)j * n + ii] / scaling;
    quartic_feq_tensor(&k, rho[ii], vel, T[ii], feq);
    for (j = 0; j < k.Q; j++) {
      f[(int64_t)j * n + ii] = feq[j];
      g[(int64_t)j * n + ii] = feq[j] * (T[ii]) * (2.0 * C_v - 2);
    }
  }
  return ORC_OK;
}

/* Quartic (quartic != 0) or second-order BGK equilibrium of the collision,
 * for tests.  u scaled; feq is Q blocks of n. */
int orc_thermal_feq(int stencil, double scaling, int quartic, int64_t n, const double* rho,
                    const double* u, const double* T, double* feq_out) {
  orc_thermal_k k;
  int64_t ii;
  if (thermal_consts(stencil, scaling, &k) != ORC_OK) return ORC_ERR_ARG;
  for (ii = 0; ii < n; ii++) {
    double vel[2], feq[32];
    int j;
    for (j = 0; j < 2; j++) vel[j] = u[(int64_t)j * n + ii] / scaling;
    if (quartic)
      quartic_feq(&k, rho[ii], vel, T[ii], feq);
    else
      bgk_feq(&k, rho[ii], vel, feq);
    for (j = 0; j < k.Q; j++) feq_out[(int64_t)j * n + ii] = feq[j];
  }
  return ORC_OK;
}

/* CollisionOperator::collideAll(f, g, ...) (CollisionOperator.h:113-224)
 * with BGKCollision::relaxWithG (CollisionSchemes.h:43-118):
 *   rho = sum f; u = sum e f / rho (AuxiliaryCollisionFunctions.h:232-242);
 *   T = 0.5 / (rho C_v) sum_i (|e_i - u|^2 f_i / c_s^2 + g_i) (:289-307);
 *   in the initialisation procedure u is then replaced by the prescribed one;
 *   f^eq from the quartic (or second-order) equilibrium, g^eq = f^eq T (2 C_v - D)
 *   (:420-431);
 *   Prandtl correction (if set): f*, g* from the centred heat flux of f^neq
 *   and the centred flux of g^neq (:445-516);
 *   Sutherland factor (T / 0.85)^0.7 (if set);
 *   tau_visc = (tau - 1/2) s / (T rho) + 1/2; Knudsen estimate
 *   sum |f - f^eq| / w / Q (:474-481) written to the shock mask (the
 *   reference's tau factor derived from it is not applied, :95-101);
 *   f -= omega f^neq - (omega - omega_Pr) f*; g likewise.
 * Writes rho, u (scaled, unless in_init), T and the mask.  Returns
 * ORC_ERR_DENSITY if a density is below 1e-10. */
int orc_collide_compressible(int stencil, double scaling, double tau, double gamma, double prandtl,
                             int prandtl_set, int sutherland_set, int quartic, int64_t n, double* f,
                             double* g, double* rho, double* u, double* T, double* mask, int in_init,
                             int nthreads) {
  orc_thermal_k k;
  int bad = 0;
  int64_t ii;
  if (thermal_consts(stencil, scaling, &k) != ORC_OK) return ORC_ERR_ARG;
  const int D = k.D, Q = k.Q;
  const double cs2 = k.cs2;
  const double C_v = 1. / (gamma - 1.0);
  (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad) num_threads(nthreads > 0 ? nthreads : 1)
#endif
  for (ii = 0; ii < n; ii++) {
    double fl[32], gl[32], feq[32], geq[32], fNeq[32], gNeq[32], fStar[32], gStar[32];
    double vel[2], dens = 0.0, temp;
    int i, a, b, c;
    for (i = 0; i < Q; i++) fl[i] = f[(int64_t)i * n + ii];
    for (i = 0; i < Q; i++) gl[i] = g[(int64_t)i * n + ii];
    for (i = 0; i < Q; i++) dens += fl[i];
    if (dens < 1e-10 || dens != dens) bad = 1;
    rho[ii] = dens;
    for (a = 0; a < D; a++) {
      vel[a] = 0.0;
      for (i = 0; i < Q; i++) vel[a] += k.e[i][a] * fl[i];
      vel[a] = vel[a] * 1.0 / dens;
    }
    temp = 0.0;
    for (i = 0; i < Q; i++) {
      double sum = 0.0;
      for (a = 0; a < D; a++) sum += (k.e[i][a] - vel[a]) * (k.e[i][a] - vel[a]);
      temp += sum * fl[i] / cs2 + gl[i];
    }
    temp = temp * 0.5 / (dens * C_v);
    T[ii] = temp;
    if (!in_init) {
      for (a = 0; a < D; a++) u[(int64_t)a * n + ii] = vel[a] * scaling;
    } else {
      for (a = 0; a < D; a++) vel[a] = u[(int64_t)a * n + ii] / scaling;
    }
    if (quartic)
      quartic_feq(&k, dens, vel, temp, feq);
    else
      bgk_feq(&k, dens, vel, feq);
    for (i = 0; i < Q; i++) geq[i] = feq[i] * (temp) * (2.0 * C_v - D);
    for (i = 0; i < Q; i++) {
      fStar[i] = 0.0;
      gStar[i] = 0.0;
      fNeq[i] = fl[i] - feq[i];
      gNeq[i] = gl[i] - geq[i];
    }
    if (prandtl_set) {
      double Qn[2][2][2] = {{{0.0}}}, F[2] = {0.0, 0.0};
      const double cs6 = 6.0 * cs2 * cs2 * cs2;
      for (i = 0; i < Q; i++)
        for (a = 0; a < D; a++)
          for (b = 0; b < D; b++)
            for (c = 0; c < D; c++)
              Qn[a][b][c] += ((k.e[i][a] - vel[a]) * (k.e[i][b] - vel[b]) * (k.e[i][c] - vel[c])) * fNeq[i];
      for (i = 0; i < Q; i++)
        for (a = 0; a < D; a++) F[a] += (k.e[i][a] - vel[a]) * gNeq[i];
      for (a = 0; a < D; a++)
        for (b = 0; b < D; b++)
          for (c = 0; c < D; c++)
            for (i = 0; i < Q; i++)
              fStar[i] += k.w[i] * (Qn[a][b][c] * (k.e[i][a] * k.e[i][b] * k.e[i][c] -
                                                  3 * cs2 * k.e[i][c] * (double)(a == b))) / cs6;
      for (a = 0; a < D; a++)
        for (i = 0; i < Q; i++) gStar[i] += k.w[i] * (F[a] * k.e[i][a]) / temp;
    }
    double sutherland_factor = 1.0;
    if (sutherland_set) sutherland_factor = pow(temp / 0.85, 0.7);
    const double visc_tau = (tau - 0.5) * sutherland_factor / (temp * dens) + 0.5;
    double knudsen = 0.0;
    for (i = 0; i < Q; i++) knudsen += fabs(fl[i] - feq[i]) / k.w[i];
    knudsen = knudsen / Q;
    mask[ii] = knudsen;
    const double prandtl_tau = (visc_tau - 0.5) / prandtl + 0.5;
    const double visc_omega = 1. / visc_tau;
    const double prandtl_omega = 1. / prandtl_tau;
    const double prandtl_diff = visc_omega - prandtl_omega;
    for (i = 0; i < Q; i++) {
      fl[i] -= visc_omega * fNeq[i] - prandtl_diff * fStar[i];
      gl[i] -= visc_omega * gNeq[i] - prandtl_diff * gStar[i];
    }
    for (i = 0; i < Q; i++) {
      f[(int64_t)i * n + ii] = fl[i];
      g[(int64_t)i * n + ii] = gl[i];
    }
  }
  return bad ? ORC_ERR_DENSITY : ORC_OK;
}

/* One step of CompressibleCFDSolver::run (CompressibleCFDSolver.h:1013-1035):
 * stream() and gStream() (copy + SpMV with the same operator, :181-314),
 * then collide() (:739-788).  work is Q*n. */
int orc_step_compressible(const orc_sl* s, int stencil, double scaling, double tau, double gamma,
                          double prandtl, int prandtl_set, int sutherland_set, int quartic, double* f,
                          double* g, double* work, double* rho, double* u, double* T, double* mask,
                          int nsteps, int nthreads) {
  int k, rc = ORC_OK;
  const size_t bytes = sizeof(double) * (size_t)s->Q * s->n;
  for (k = 0; k < nsteps; k++) {
    orc_sl_stream(s, f, work, nthreads);
    memcpy(f, work, bytes);
    orc_sl_stream_g(s, g, work, nthreads);
    memcpy(g, work, bytes);
    rc = orc_collide_compressible(stencil, scaling, tau, gamma, prandtl, prandtl_set, sutherland_set, quartic,
                                  s->n, f, g, rho, u, T, mask, 0, nthreads);
    if (rc != ORC_OK) return rc;
  }
  return rc;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
