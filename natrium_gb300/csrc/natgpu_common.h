// Data structures shared by the host API (natgpu_api.cu) and the kernels.
//
// Device data layout (HBM):
//   f:    Q blocks of n_dev values (SoA), block 0 = rest population; a block
//         is the node lattice of the periodic box stored x fastest, then y,
//         then z.  On a periodic FE_Q lattice the duplicate nodes at x = L
//         are folded onto x = 0, so an axis holds N p nodes (N (p+1) for DG).
//   rho:  n_dev doubles; u: D blocks of n_dev doubles (scaled velocity).
// The streaming operator of every direction is a Kronecker product of 1-D
// banded operators (Cartesian cells, tensor-product Lagrange basis):
//   (A_alpha f)(x,y,z) = sum_{i,j,k} Wx[x][i] Wy[y][j] Wz[z][k]
//                        f(sx(x)+i, sy(y)+j, sz(z)+k),
// with identity factors on axes where e_alpha has no component.  A 1-D
// factor depends only on the node's class (its local index in the cell) and
// on the displacement class of the direction on that axis; the tables below
// hold, per axis / displacement class / node class, the window offset and the
// p+1 weights.
#pragma once

#include <stdint.h>

namespace natgpu {

constexpr int PMAX = 6;          // highest FE order supported
constexpr int PMAX1 = PMAX + 1;  // window length bound
constexpr int PER_MAX = PMAX + 1;
constexpr int ND_MAX = 4;        // nonzero displacement classes per axis
constexpr int BMAX = 64;         // tile extent bound per axis (nodes)
constexpr int RMAX = BMAX + 2 * PMAX1 + 2;  // region extent bound per axis

// collision selectors of the fused kernels
constexpr int COLL_NONE = 0;
constexpr int COLL_BGK = 1;
constexpr int COLL_BGK_INC = 2;
constexpr int COLL_KBC = 3;

// device status word bits
constexpr int ST_DENSITY = 1;
constexpr int ST_NAN = 2;

struct AxisGeom {
  int n;       // lattice nodes on this axis (periodic torus)
  int period;  // node classes per cell (p for FE_Q, p + 1 for DG)
  int B;       // tile extent in nodes (a multiple of period)
  int ntiles;  // n / B
  int nd;      // number of nonzero displacement classes on this axis
  int lo[ND_MAX];  // source region start relative to the tile start
  int R[ND_MAX];   // source region extent
};

// Streaming tables, one copy per solver in device memory (loaded into
// shared memory by every CTA).
struct SLTables {
  AxisGeom ax[3];
  int p;
  int dim;
  int Rmax[3];  // max over classes of R (B when the axis has no class)
  // weights[axis][dclass][node class][j], j <= p (double; float copy below)
  double w[3][ND_MAX][PER_MAX][PMAX1];
  float wf[3][ND_MAX][PER_MAX][PMAX1];
  // window start, local to the source region, of tile output o
  int wst[3][ND_MAX][BMAX];
  // window offset relative to the node itself, per node class
  int off[3][ND_MAX][PER_MAX];
  // index inside the window of the dominant weight (the source node at the
  // destination node's own position), per node class
  int j0[3][ND_MAX][PER_MAX];
};

struct StepParams {
  const void* f_in;
  void* f_out;
  double* rho;
  double* u;
  int* status;
  const SLTables* tab;
  long long n;  // nodes per block
  int nx, ny, nz;
  double tau;
  double scaling;
  int write_macro;
  int in_init;
  int collide;  // 0: stream only
  // constant body force (BGK only): 0 none, 1 shifting velocity, 2 exact
  // difference; dF = dt F / scaling, the momentum a node gains per step
  int force_scheme;
  double dF[3];
};

constexpr int TH_WARPS = 8;   // warps per CTA of the fused kernel
constexpr int TH_WARPS_SS = 4;  // warps per CTA of its shared-memory (FP32) form
constexpr int TH_BWMAX = 64;  // x buffer width bound: 32 nodes + window halo
constexpr int TH_Q = 25;
constexpr int TH_NG = 9;

// Compressible two-population model (D2Q25H, sl_thermal.cuh).
// Per-solve constants of the collision (built on the host from the
// reference's stencil formulas) in the arithmetic type Real.  Group values
// are for the member with e_x >= 0, e_y >= 0.
template <class Real>
struct ThermalModelT {
  Real X[TH_NG], Y[TH_NG];  // |e_x|, |e_y| (unscaled)
  Real e2[TH_NG];           // |e|^2
  Real w[TH_NG];            // weight of every member
  Real winv[TH_NG];         // 1 / weight (Knudsen estimate)
  Real h3[TH_NG][4];        // H_xxx, H_xxy, H_xyy, H_yyy
  Real h4[TH_NG][5];        // H_xxxx, H_xxxy, H_xxyy, H_xyyy, H_yyyy
  Real cs2;                 // unscaled c_s^2 (scaled c_s^2 / scaling^2)
  Real tau;                 // nu / (dt c_s^2 scaled) + 1/2
  Real C_v;                 // 1 / (gamma - 1)
  Real gfac;                // 2 C_v - D
  Real gref;                // deviation storage of g: g - w_i gref (fixed per solve)
  Real prandtl;
  double scaling;
  int prandtl_set;
  int sutherland_set;
  int quartic;              // 1: quartic equilibrium, 0: second-order BGK equilibrium
};

// Streaming tables of the two axes: [axis][displacement class][node class].
template <class Real>
struct ThermalTablesT {
  Real w[2][ND_MAX][PER_MAX][PMAX1];
  int off[2][ND_MAX][PER_MAX];
  int j0[2][ND_MAX][PER_MAX];  // window index of the dominant weight
  int offy[ND_MAX][PER_MAX];   // y window offset reduced to [0, ny): rows wrap by subtraction only
  int p, per;
  int xl;  // first buffer position relative to the segment start
  int bw;  // buffer width (<= TH_BWMAX)
};

// Real = double: plain FP64 state.  Real = float: deviations f - w_i and
// g - w_i gref stored and computed in float.
template <class Real>
struct ThermalStepT {
  const Real* f_in;
  const Real* g_in;
  Real* f_out;
  Real* g_out;
  double* rho;
  double* u;
  double* T;
  double* mask;
  int* status;
  int n, nx, ny, nseg;
  int write_macro;
  // wall nodes: one word per warp row segment (y nseg + x / 32), bit x % 32;
  // their streamed values wait in f_out / g_out (written by k_thermal_rows
  // before the step) and replace the lattice stencil's.  nullptr: no walls.
  const unsigned* wall_bits;
  ThermalTablesT<Real> tb;
  ThermalModelT<Real> M;
};

template <class Real>
struct ThermalPointT {
  Real* f;  // collide / init: in place
  Real* g;
  double* rho;
  double* u;
  double* T;
  double* mask;
  int* status;
  long long n;
  int in_init;
  ThermalModelT<Real> M;
};

}  // namespace natgpu
