// Host side of libnatgpu.so: the C ABI declared in include/natgpu.h.
//
// Owns the device state of one solve (distribution functions in HBM,
// macroscopic fields, streaming tables, status word) and enqueues the
// kernels on the handle's CUDA stream.  Operator assembly (the reference's
// SemiLagrangian::updateSparsityPattern + reassemble,
// advection/SemiLagrangian.cpp:93-141, 145-522) reduces on a Cartesian box to
// the per-axis 1-D tables built in build_tables(): departure point of every
// node class, the cell that holds it, and the Lagrange weights there, in FP64.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <thread>
#include <vector>

#include "../../include/natgpu.h"
#include "collision.cuh"
#include "launch.h"
#include "natgpu_common.h"
#include "sl_mapped.cuh"
#include "sl_row.cuh"
#include "sl_rowt.cuh"
#include "sl_step.cuh"
#include "sl_step_v2.cuh"
#include "solver.h"

using namespace natgpu;


namespace natgpu {
namespace api {

int fail(nat_solver* s, int code, const char* fmt, ...) {
  if (s) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    s->err = buf;
  }
  return code;
}

int cuda_fail(nat_solver* s, cudaError_t e, const char* what) {
  return fail(s, NAT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}



template <class S>
HostStencil host_stencil(double scaling) {
  HostStencil h;
  h.D = S::D;
  h.Q = S::Q;
  for (int i = 0; i < S::Q; ++i) {
    for (int a = 0; a < 3; ++a) h.e[i][a] = S::e(i, a);
    h.w[i] = S::w(i);
  }
  h.nd = 2;
  h.cls[0] = scaling;  // e_a = +1
  h.cls[1] = -scaling;
  return h;
}

// D2Q25H speeds and weights exactly as the reference forms them
// (stencils/D2Q25H.cpp:37-84); e unscaled = direction / scaling, as
// GeneralCollisionData does (AuxiliaryCollisionFunctions.h:161-165).
void d2q25h_speeds(double scaling, double* cm_s, double* cn_s) {
  *cm_s = scaling * sqrt(5. - sqrt(10.)) / sqrt(3.);
  *cn_s = sqrt(5. + sqrt(10.)) * scaling / sqrt(3.);
}

void d2q25h_weights(double* w0, double* wm, double* wn) {
  const double r = (sqrt(5.) - sqrt(2.)) / sqrt(3.);
  *w0 = (-3 - 3 * r * r * r * r + 54 * r * r) / (75 * r * r);
  *wm = (9 * r * r * r * r - 6 - 27 * r * r) / (300 * r * r * (r * r - 1));
  *wn = (9 - 6 * r * r * r * r - 27 * r * r) / (300 * (1 - r * r));
}

HostStencil host_stencil_d2q25h(double scaling) {
  HostStencil h;
  memset(&h, 0, sizeof(h));
  h.D = 2;
  h.Q = 25;
  double cm_s, cn_s, w0, wm, wn;
  d2q25h_speeds(scaling, &cm_s, &cn_s);
  d2q25h_weights(&w0, &wm, &wn);
  const double sp[3] = {0.0, cm_s / scaling, cn_s / scaling};
  const double w1[3] = {w0, wm, wn};
  for (int i = 0; i < 25; ++i) {
    for (int a = 0; a < 2; ++a) {
      const int c = SD2Q25H::code(i, a);
      h.e[i][a] = c < 0 ? -sp[-c] : sp[c];
    }
    const int cx = SD2Q25H::code(i, 0), cy = SD2Q25H::code(i, 1);
    h.w[i] = w1[cx < 0 ? -cx : cx] * w1[cy < 0 ? -cy : cy];
  }
  h.nd = 4;
  h.cls[0] = cm_s;  // dcls order: +c_m, -c_m, +c_n, -c_n
  h.cls[1] = -cm_s;
  h.cls[2] = cn_s;
  h.cls[3] = -cn_s;
  return h;
}

bool get_host_stencil(int id, HostStencil* out, double scaling) {
  switch (id) {
    case NAT_D2Q9: *out = host_stencil<SD2Q9>(scaling); return true;
    case NAT_D3Q19: *out = host_stencil<SD3Q19>(scaling); return true;
    case NAT_D3Q27: *out = host_stencil<SD3Q27>(scaling); return true;
    case NAT_D2Q25H: *out = host_stencil_d2q25h(scaling); return true;
    default: return false;
  }
}

// ---- 1-D Gauss-Lobatto points and Lagrange basis ----------------------------
// Points: the end points and the roots of P_p' (Newton iteration on the
// Legendre ODE, long double), mapped to [0, 1].
void gl_points(int p, double* xi) {
  xi[0] = 0.0;
  xi[p] = 1.0;
  for (int j = 1; j < p; ++j) {
    long double x = -cosl(3.14159265358979323846264338327950288L * j / p);
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1, p1 = x, d0 = 0, d1 = 1;
      for (int k = 2; k <= p; ++k) {
        long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        long double d2 = d0 + (2 * k - 1) * p1;
        p0 = p1; p1 = p2; d0 = d1; d1 = d2;
      }
      long double d2P = (2 * x * d1 - p * (p + 1) * p1) / (1 - x * x);
      long double dx = d1 / d2P;
      x -= dx;
      if (fabsl(dx) < 1e-22L) break;
    }
    xi[j] = (double)((x + 1.0L) / 2.0L);
  }
  for (int j = 1; j < p - j; ++j) {
    double a = 0.5 * (xi[j] + (1.0 - xi[p - j]));
    xi[j] = a;
    xi[p - j] = 1.0 - a;
  }
  if (p % 2 == 0) xi[p / 2] = 0.5;
}

double lagrange(int p, const double* xi, int j, double x) {
  double v = 1.0;
  for (int k = 0; k <= p; ++k)
    if (k != j) v *= (x - xi[k]) / (xi[j] - xi[k]);
  return v;
}

// GL quadrature weights on [0, 1]
void gl_weights(int p, const double* xi, double* wq) {
  for (int j = 0; j <= p; ++j) {
    long double x = 2.0L * xi[j] - 1.0L, p0 = 1, p1 = x;
    for (int k = 2; k <= p; ++k) {
      long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    if (p == 1) p1 = x;
    wq[j] = (double)(1.0L / ((long double)p * (p + 1) * p1 * p1));
  }
}

// ---- tile choice -------------------------------------------------------------
// Cells per tile per axis: divides N, tile extent <= BMAX, tile nodes <= the
// CTA's node slots, shared memory within the opt-in limit.  Prefers the
// largest tile (least halo re-read), then the longest x extent.
bool choose_tiles(nat_solver* s, int prec, int smem_limit) {
  const int D = s->D;
  int best[3] = {1, 1, 1};
  long long best_score = -1;
  std::vector<int> cand[3];
  for (int a = 0; a < 3; ++a) {
    if (a >= D) {
      cand[a].push_back(1);
      continue;
    }
    for (int c = 1; c <= s->spec.cells[a]; ++c)
      if (s->spec.cells[a] % c == 0 && c * s->period <= BMAX) cand[a].push_back(c);
  }
  const int p = s->spec.order;
  for (int cx : cand[0])
    for (int cy : cand[1])
      for (int cz : cand[2]) {
        int B[3] = {cx * s->period, D > 1 ? cy * s->period : 1, D > 2 ? cz * s->period : 1};
        long long TB = (long long)B[0] * B[1] * B[2];
        if (TB > STEP_THREADS * STEP_NPT) continue;
        int Rm[3];
        bool ok = true;
        for (int a = 0; a < 3; ++a) {
          Rm[a] = a < D ? B[a] + 2 * (p + 1) + 2 : 1;  // bound, refined later
          if (Rm[a] > RMAX) ok = false;
        }
        if (!ok) continue;
        if ((long long)step_smem_bytes(prec, Rm, B) > smem_limit) continue;
        long long score = TB * 1000 + B[0];
        if (score > best_score) {
          best_score = score;
          best[0] = cx; best[1] = cy; best[2] = cz;
        }
      }
  if (best_score < 0) return false;
  for (int a = 0; a < 3; ++a) s->B[a] = a < D ? best[a] * s->period : 1;
  return true;
}

// ---- streaming tables --------------------------------------------------------
int build_tables(nat_solver* s, const HostStencil& hs) {
  SLTables& T = s->h_tab;
  memset(&T, 0, sizeof(T));
  const int p = s->spec.order, D = s->D;
  double xi[PMAX1 + 1];
  gl_points(p, xi);
  T.p = p;
  T.dim = D;
  for (int a = 0; a < 3; ++a) {
    AxisGeom& G = T.ax[a];
    if (a >= D) {
      G.n = 1; G.period = 1; G.B = 1; G.ntiles = 1; G.nd = 0;
      T.Rmax[a] = 1;
      continue;
    }
    G.n = s->n_ax[a];
    G.period = s->period;
    G.B = s->B[a];
    G.ntiles = G.n / G.B;
    // displacement classes of the stencil (unit stencils: 0 for e_a > 0,
    // 1 for e_a < 0; D2Q25H: +c_m, -c_m, +c_n, -c_n)
    G.nd = hs.nd;
    int Rmax = G.B;
    for (int d = 0; d < G.nd; ++d) {
      // departure x - dt * e: displacement in cell units
      const double delta = s->dt * hs.cls[d] / s->h[a];
      int lo = 1 << 30, hi = -(1 << 30);
      for (int c = 0; c < G.period; ++c) {
        const double xdep = xi[c] - delta;
        int m;
        if (xdep >= -1e-10 && xdep <= 1.0 + 1e-10)
          m = 0;  // found in the node's own (closed) cell
        else
          m = (int)floor(xdep);
        double xl = xdep - m;
        if (fabs(xl) < 1e-10) xl = 0;
        if (fabs(xl - 1) < 1e-10) xl = 1;
        for (int j = 0; j <= p; ++j) {
          double wv = lagrange(p, xi, j, xl);
          if (fabs(wv) < 1e-10) wv = 0.0;  // SemiLagrangian.cpp:483
          T.w[a][d][c][j] = wv;
          T.wf[a][d][c][j] = (float)wv;
        }
        int jm = 0;
        for (int j = 1; j <= p; ++j)
          if (fabs(T.w[a][d][c][j]) > fabs(T.w[a][d][c][jm])) jm = j;
        T.j0[a][d][c] = jm;
        const int off = m * G.period - c;  // window start relative to the node
        T.off[a][d][c] = off;
        lo = std::min(lo, c + off);
        hi = std::max(hi, c + off);
      }
      G.lo[d] = lo;
      const int hiw = (G.B - G.period) + hi + p;
      G.R[d] = hiw - lo + 1;
      if (G.R[d] > RMAX) return fail(s, NAT_ERR_UNSUPPORTED, "time step too large for the tile halo (axis %d)", a);
      Rmax = std::max(Rmax, G.R[d]);
      for (int o = 0; o < G.B; ++o) T.wst[a][d][o] = o + T.off[a][d][o % G.period] - lo;
    }
    T.Rmax[a] = Rmax;
  }
  return NAT_OK;
}

// ---- conversion / reduction kernels ---------------------------------------

// Layout conversions.  Grid: (chunks of one z plane, z, component); the
// index arithmetic inside a plane is 32-bit (one division by the row length
// per element), which keeps these copies memory-bound.
//   device layout:    [comp][z][y][x], nx * ny * nz per component
//   reference layout: [comp][z][y][x] over rx * ry * rz (FE_Q: the periodic
//                     duplicate layer included, rx <= nx + 1, ...)

__host__ __forceinline__ dim3 plane_grid(long long plane, int planes, int comps) {
  long long gx = (plane + 1023) / 1024;  // 256 threads, about 4 elements each
  if (gx < 1) gx = 1;
  return dim3((unsigned)gx, (unsigned)planes, (unsigned)comps);
}

__device__ __forceinline__ int wrap_once(int v, int n) { return v >= n ? v - n : v; }

// grids of the conversions: over the device lattice (k_upload,
// k_fields_from_ref) and over the reference lattice (k_download,
// k_fields_to_ref)
__host__ __forceinline__ dim3 dev_grid(const Dims& d, int comps) {
  return plane_grid((long long)d.nx * d.ny, d.nz, comps);
}
__host__ __forceinline__ dim3 ref_grid(const Dims& d, int comps) {
  return plane_grid((long long)d.rx * d.ry, d.rz, comps);
}

// reference layout (double) -> device layout
template <class Real>
__global__ void k_upload(const double* __restrict__ src, Real* __restrict__ dst,
                         Dims d, int Q, const double* rest_dev) {
  const int z = blockIdx.y, q = blockIdx.z;
  const int plane = d.nx * d.ny;
  const double* __restrict__ s = src + ((size_t)q * d.rz + z) * ((size_t)d.ry * d.rx);
  Real* __restrict__ o = dst + ((size_t)q * d.nz + z) * (size_t)plane;
  const double rest = sizeof(Real) == 4 ? rest_dev[q] : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x) {
    const int y = i / d.nx, x = i - y * d.nx;
    const double v = s[(size_t)y * d.rx + x];
    if constexpr (sizeof(Real) == 4)
      o[i] = (Real)(v - rest);
    else
      o[i] = (Real)v;
  }
}

// device layout -> reference layout (periodic duplicates filled)
template <class Real>
__global__ void k_download(const Real* __restrict__ src, double* __restrict__ dst,
                           Dims d, int Q, const double* rest_dev) {
  const int zr = blockIdx.y, q = blockIdx.z;
  const int plane = d.rx * d.ry;
  const int z = wrap_once(zr, d.nz);
  const Real* __restrict__ s = src + ((size_t)q * d.nz + z) * ((size_t)d.ny * d.nx);
  double* __restrict__ o = dst + ((size_t)q * d.rz + zr) * (size_t)plane;
  const double rest = sizeof(Real) == 4 ? rest_dev[q] : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x) {
    const int yr = i / d.rx, xr = i - yr * d.rx;
    const double v = (double)s[(size_t)wrap_once(yr, d.ny) * d.nx + wrap_once(xr, d.nx)];
    o[i] = sizeof(Real) == 4 ? v + rest : v;
  }
}

// double fields: device layout <-> reference layout (ncomp blocks)
__global__ void k_fields_to_ref(const double* __restrict__ src, double* __restrict__ dst,
                                Dims d, int ncomp) {
  const int zr = blockIdx.y, q = blockIdx.z;
  const int plane = d.rx * d.ry;
  const int z = wrap_once(zr, d.nz);
  const double* __restrict__ s = src + ((size_t)q * d.nz + z) * ((size_t)d.ny * d.nx);
  double* __restrict__ o = dst + ((size_t)q * d.rz + zr) * (size_t)plane;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x) {
    const int yr = i / d.rx, xr = i - yr * d.rx;
    o[i] = s[(size_t)wrap_once(yr, d.ny) * d.nx + wrap_once(xr, d.nx)];
  }
}

__global__ void k_fields_from_ref(const double* __restrict__ src, double* __restrict__ dst,
                                  Dims d, int ncomp) {
  const int z = blockIdx.y, q = blockIdx.z;
  const int plane = d.nx * d.ny;
  const double* __restrict__ s = src + ((size_t)q * d.rz + z) * ((size_t)d.ry * d.rx);
  double* __restrict__ o = dst + ((size_t)q * d.nz + z) * (size_t)plane;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += gridDim.x * blockDim.x) {
    const int y = i / d.nx, x = i - y * d.nx;
    o[i] = s[(size_t)y * d.rx + x];
  }
}

// FP64 mass / kinetic energy with Gauss-Lobatto node weights (a node on a
// cell face of the FE_Q lattice carries the weights of both cells).
struct QuadW {
  double w[3][PER_MAX];
  int period;
};

__global__ void k_mass_energy(const double* __restrict__ rho, const double* __restrict__ u,
                              Dims d, int D, QuadW qw, const double* __restrict__ node_w, double* out) {
  const long long n = (long long)d.nx * d.ny * d.nz;
  double m = 0, e = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % d.nx);
    const int y = (int)((i / d.nx) % d.ny);
    const int z = (int)(i / ((long long)d.nx * d.ny));
    double wgt = qw.w[0][x % qw.period] * qw.w[1][y % qw.period];
    if (D == 3) wgt *= qw.w[2][z % qw.period];
    if (node_w) wgt = node_w[i];  // mapped cells: per-node weights
    double uu = u[i] * u[i] + u[n + i] * u[n + i];
    if (D == 3) uu += u[2 * n + i] * u[2 * n + i];
    m += wgt * rho[i];
    e += wgt * rho[i] * uu;
  }
  __shared__ double sm[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    m += __shfl_down_sync(0xffffffffu, m, o);
    e += __shfl_down_sync(0xffffffffu, e, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sm[0][wid] = m;
    sm[1][wid] = e;
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    m = lane < nw ? sm[0][lane] : 0.0;
    e = lane < nw ? sm[1][lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      m += __shfl_down_sync(0xffffffffu, m, o);
      e += __shfl_down_sync(0xffffffffu, e, o);
    }
    if (lane == 0) {
      atomicAdd(out, m);
      atomicAdd(out + 1, 0.5 * e);
    }
  }
}

int grid_for(long long work) {
  long long g = (work + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  if (g < 1) g = 1;
  return (int)g;
}

Dims dims_of(const nat_solver* s) {
  Dims d;
  d.nx = s->n_ax[0]; d.ny = s->n_ax[1]; d.nz = s->n_ax[2];
  d.rx = s->n_ref_ax[0]; d.ry = s->n_ref_ax[1]; d.rz = s->n_ref_ax[2];
  return d;
}

StepParams step_params(nat_solver* s, const void* fin, void* fout, int collide,
                       int write_macro, int in_init) {
  StepParams P;
  P.f_in = fin;
  P.f_out = fout;
  P.rho = s->rho;
  P.u = s->u;
  P.status = s->status;
  P.tab = s->d_tab;
  P.n = s->n_dev;
  P.nx = s->n_ax[0];
  P.ny = s->n_ax[1];
  P.nz = s->n_ax[2];
  P.tau = s->tau;
  P.scaling = s->spec.scaling;
  P.write_macro = write_macro;
  P.in_init = in_init;
  P.collide = collide;
  P.force_scheme = s->force_scheme;
  for (int a = 0; a < 3; ++a) P.dF[a] = s->dt * s->force[a] / s->spec.scaling;
  return P;
}

int launch_step(nat_solver* s, const KernelSet& ks, int collide, int write_macro) {
  void* fin = s->f[s->cur];
  void* fout = s->f[1 - s->cur];
  StepParams P = step_params(s, fin, fout, collide, write_macro, 0);
  void* args[] = {&P};
  const void* fn = (s->force_scheme && collide && ks.step_force) ? ks.step_force : ks.step;
  cudaError_t e = cudaLaunchKernel(fn, dim3(s->ntiles), dim3(STEP_THREADS), args,
                                   s->smem_step, s->stream);
  if (e != cudaSuccess) return cuda_fail(s, e, "stream-collide launch");
  s->launches++;
  s->cur = 1 - s->cur;
  return NAT_OK;
}

// Departure-point kernel of a mapped mesh (sl_mapped.cuh): stream (+ collide)
// every node from its rows.
template <class Real>
int launch_mapped_t(nat_solver* s, const void* kern, int collide, int write_macro) {
  StepParams P = step_params(s, s->f[s->cur], s->f[1 - s->cur], collide, write_macro, 0);
  MappedRows<Real> R;
  R.base = s->d_mp_base;
  R.u = static_cast<const Real*>(s->d_mp_u);
  R.cst = static_cast<const Real*>(s->d_mp_c);
  R.flags = s->d_mp_flags;
  for (int a = 0; a < 3; ++a) R.nax[a] = s->n_ax[a];
  LagrangeTab<Real> L;
  memset(&L, 0, sizeof(L));
  double xi[PMAX1 + 1];
  const int p = s->spec.order;
  gl_points(p, xi);
  for (int j = 0; j <= p; ++j) {
    double R = 1.0;
    for (int m = 0; m <= p; ++m)
      if (m != j) R /= xi[j] - xi[m];
    L.xi[j] = (Real)xi[j];
    L.R[j] = (Real)R;
  }
  void* args[] = {&P, &R, &L};
  const long long blocks = (s->n_dev + MAP_THREADS - 1) / MAP_THREADS;
  cudaError_t e = cudaLaunchKernel(kern, dim3((unsigned)blocks), dim3(MAP_THREADS), args, 0, s->stream);
  if (e != cudaSuccess) return cuda_fail(s, e, "departure-point kernel launch");
  s->launches++;
  s->cur = 1 - s->cur;
  return NAT_OK;
}

int launch_mapped(nat_solver* s, bool collide, int write_macro) {
  const void* k = collide ? (s->force_scheme ? s->mp_step_force : s->mp_step) : s->mp_stream;
  if (!k) return fail(s, NAT_ERR_UNSUPPORTED, "no departure-point kernel for this configuration");
  return s->spec.precision == NAT_FP64 ? launch_mapped_t<double>(s, k, collide, write_macro)
                                       : launch_mapped_t<float>(s, k, collide, write_macro);
}

// Decide whether the specialised kernel applies: an instantiation exists for
// (stencil, collision, precision, order, topology), its tile divides the
// mesh, and every departure point lies in the node's own cell or the
// adjacent upwind cell with the dominant weight at the node's own position
// (the compile-time window pattern of Geo<P, DG>).
template <int P, bool DG>
bool pattern_matches(const SLTables& T, int D) {
  using G = Geo<P, DG>;
  for (int a = 0; a < D; ++a) {
    for (int d = 0; d < 2; ++d) {
      const int s = d == 0 ? 1 : -1;
      for (int c = 0; c < G::PER; ++c) {
        const int cell_shift = s > 0 ? (c == 0 ? -1 : 0) : ((DG && c == P) ? 1 : 0);
        if (T.off[a][d][c] != cell_shift * G::PER - c) return false;
        int jm = 0;
        for (int j = 1; j <= P; ++j)
          if (fabs(T.w[a][d][c][j]) > fabs(T.w[a][d][c][jm])) jm = j;
        if (jm != G::J0(s, c)) return false;
      }
    }
  }
  return true;
}

bool pattern_ok(const SLTables& T, int D, int P, bool dg) {
  switch (P * 2 + (dg ? 1 : 0)) {
    case 2 * 1: return pattern_matches<1, false>(T, D);
    case 2 * 1 + 1: return pattern_matches<1, true>(T, D);
    case 2 * 2: return pattern_matches<2, false>(T, D);
    case 2 * 2 + 1: return pattern_matches<2, true>(T, D);
    case 2 * 3: return pattern_matches<3, false>(T, D);
    case 2 * 3 + 1: return pattern_matches<3, true>(T, D);
    case 2 * 4: return pattern_matches<4, false>(T, D);
    case 2 * 4 + 1: return pattern_matches<4, true>(T, D);
    case 2 * 5: return pattern_matches<5, false>(T, D);
    case 2 * 5 + 1: return pattern_matches<5, true>(T, D);
    case 2 * 6: return pattern_matches<6, false>(T, D);
    case 2 * 6 + 1: return pattern_matches<6, true>(T, D);
  }
  return false;
}

void set_v2_weights(nat_solver* s) {
  memset(&s->w64, 0, sizeof(s->w64));
  memset(&s->w32, 0, sizeof(s->w32));
  for (int a = 0; a < 3; ++a)
    for (int d = 0; d < 2; ++d)
      for (int c = 0; c < PER_MAX; ++c)
        for (int j = 0; j < PMAX1; ++j) {
          s->w64.w[a][d][c][j] = s->h_tab.w[a][d][c][j];
          s->w32.w[a][d][c][j] = (float)s->h_tab.w[a][d][c][j];
        }
}

// A specialised fused kernel: the row-segment kernel (sl_row.cuh) or the
// tile kernel (sl_step_v2.cuh).
struct Cand {
  int kind;  // 2 tile, 3 row
  V2Launch v2;
  RowLaunch row;
};

const std::vector<RowLaunch>& row_table() {
  static const std::vector<RowLaunch> t = [] {
    std::vector<RowLaunch> v;
    row_kernels_d2q9(v);
    // the cell-row kernels first, then the row-group and shared-state float
    // variants: preferred when they apply
    cell_kernels(v);
    rowg_kernels_d3q19(v);
    rowg_kernels_d3q27(v);
    row_ss_kernels_d3q19(v);
    row_ss_kernels_d3q27(v);
    row_kernels_d3q19(v);
    row_kernels_d3q27(v);
    rowt_kernels_d3q19(v);
    rowt_kernels_d3q27_bgk(v);
    rowt_kernels_d3q27_kbc(v);
    return v;
  }();
  return t;
}

// Candidate specialised kernels for the current configuration, in order of
// preference (row kernels first).
std::vector<Cand> v2_candidates(nat_solver* s, int coll_sel, int smem_optin) {
  std::vector<Cand> out;
  const bool dg = s->spec.topology == NAT_TOPO_DG;
  if (!pattern_ok(s->h_tab, s->D, s->spec.order, dg)) return out;
  for (const RowLaunch& e : row_table()) {
    if (e.stencil != s->spec.stencil || e.coll != coll_sel || e.prec != s->spec.precision ||
        e.P != s->spec.order || e.dg != dg)
      continue;
    if (s->n_ax[1] % e.wy != 0 || s->n_ax[2] % e.wz != 0) continue;
    if (e.kind == 6 && (s->n_ax[0] % e.align != 0 || s->n_ax[0] < e.min_nx || (long long)e.smem > smem_optin))
      continue;
    if (e.kind == 7 && (s->n_ax[0] > 32 * e.g || s->n_ax[0] <= 32 * (e.g - 1) || s->n_ax[0] < e.min_nx))
      continue;
    if ((e.kind == 11 || e.kind == 12 || e.kind == 13) &&
        (s->n_ax[0] != e.g * (e.dg ? e.P + 1 : e.P) || (long long)e.smem > smem_optin))
      continue;
    // the tensor-core corner form runs only when asked for: it is slower and
    // misses the FP32 path's accuracy (kernel variant 12)
    if (e.kind == 12 && s->variant != 12) continue;
    Cand c;
    c.kind = e.kind;
    c.row = e;
    out.push_back(c);
  }
  for (const V2Launch& e :
       find_v2(s->spec.stencil, coll_sel, s->spec.precision, s->spec.order, dg, s->spec.cells, s->D, s->n_ax[0]))
    if ((long long)e.smem <= smem_optin) {
      Cand c;
      c.kind = 2;
      c.v2 = e;
      out.push_back(c);
    }
  return out;
}

int use_candidate(nat_solver* s, const Cand& c) {
  if (c.kind == 2) {
    cudaError_t ce = cudaFuncSetAttribute(c.v2.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.v2.smem);
    if (ce != cudaSuccess) return cuda_fail(s, ce, "v2 smem attribute");
    s->v2 = c.v2;
  } else {
    if (c.row.smem > 0) {
      cudaError_t ce =
          cudaFuncSetAttribute(c.row.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.row.smem);
      if (ce != cudaSuccess) return cuda_fail(s, ce, "row smem attribute");
    }
    s->row = c.row;
  }
  set_v2_weights(s);
  s->kind = c.kind;
  s->use_v2 = true;
  return NAT_OK;
}

// kernel kind required by a nat_set_kernel_variant value >= 3
int variant_kind(int variant) { return variant == 3 ? 2 : (variant == 4 ? 3 : variant); }

int select_v2(nat_solver* s, int coll_sel, int smem_optin) {
  s->use_v2 = false;
  s->kind = 1;
  if (s->variant == 1) return NAT_OK;
  // a body force runs in the generic kernel only
  if (s->force_scheme)
    return s->variant >= 2 ? fail(s, NAT_ERR_UNSUPPORTED, "with a body force only the generic kernel runs")
                           : NAT_OK;
  std::vector<Cand> all = v2_candidates(s, coll_sel, smem_optin), c;
  for (const Cand& k : all)
    if (s->variant <= 2 || variant_kind(s->variant) == k.kind) c.push_back(k);
  if (c.empty()) {
    if (s->variant >= 2) return fail(s, NAT_ERR_UNSUPPORTED, "no specialised kernel of the requested kind");
    return NAT_OK;
  }
  return use_candidate(s, c.front());
}

int coll_selector(int collision) {
  return collision == NAT_BGK_STANDARD ? L_COLL_BGK
                                       : (collision == NAT_BGK_INCOMPRESSIBLE ? L_COLL_BGK_INC : L_COLL_KBC);
}

template <class Real>
int launch_v2_t(nat_solver* s, const SpecWeights<Real>& W, int write_macro) {
  StepParams2<Real> P;
  P.f_in = static_cast<const Real*>(s->f[s->cur]);
  P.f_out = static_cast<Real*>(s->f[1 - s->cur]);
  P.rho = s->rho;
  P.u = s->u;
  P.status = s->status;
  P.n = s->n_dev;
  P.nx = s->n_ax[0];
  P.ny = s->n_ax[1];
  P.nz = s->n_ax[2];
  P.ntx = s->n_ax[0] / s->v2.B[0];
  P.nty = s->n_ax[1] / s->v2.B[1];
  P.tau = s->tau;
  P.scaling = s->spec.scaling;
  P.write_macro = write_macro;
  P.wait_polls = s->wait_polls;
  P.W = W;
  const int grid = P.ntx * P.nty * (s->n_ax[2] / s->v2.B[2]);
  void* args[] = {&P};
  cudaError_t e = cudaLaunchKernel(s->v2.fn, dim3(grid), dim3(s->v2.nth), args, s->v2.smem, s->stream);
  if (e != cudaSuccess) return cuda_fail(s, e, "specialised stream-collide launch");
  s->launches++;
  s->cur = 1 - s->cur;
  return NAT_OK;
}

template <class Real>
int launch_row_t(nat_solver* s, const SpecWeights<Real>& W, int write_macro) {
  RowParams<Real> P;
  P.f_in = static_cast<const Real*>(s->f[s->cur]);
  P.f_out = static_cast<Real*>(s->f[1 - s->cur]);
  P.rho = s->rho;
  P.u = s->u;
  P.status = s->status;
  P.n = (int)s->n_dev;
  P.nx = s->n_ax[0];
  P.ny = s->n_ax[1];
  P.nz = s->n_ax[2];
  P.nseg = (s->n_ax[0] + 31) / 32;
  P.tau = s->tau;
  P.scaling = s->spec.scaling;
  P.write_macro = write_macro;
  P.wait_polls = s->wait_polls;
  P.W = W;
  int grid = P.nseg * (P.ny / s->row.wy) * (P.nz / s->row.wz);
  int nth = 32 * s->row.wy * s->row.wz;
  if (s->row.kind == 7) {  // row group: g warps per row, wy rows per CTA
    grid = (P.ny / s->row.wy) * P.nz;
    nth = 32 * s->row.g * s->row.wy;
  }
  if (s->row.kind >= 11 && s->row.kind <= 13) {  // cell rows: wy rows per CTA of `warps` warps
    grid = (P.ny / s->row.wy) * P.nz;
    nth = 32 * s->row.warps;
  }
  void* args[] = {&P};
  cudaError_t e = cudaLaunchKernel(s->row.fn, dim3(grid), dim3(nth), args, s->row.smem, s->stream);
  if (e != cudaSuccess) return cuda_fail(s, e, "row stream-collide launch");
  s->launches++;
  s->cur = 1 - s->cur;
  return NAT_OK;
}

int launch_v2(nat_solver* s, int write_macro) {
  if (s->kind == 3 || s->kind == 6 || s->kind == 7 || (s->kind >= 11 && s->kind <= 13))
    return s->spec.precision == NAT_FP64 ? launch_row_t<double>(s, s->w64, write_macro)
                                         : launch_row_t<float>(s, s->w32, write_macro);
  return s->spec.precision == NAT_FP64 ? launch_v2_t<double>(s, s->w64, write_macro)
                                       : launch_v2_t<float>(s, s->w32, write_macro);
}

// ---- compressible two-population model ------------------------------------
// Per-solve constants of the collision, from the reference's stencil formulas.
void fill_thermal_model(nat_solver* s) {
  ThermalModelT<double>& m = s->tm;
  memset(&m, 0, sizeof(m));
  const double sc = s->spec.scaling;
  double cm_s, cn_s, w0, wm, wn;
  d2q25h_speeds(sc, &cm_s, &cn_s);
  d2q25h_weights(&w0, &wm, &wn);
  const double sp[3] = {0.0, cm_s / sc, cn_s / sc};
  const double w1[3] = {w0, wm, wn};
  // unscaled c_s^2 = scaled c_s^2 / scaling^2 (AuxiliaryCollisionFunctions.h:171-172)
  const double c = s->cs2_scaled / (sc * sc);
  m.cs2 = c;
  for (int g = 0; g < TH_NG; ++g) {
    const double X = sp[SD2Q25H::gx(g)], Y = sp[SD2Q25H::gy(g)];
    m.X[g] = X;
    m.Y[g] = Y;
    m.e2[g] = X * X + Y * Y;
    m.w[g] = w1[SD2Q25H::gx(g)] * w1[SD2Q25H::gy(g)];
    m.winv[g] = 1.0 / m.w[g];
    // Hermite tensors at (+X, +Y) (AuxiliaryCollisionFunctions.h:520-566)
    m.h3[g][0] = X * X * X - 3.0 * c * X;
    m.h3[g][1] = X * X * Y - c * Y;
    m.h3[g][2] = X * Y * Y - c * X;
    m.h3[g][3] = Y * Y * Y - 3.0 * c * Y;
    m.h4[g][0] = X * X * X * X - 6.0 * c * X * X + 3.0 * c * c;
    m.h4[g][1] = X * X * X * Y - 3.0 * c * X * Y;
    m.h4[g][2] = X * X * Y * Y - c * (X * X + Y * Y) + c * c;
    m.h4[g][3] = X * Y * Y * Y - 3.0 * c * X * Y;
    m.h4[g][4] = Y * Y * Y * Y - 6.0 * c * Y * Y + 3.0 * c * c;
  }
  m.tau = s->tau;
  m.scaling = sc;
  m.C_v = 1.0 / (s->th.gamma - 1.0);
  m.gfac = 2.0 * m.C_v - s->D;
  m.prandtl = s->th.prandtl;
  m.prandtl_set = s->th.prandtl_set ? 1 : 0;
  m.sutherland_set = s->th.sutherland_set ? 1 : 0;
  m.quartic = s->th.equilibrium == NAT_EQ_QUARTIC ? 1 : 0;
  m.gref = s->gref;
  // float copy for the FP32 deviation form
  ThermalModelT<float>& mf = s->tmf;
  for (int g = 0; g < TH_NG; ++g) {
    mf.X[g] = (float)m.X[g];
    mf.Y[g] = (float)m.Y[g];
    mf.e2[g] = (float)m.e2[g];
    mf.w[g] = (float)m.w[g];
    mf.winv[g] = (float)m.winv[g];
    for (int k = 0; k < 4; ++k) mf.h3[g][k] = (float)m.h3[g][k];
    for (int k = 0; k < 5; ++k) mf.h4[g][k] = (float)m.h4[g][k];
  }
  mf.cs2 = (float)m.cs2;
  mf.tau = (float)m.tau;
  mf.C_v = (float)m.C_v;
  mf.gfac = (float)m.gfac;
  mf.gref = (float)m.gref;
  mf.prandtl = (float)m.prandtl;
  mf.scaling = m.scaling;
  mf.prandtl_set = m.prandtl_set;
  mf.sutherland_set = m.sutherland_set;
  mf.quartic = m.quartic;
}

// Window tables of the two-population row kernel from the operator tables.
int setup_thermal_tables(nat_solver* s) {
  ThermalTablesT<double>& t = s->tt;
  memset(&t, 0, sizeof(t));
  const SLTables& T = s->h_tab;
  t.p = T.p;
  t.per = s->period;
  int lo = 1 << 30, hi = -(1 << 30);
  for (int a = 0; a < 2; ++a)
    for (int d = 0; d < T.ax[a].nd; ++d)
      for (int c = 0; c < s->period; ++c) {
        t.off[a][d][c] = T.off[a][d][c];
        t.j0[a][d][c] = T.j0[a][d][c];
        for (int j = 0; j <= T.p; ++j) t.w[a][d][c][j] = T.w[a][d][c][j];
        if (a == 0) {
          lo = std::min(lo, T.off[0][d][c]);
          hi = std::max(hi, T.off[0][d][c] + T.p);
        }
      }
  t.xl = lo;
  t.bw = 32 + hi - lo;
  const int ny = s->n_ax[1];
  for (int d = 0; d < ND_MAX; ++d)
    for (int c = 0; c < PER_MAX; ++c) t.offy[d][c] = ((t.off[1][d][c] % ny) + ny) % ny;
  if (t.bw > TH_BWMAX)
    return fail(s, NAT_ERR_UNSUPPORTED, "time step too large for the x window of the two-population kernel");
  ThermalTablesT<float>& tf = s->ttf;
  memset(&tf, 0, sizeof(tf));
  for (int a = 0; a < 2; ++a)
    for (int d = 0; d < ND_MAX; ++d)
      for (int c = 0; c < PER_MAX; ++c) {
        tf.off[a][d][c] = t.off[a][d][c];
        tf.j0[a][d][c] = t.j0[a][d][c];
        if (a == 0) tf.offy[d][c] = t.offy[d][c];
        for (int j = 0; j < PMAX1; ++j) tf.w[a][d][c][j] = (float)t.w[a][d][c][j];
      }
  tf.p = t.p;
  tf.per = t.per;
  tf.xl = t.xl;
  tf.bw = t.bw;
  fill_thermal_model(s);
  return NAT_OK;
}

template <class Real>
ThermalStepT<Real> thermal_step_params(nat_solver* s, int write_macro, const ThermalTablesT<Real>& tb,
                                       const ThermalModelT<Real>& M) {
  ThermalStepT<Real> P;
  P.f_in = static_cast<const Real*>(s->f[s->cur]);
  P.g_in = static_cast<const Real*>(s->g[s->cur]);
  P.f_out = static_cast<Real*>(s->f[1 - s->cur]);
  P.g_out = static_cast<Real*>(s->g[1 - s->cur]);
  P.rho = s->rho;
  P.u = s->u;
  P.T = s->T;
  P.mask = s->mask;
  P.status = s->status;
  P.n = (int)s->n_dev;
  P.nx = s->n_ax[0];
  P.ny = s->n_ax[1];
  P.nseg = (s->n_ax[0] + 31) / 32;
  P.write_macro = write_macro;
  P.wall_bits = nullptr;
  P.tb = tb;
  P.M = M;
  return P;
}

template <class Real>
ThermalPointT<Real> thermal_point_params(nat_solver* s, int in_init, const ThermalModelT<Real>& M) {
  ThermalPointT<Real> P;
  P.f = static_cast<Real*>(s->f[s->cur]);
  P.g = static_cast<Real*>(s->g[s->cur]);
  P.rho = s->rho;
  P.u = s->u;
  P.T = s->T;
  P.mask = s->mask;
  P.status = s->status;
  P.n = s->n_dev;
  P.in_init = in_init;
  P.M = M;
  return P;
}

// One fused step of the two-population lattice.  With walls (collide), the
// wall nodes' sparse rows go first into the output buffers and the step kernel
// collides those nodes with the rest (ThermalStepT::wall_bits).
template <class Real>
static cudaError_t thermal_launches(nat_solver* s, ThermalStepT<Real> P, const Real* wrow, bool collide, int form) {
  if (collide && s->d_bn_bits && s->nbn > 0) {
    cudaError_t e = launch_thermal_wall_nodes(P, s->nbn, s->d_bn_node, s->d_br_ptr, s->d_br_col, wrow, s->d_br_c,
                                              false, s->stream);
    if (e != cudaSuccess) return e;
    s->launches++;
    P.wall_bits = s->d_bn_bits;
  }
  return launch_thermal_step(P, collide, s->stream, form);
}

int launch_thermal(nat_solver* s, bool collide, int write_macro) {
  cudaError_t e;
  if (s->spec.precision == NAT_FP64)
    e = thermal_launches(s, thermal_step_params<double>(s, write_macro, s->tt, s->tm), s->d_br_w, collide, 0);
  else
    e = thermal_launches(s, thermal_step_params<float>(s, write_macro, s->ttf, s->tmf), s->d_br_wf, collide,
                         s->th_form);
  if (e != cudaSuccess) return cuda_fail(s, e, "two-population stream-collide launch");
  s->launches++;
  s->cur = 1 - s->cur;
  return NAT_OK;
}

int upload_rest(nat_solver* s) {
  // the rest state is stored after the two doubles of the reduction buffer
  CK(cudaMemcpyAsync(s->red + 2, s->rest, sizeof(double) * s->Q, cudaMemcpyHostToDevice,
                     s->stream), "rest upload");
  return NAT_OK;
}

}  // namespace api
}  // namespace natgpu

using namespace natgpu::api;

// Operator tables of a solve described by spec at time step dt (used by the
// server for its slots).  Requires the compile-time window pattern of the
// row kernel.
int natgpu::build_solver_tables(const nat_spec* spec, double dt, SLTables* T, std::string* err) {
  nat_solver tmp;
  tmp.spec = *spec;
  HostStencil hs;
  if (!get_host_stencil(spec->stencil, &hs, spec->scaling)) return NAT_ERR_UNSUPPORTED;
  tmp.D = hs.D;
  tmp.Q = hs.Q;
  const bool dg = spec->topology == NAT_TOPO_DG;
  tmp.period = dg ? spec->order + 1 : spec->order;
  for (int a = 0; a < 3; ++a) {
    if (a < tmp.D) {
      tmp.n_ax[a] = spec->cells[a] * tmp.period;
      tmp.h[a] = spec->length[a] / spec->cells[a];
      tmp.B[a] = tmp.period;
    }
  }
  tmp.dt = dt;
  int rc = build_tables(&tmp, hs);
  if (rc) {
    if (err) *err = tmp.err;
    return rc;
  }
  if (!pattern_ok(tmp.h_tab, tmp.D, spec->order, dg)) {
    if (err) *err = "time step too large for the row kernel's window pattern";
    return NAT_ERR_UNSUPPORTED;
  }
  *T = tmp.h_tab;
  return NAT_OK;
}

void natgpu::gl_points_host(int p, double* xi) { gl_points(p, xi); }

size_t natgpu::step_smem_bytes(int prec, const int Rmax[3], const int B[3]) {
  return prec == 0 ? smem_layout<double>(Rmax, B).total : smem_layout<float>(Rmax, B).total;
}

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

const char* nat_version(void) { return "natgpu 0.1 (sm_103a)"; }

static int launch_collide(nat_solver* s, int in_init);
static int launch_walls(nat_solver* s);
static int launch_wall_nodes(nat_solver* s, int write_macro);

int nat_destroy(nat_solver* s) {
  if (!s) return NAT_OK;
  // outstanding copies into host memory and from the input staging buffers
  for (int k = 0; k < nat_solver::NTICKET; ++k)
    if (s->tk_ev[k]) {
      cudaEventSynchronize(s->tk_ev[k]);
      cudaEventDestroy(s->tk_ev[k]);
    }
  if (s->h2d) {
    cudaStreamSynchronize(s->h2d);
    cudaStreamDestroy(s->h2d);
  }
  if (s->conv) {
    cudaStreamSynchronize(s->conv);
    cudaStreamDestroy(s->conv);
  }
  if (s->spare_free) cudaEventDestroy(s->spare_free);
  cudaFree(s->f_spare);
  if (s->d2h) {
    cudaStreamSynchronize(s->d2h);
    cudaStreamDestroy(s->d2h);
  }
  for (int k = 0; k < 2; ++k) {
    if (s->rb_done[k]) cudaEventDestroy(s->rb_done[k]);
    cudaFree(s->rb_stage[k]);
  }
  if (s->rb_ready) cudaEventDestroy(s->rb_ready);
  for (int k = 0; k < 2; ++k) {
    if (s->in_free[k]) {
      cudaEventSynchronize(s->in_free[k]);
      cudaEventDestroy(s->in_free[k]);
    }
    if (s->in_full[k]) cudaEventDestroy(s->in_full[k]);
    cudaFree(s->in_stage[k]);
  }
  cudaFreeHost(s->tk_status);
  cudaFree(s->f[0]);
  cudaFree(s->f[1]);
  cudaFree(s->rho);
  cudaFree(s->u);
  cudaFree(s->staging);
  cudaFree(s->red);
  cudaFree(s->status);
  cudaFree(s->d_tab);
  cudaFree(s->g[0]);
  cudaFree(s->g[1]);
  cudaFree(s->T);
  cudaFree(s->mask);
  cudaFree(s->d_br_dst);
  cudaFree(s->d_br_ptr);
  cudaFree(s->d_br_col);
  cudaFree(s->d_br_w);
  cudaFree(s->d_br_wf);
  cudaFree(s->d_br_c);
  cudaFree(s->d_bn_node);
  cudaFree(s->d_bn_bits);
  cudaFree(s->d_mw);
  free_mapped_rows(s);
  delete s;
  return NAT_OK;
}

static int setup_dt(nat_solver* s, double dt) {
  HostStencil hs;
  get_host_stencil(s->spec.stencil, &hs, s->spec.scaling);
  s->dt = dt;
  // tau = nu / (dt c_s^2) + 1/2 with the scaled c_s^2
  // (collision_advanced/AuxiliaryCollisionFunctions.h:63-68, 177)
  s->tau = s->spec.viscosity / (dt * s->cs2_scaled) + 0.5;
  int rc = build_tables(s, hs);
  if (rc) return rc;
  if (s->walls || s->mapped) {
    rc = build_wall_rows(s);
    if (rc) return rc;
  }
  if (s->thermal) return setup_thermal_tables(s);
  int Rm[3] = {s->h_tab.Rmax[0], s->h_tab.Rmax[1], s->h_tab.Rmax[2]};
  s->smem_step = step_smem_bytes(s->spec.precision, Rm, s->B);
  for (const KernelSet* ks : {&s->ks_coll, &s->ks_stream}) {
    if (ks->step) {
      CK(cudaFuncSetAttribute(ks->step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)s->smem_step), "smem attribute");
    }
  }
  s->ntiles = 1;
  for (int a = 0; a < 3; ++a) s->ntiles *= s->h_tab.ax[a].ntiles;
  CK(cudaMemcpyAsync(s->d_tab, &s->h_tab, sizeof(SLTables), cudaMemcpyHostToDevice, s->stream),
     "table upload");
  CK(cudaStreamSynchronize(s->stream), "table upload sync");
  int smem_optin = 0;
  CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device),
     "device attribute");
  return select_v2(s, coll_selector(s->spec.collision), smem_optin);
}

// Device state of a NAT_BGK_COMPRESSIBLE handle: f and g double-buffered,
// rho, u, T, mask; the window tables live in the launch parameters.
static int create_thermal(nat_solver* s, double hmin) {
  const int p = s->spec.order;
  for (int a = 0; a < 3; ++a) s->B[a] = a < s->D ? s->period : 1;
  const size_t es = s->spec.precision == NAT_FP64 ? sizeof(double) : sizeof(float);
  const size_t fbytes = es * (size_t)s->Q * s->n_dev;
#define ALLOC(ptr, bytes)                                             \
  do {                                                                \
    cudaError_t e_ = cudaMalloc((void**)&(ptr), (bytes));             \
    if (e_ != cudaSuccess) {                                          \
      cudaGetLastError();                                             \
      return fail(s, NAT_ERR_OOM, "cudaMalloc(%zu) failed", (size_t)(bytes)); \
    }                                                                 \
  } while (0)
  ALLOC(s->f[0], fbytes);
  ALLOC(s->f[1], fbytes);
  ALLOC(s->g[0], fbytes);
  ALLOC(s->g[1], fbytes);
  ALLOC(s->rho, sizeof(double) * s->n_dev);
  ALLOC(s->u, sizeof(double) * s->D * s->n_dev);
  ALLOC(s->T, sizeof(double) * s->n_dev);
  ALLOC(s->mask, sizeof(double) * s->n_dev);
  ALLOC(s->staging, sizeof(double) * (size_t)s->Q * s->n_ref);
  ALLOC(s->red, sizeof(double) * (2 + 32 + 32));
  ALLOC(s->status, sizeof(int));
  ALLOC(s->d_tab, sizeof(SLTables));
#undef ALLOC
  CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream), "memset");
  CK(cudaMemsetAsync(s->rho, 0, sizeof(double) * s->n_dev, s->stream), "memset");
  CK(cudaMemsetAsync(s->u, 0, sizeof(double) * s->D * s->n_dev, s->stream), "memset");
  CK(cudaMemsetAsync(s->T, 0, sizeof(double) * s->n_dev, s->stream), "memset");
  // deviation reference states of the FP32 form: f - w_i, g - w_i gref
  // (gref: g^eq / f^eq at T = 1 for the default gamma 1.4; fixed per solve)
  s->gref = 2.0 / (1.4 - 1.0) - s->D;
  double grest[32];
  for (int q = 0; q < s->Q; ++q) grest[q] = s->rest[q] * s->gref;
  int rc0 = upload_rest(s);
  if (rc0) return rc0;
  CK(cudaMemcpyAsync(s->red + 2 + 32, grest, sizeof(double) * s->Q, cudaMemcpyHostToDevice, s->stream),
     "g rest upload");
  CK(cudaStreamSynchronize(s->stream), "rest upload sync");
  CK(cudaMemsetAsync(s->mask, 0, sizeof(double) * s->n_dev, s->stream), "memset");
  // SolverConfiguration defaults (solver/SolverConfiguration.cpp:21-31)
  s->th.gamma = 1.4;
  s->th.prandtl = 1.0;
  s->th.prandtl_set = 0;
  s->th.sutherland_set = 0;
  s->th.equilibrium = NAT_EQ_QUARTIC;
  s->kind = 5;
  double dt = s->spec.dt;
  if (!(dt > 0)) dt = s->spec.cfl * hmin / (sqrt(2.0) * s->spec.scaling * p * p);
  return setup_dt(s, dt);
}

int nat_create(const nat_spec* spec, nat_solver** out) {
  if (!spec || !out) return NAT_ERR_INVALID_ARG;
  *out = nullptr;
  nat_solver* s = new nat_solver();
  s->spec = *spec;
  HostStencil hs;
  if (!get_host_stencil(spec->stencil, &hs, spec->scaling)) {
    int rc = fail(s, NAT_ERR_UNSUPPORTED, "unsupported stencil %d", spec->stencil);
    *out = s;
    return rc;
  }
  s->D = hs.D;
  s->Q = hs.Q;
  auto bad = [&](const char* m) {
    fail(s, NAT_ERR_INVALID_ARG, "%s", m);
    *out = s;
    return NAT_ERR_INVALID_ARG;
  };
  if (spec->dim != hs.D) return bad("dim does not match the stencil");
  if (spec->order < 1 || spec->order > PMAX) return bad("order must be 1..6");
  if (spec->topology != NAT_TOPO_FEQ && spec->topology != NAT_TOPO_DG) return bad("bad topology");
  if (spec->precision != NAT_FP64 && spec->precision != NAT_FP32_DEV) return bad("bad precision");
  if (!(spec->scaling > 0) || !(spec->viscosity > 0)) return bad("scaling and viscosity must be > 0");
  for (int a = 0; a < s->D; ++a) {
    if (spec->cells[a] < 1) return bad("cells must be >= 1");
    if (!(spec->length[a] > 0)) return bad("length must be > 0");
    if (!spec->periodic[a]) {
      if (spec->topology != NAT_TOPO_DG) {
        fail(s, NAT_ERR_UNSUPPORTED, "wall boundaries need the DG node topology");
        *out = s;
        return NAT_ERR_UNSUPPORTED;
      }
      // walls default to bounce-back at rest (VelocityNeqBounceBack, u = 0)
      s->walls = true;
      s->bc[2 * a] = s->bc[2 * a + 1] = NAT_BC_VELOCITY_BOUNCE_BACK;
    }
  }
  int coll;
  switch (spec->collision) {
    case NAT_BGK_STANDARD: coll = L_COLL_BGK; break;
    case NAT_BGK_INCOMPRESSIBLE: coll = L_COLL_BGK_INC; break;
    case NAT_KBC_STANDARD: coll = L_COLL_KBC; break;
    case NAT_BGK_COMPRESSIBLE: coll = L_COLL_NONE; break;
    default: return bad("bad collision model");
  }
  s->thermal = spec->collision == NAT_BGK_COMPRESSIBLE;
  if (s->thermal != (spec->stencil == NAT_D2Q25H)) {
    fail(s, NAT_ERR_UNSUPPORTED,
         "the compressible two-population model runs on D2Q25H, and D2Q25H runs only that model");
    *out = s;
    return NAT_ERR_UNSUPPORTED;
  }
  auto pick = [&](int c) -> KernelSet {
    switch (spec->stencil) {
      case NAT_D2Q9: return kernels_d2q9(c, spec->precision);
      case NAT_D3Q19: return kernels_d3q19(c, spec->precision);
      case NAT_D3Q27: return kernels_d3q27(c, spec->precision);
    }
    return KernelSet{};
  };
  if (!s->thermal) {
    s->ks_coll = pick(coll);
    s->ks_stream = pick(L_COLL_NONE);
  }
  if (!s->thermal && spec->vertices) {
    auto mk = [&](int c) -> const void* {
      switch (spec->stencil) {
        case NAT_D2Q9: return mapped_kernel_d2q9(c, spec->precision, spec->order);
        case NAT_D3Q19: return mapped_kernel_d3q19(c, spec->precision, spec->order);
        case NAT_D3Q27: return mapped_kernel_d3q27(c, spec->precision, spec->order);
      }
      return nullptr;
    };
    s->mp_step = mk(coll);
    s->mp_stream = mk(L_COLL_NONE);
    if (coll == L_COLL_BGK) s->mp_step_force = mk(L_COLL_BGK_FORCE);
  }
  if (!s->thermal && !s->ks_coll.step) {
    // the reference throws for these combinations too
    // (collision/BGKIncompressible.cpp:54-55, collision/KBCStandard.cpp:79-81)
    fail(s, NAT_ERR_UNSUPPORTED, "collision model %d is not implemented for stencil %d",
         spec->collision, spec->stencil);
    *out = s;
    return NAT_ERR_UNSUPPORTED;
  }
  const int p = spec->order;
  const bool dg = spec->topology == NAT_TOPO_DG;
  s->period = dg ? p + 1 : p;
  s->n_dev = 1;
  s->n_ref = 1;
  double hmin = 1e300;
  for (int a = 0; a < 3; ++a) {
    if (a < s->D) {
      s->n_ax[a] = spec->cells[a] * s->period;
      s->n_ref_ax[a] = dg ? s->n_ax[a] : s->n_ax[a] + 1;
      s->h[a] = spec->length[a] / spec->cells[a];
      s->pv[a][a] = spec->length[a];
      hmin = std::min(hmin, s->h[a]);
    }
    s->n_dev *= s->n_ax[a];
    s->n_ref *= s->n_ref_ax[a];
  }
  s->cs2_scaled = spec->scaling * spec->scaling / 3.0;
  for (int q = 0; q < s->Q; ++q)
    s->rest[q] = spec->collision == NAT_BGK_INCOMPRESSIBLE ? inc_rest(q) : hs.w[q];
  *out = s;
  // the kernels index one population buffer (Q blocks of n nodes) with 32-bit
  // integers: refuse lattices beyond that before anything is allocated
  if ((long long)s->Q * std::max(s->n_dev, s->n_ref) >= (long long)INT32_MAX)
    return fail(s, NAT_ERR_UNSUPPORTED, "lattice too large: Q x nodes = %lld must stay below 2^31",
                (long long)s->Q * std::max(s->n_dev, s->n_ref));
  s->spec.vertices = nullptr;  // not retained: the grid is copied
  CK(cudaGetDevice(&s->device), "cudaGetDevice");
  if (spec->vertices) {
    int rc = setup_mapping(s, spec->vertices, &hmin);
    if (rc) return rc;
  }
  if (s->thermal) return create_thermal(s, hmin);
  int smem_optin = 0;
  CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device),
     "device attribute");
  if (!choose_tiles(s, spec->precision, smem_optin))
    return fail(s, NAT_ERR_UNSUPPORTED, "no tile shape fits (cells %d %d %d, p %d)",
                spec->cells[0], spec->cells[1], spec->cells[2], p);
  const size_t es = spec->precision == NAT_FP64 ? 8 : 4;
  const size_t fbytes = es * (size_t)s->Q * s->n_dev;
#define ALLOC(ptr, bytes)                                             \
  do {                                                                \
    cudaError_t e_ = cudaMalloc((void**)&(ptr), (bytes));             \
    if (e_ != cudaSuccess) {                                          \
      cudaGetLastError();                                             \
      return fail(s, NAT_ERR_OOM, "cudaMalloc(%zu) failed", (size_t)(bytes)); \
    }                                                                 \
  } while (0)
  ALLOC(s->f[0], fbytes);
  ALLOC(s->f[1], fbytes);
  ALLOC(s->rho, sizeof(double) * s->n_dev);
  ALLOC(s->u, sizeof(double) * s->D * s->n_dev);
  ALLOC(s->staging, sizeof(double) * (size_t)std::max(s->Q, s->D + 1) * s->n_ref);
  ALLOC(s->red, sizeof(double) * (2 + 32));
  ALLOC(s->status, sizeof(int));
  ALLOC(s->d_tab, sizeof(SLTables));
#undef ALLOC
  CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream), "memset");
  CK(cudaMemsetAsync(s->rho, 0, sizeof(double) * s->n_dev, s->stream), "memset");
  CK(cudaMemsetAsync(s->u, 0, sizeof(double) * s->D * s->n_dev, s->stream), "memset");
  int rc = upload_rest(s);
  if (rc) return rc;
  double dt = spec->dt;
  if (!(dt > 0)) {
    // utilities/CFDSolverUtilities.cpp:92-100: |e|_max = sqrt(2) * scaling
    dt = spec->cfl * hmin / (sqrt(2.0) * spec->scaling * p * p);
  }
  return setup_dt(s, dt);
}

int nat_sizes(const nat_solver* s, int64_t* n_ref, int64_t* n_dev, int* Q, int* D) {
  if (!s) return NAT_ERR_INVALID_ARG;
  if (n_ref) *n_ref = s->n_ref;
  if (n_dev) *n_dev = s->n_dev;
  if (Q) *Q = s->Q;
  if (D) *D = s->D;
  return NAT_OK;
}

int nat_get_dt(const nat_solver* s, double* dt, double* tau) {
  if (!s) return NAT_ERR_INVALID_ARG;
  if (dt) *dt = s->dt;
  if (tau) *tau = s->tau;
  return NAT_OK;
}

int nat_set_dt(nat_solver* s, double dt) {
  if (!s) return NAT_ERR_INVALID_ARG;
  if (!(dt > 0)) return fail(s, NAT_ERR_INVALID_ARG, "dt must be > 0");
  return setup_dt(s, dt);
}

int nat_set_stream(nat_solver* s, void* stream) {
  if (!s) return NAT_ERR_INVALID_ARG;
  cudaStream_t ns = (cudaStream_t)stream;
  if (ns != s->stream) {
    // what is enqueued on the old stream (an upload's conversion, a step)
    // comes before anything enqueued on the new one
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "stream switch");
    cudaError_t e = cudaEventRecord(ev, s->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ns, ev, 0);
    cudaEventDestroy(ev);  // released once the recorded work completes
    if (e != cudaSuccess) return cuda_fail(s, e, "stream switch");
  }
  s->stream = ns;
  return NAT_OK;
}

// The copy stream, events and input staging buffers of nat_upload_f.
// Each piece is created once; a call after a failed one creates what is
// still missing (nat_destroy frees whatever exists).
static int ensure_upload_path(nat_solver* s) {
  if (s->h2d) return NAT_OK;
  const size_t bytes = sizeof(double) * (size_t)s->Q * s->n_ref;
  const size_t fbytes = (s->spec.precision == NAT_FP64 ? sizeof(double) : sizeof(float)) * (size_t)s->Q * s->n_dev;
  if (!s->f_spare && cudaMalloc(&s->f_spare, fbytes) != cudaSuccess) {
    cudaGetLastError();
    s->f_spare = nullptr;
    return fail(s, NAT_ERR_OOM, "cudaMalloc(%zu) failed (spare state buffer)", fbytes);
  }
  if (!s->spare_free) {
    CK(cudaEventCreateWithFlags(&s->spare_free, cudaEventDisableTiming), "upload events");
    CK(cudaEventRecord(s->spare_free, s->stream), "upload events");
  }
  if (!s->conv) CK(cudaStreamCreateWithFlags(&s->conv, cudaStreamNonBlocking), "conversion stream");
  for (int k = 0; k < 2; ++k) {
    if (!s->in_stage[k] && cudaMalloc((void**)&s->in_stage[k], bytes) != cudaSuccess) {
      cudaGetLastError();
      s->in_stage[k] = nullptr;
      return fail(s, NAT_ERR_OOM, "cudaMalloc(%zu) failed (input staging)", bytes);
    }
    if (!s->in_full[k]) CK(cudaEventCreateWithFlags(&s->in_full[k], cudaEventDisableTiming), "upload events");
    if (!s->in_free[k]) CK(cudaEventCreateWithFlags(&s->in_free[k], cudaEventDisableTiming), "upload events");
  }
  // last: its presence marks the path complete.  Non-blocking: no implicit
  // ordering against the legacy default stream
  CK(cudaStreamCreateWithFlags(&s->h2d, cudaStreamNonBlocking), "copy stream");
  return NAT_OK;
}

int nat_upload_f(nat_solver* s, const double* f_host) {
  if (!s || !f_host) return NAT_ERR_INVALID_ARG;
  int rc = ensure_upload_path(s);
  if (rc) return rc;
  const int k = s->in_slot;
  // the copy waits for the conversion that last read this staging buffer;
  // the conversion waits for the copy and for the spare's last use
  CK(cudaStreamWaitEvent(s->h2d, s->in_free[k], 0), "upload order");
  CK(cudaMemcpyAsync(s->in_stage[k], f_host, sizeof(double) * s->Q * s->n_ref, cudaMemcpyHostToDevice, s->h2d),
     "upload f");
  CK(cudaEventRecord(s->in_full[k], s->h2d), "upload event");
  CK(cudaStreamWaitEvent(s->conv, s->in_full[k], 0), "upload order");
  CK(cudaStreamWaitEvent(s->conv, s->spare_free, 0), "upload order");
  Dims d = dims_of(s);
  if (s->spec.precision == NAT_FP64)
    k_upload<double><<<dev_grid(d, s->Q), 256, 0, s->conv>>>(s->in_stage[k], (double*)s->f_spare, d, s->Q, s->red + 2);
  else
    k_upload<float><<<dev_grid(d, s->Q), 256, 0, s->conv>>>(s->in_stage[k], (float*)s->f_spare, d, s->Q, s->red + 2);
  CK(cudaGetLastError(), "upload kernel");
  s->launches++;
  CK(cudaEventRecord(s->in_free[k], s->conv), "upload event");
  // the converted state becomes the current one; the previous current
  // buffer is the spare once the work enqueued on the solver stream so far
  // (the steps that read or wrote it) is done
  CK(cudaStreamWaitEvent(s->stream, s->in_free[k], 0), "upload order");
  std::swap(s->f[s->cur], s->f_spare);
  CK(cudaEventRecord(s->spare_free, s->stream), "upload event");
  s->in_slot = 1 - k;
  return NAT_OK;
}

int nat_download_f(nat_solver* s, double* f_host) {
  if (!s || !f_host) return NAT_ERR_INVALID_ARG;
  Dims d = dims_of(s);
  if (s->spec.precision == NAT_FP64)
    k_download<double><<<ref_grid(d, s->Q), 256, 0, s->stream>>>((const double*)s->f[s->cur], s->staging, d, s->Q, s->red + 2);
  else
    k_download<float><<<ref_grid(d, s->Q), 256, 0, s->stream>>>((const float*)s->f[s->cur], s->staging, d, s->Q, s->red + 2);
  CK(cudaGetLastError(), "download kernel");
  s->launches++;
  CK(cudaMemcpyAsync(f_host, s->staging, sizeof(double) * s->Q * s->n_ref,
                     cudaMemcpyDeviceToHost, s->stream), "download f");
  CK(cudaStreamSynchronize(s->stream), "download sync");
  return NAT_OK;
}

// rho and u in the reference layout (staging buffer), then copied to the
// host, all enqueued on the handle's stream.
static int enqueue_macro_readback(nat_solver* s, double* rho_host, double* u_host) {
  Dims d = dims_of(s);
  k_fields_to_ref<<<ref_grid(d, 1), 256, 0, s->stream>>>(s->rho, s->staging, d, 1);
  k_fields_to_ref<<<ref_grid(d, s->D), 256, 0, s->stream>>>(s->u, s->staging + s->n_ref, d, s->D);
  CK(cudaGetLastError(), "macro kernel");
  s->launches += 2;
  CK(cudaMemcpyAsync(rho_host, s->staging, sizeof(double) * s->n_ref, cudaMemcpyDeviceToHost, s->stream),
     "download rho");
  CK(cudaMemcpyAsync(u_host, s->staging + s->n_ref, sizeof(double) * s->D * s->n_ref, cudaMemcpyDeviceToHost,
                     s->stream),
     "download u");
  return NAT_OK;
}

int nat_download_macro(nat_solver* s, double* rho_host, double* u_host) {
  if (!s || !rho_host || !u_host) return NAT_ERR_INVALID_ARG;
  int rc = enqueue_macro_readback(s, rho_host, u_host);
  if (rc) return rc;
  CK(cudaStreamSynchronize(s->stream), "download sync");
  return NAT_OK;
}

// The error of a non-zero device status word: a wait that ran out first (the
// step did not complete), then NaN, then a density below 1e-10.
static int status_error(nat_solver* s, int st) {
  if (st & ST_TIMEOUT)
    return fail(s, NAT_ERR_TIMEOUT, "a wait for a bulk copy ran out; the step is incomplete");
  if (st & ST_NAN) return fail(s, NAT_ERR_NAN, "NaN density in collision");
  return fail(s, NAT_ERR_DENSITY_UNDERFLOW, "Densities too small (< 1e-10) for collisions. Decrease time step size.");
}

int nat_download_macro_async(nat_solver* s, double* rho_host, double* u_host, uint64_t* ticket) {
  if (!s || !rho_host || !u_host || !ticket) return NAT_ERR_INVALID_ARG;
  if (!s->tk_ev[nat_solver::NTICKET - 1]) {  // created last: the ring is complete
    if (!s->tk_status) {
      CK(cudaHostAlloc((void**)&s->tk_status, sizeof(int) * nat_solver::NTICKET, cudaHostAllocDefault),
         "ticket status words");
      memset(s->tk_status, 0, sizeof(int) * nat_solver::NTICKET);
    }
    for (int k = 0; k < nat_solver::NTICKET; ++k)
      if (!s->tk_ev[k]) CK(cudaEventCreateWithFlags(&s->tk_ev[k], cudaEventDisableTiming), "ticket events");
  }
  const unsigned long long t = s->tk_next;
  const int k = (int)(t % nat_solver::NTICKET);
  if (s->tk_held[k]) {
    // the slot's old ticket: wait for it and keep its status for the next wait
    CK(cudaEventSynchronize(s->tk_ev[k]), "ticket reuse");
    s->tk_lost |= s->tk_status[k];
    s->tk_status[k] = 0;
    s->tk_held[k] = 0;
  }
  // read-back stream and staging slots, created on first use
  if (!s->rb_ready) {
    if (!s->d2h) CK(cudaStreamCreateWithFlags(&s->d2h, cudaStreamNonBlocking), "read-back stream");
    for (int b = 0; b < 2; ++b) {
      if (!s->rb_stage[b])
        CK(cudaMalloc((void**)&s->rb_stage[b], sizeof(double) * (1 + s->D) * s->n_ref), "read-back staging");
      if (!s->rb_done[b]) {
        CK(cudaEventCreateWithFlags(&s->rb_done[b], cudaEventDisableTiming), "read-back events");
        CK(cudaEventRecord(s->rb_done[b], s->d2h), "read-back events");
      }
    }
    CK(cudaEventCreateWithFlags(&s->rb_ready, cudaEventDisableTiming), "read-back events");
  }
  const int b = (int)(t & 1);
  // the slot's previous copies must have left it before it is refilled
  CK(cudaStreamWaitEvent(s->stream, s->rb_done[b], 0), "read-back slot reuse");
  Dims d = dims_of(s);
  k_fields_to_ref<<<ref_grid(d, 1), 256, 0, s->stream>>>(s->rho, s->rb_stage[b], d, 1);
  k_fields_to_ref<<<ref_grid(d, s->D), 256, 0, s->stream>>>(s->u, s->rb_stage[b] + s->n_ref, d, s->D);
  CK(cudaGetLastError(), "macro kernel");
  s->launches += 2;
  // the status of the steps since the previous read of it, then cleared
  CK(cudaMemcpyAsync(&s->tk_status[k], s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "status read");
  CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream), "status clear");
  // the copies to the host on the read-back stream, overlapping later steps
  CK(cudaEventRecord(s->rb_ready, s->stream), "read-back event");
  CK(cudaStreamWaitEvent(s->d2h, s->rb_ready, 0), "read-back order");
  CK(cudaMemcpyAsync(rho_host, s->rb_stage[b], sizeof(double) * s->n_ref, cudaMemcpyDeviceToHost, s->d2h),
     "download rho");
  CK(cudaMemcpyAsync(u_host, s->rb_stage[b] + s->n_ref, sizeof(double) * s->D * s->n_ref, cudaMemcpyDeviceToHost,
                     s->d2h),
     "download u");
  CK(cudaEventRecord(s->rb_done[b], s->d2h), "read-back done");
  CK(cudaEventRecord(s->tk_ev[k], s->d2h), "ticket event");
  s->tk_held[k] = t;
  s->tk_next = t + 1;
  *ticket = t;
  return NAT_OK;
}

int nat_wait(nat_solver* s, uint64_t ticket) {
  if (!s) return NAT_ERR_INVALID_ARG;
  if (ticket == 0 || ticket >= s->tk_next) return fail(s, NAT_ERR_INVALID_ARG, "unknown ticket %llu",
                                                       (unsigned long long)ticket);
  const int k = (int)(ticket % nat_solver::NTICKET);
  int st = 0;
  if (s->tk_held[k] == ticket) {
    CK(cudaEventSynchronize(s->tk_ev[k]), "ticket wait");
    st = s->tk_status[k];
    s->tk_status[k] = 0;
  }
  // an older ticket whose slot was reused is complete already; its status,
  // like that of every reused slot nobody waited for, is in tk_lost
  st |= s->tk_lost;
  s->tk_lost = 0;
  return st ? status_error(s, st) : NAT_OK;
}

int nat_upload_macro(nat_solver* s, const double* rho_host, const double* u_host) {
  if (!s || !rho_host || !u_host) return NAT_ERR_INVALID_ARG;
  CK(cudaMemcpyAsync(s->staging, rho_host, sizeof(double) * s->n_ref, cudaMemcpyHostToDevice,
                     s->stream), "upload rho");
  CK(cudaMemcpyAsync(s->staging + s->n_ref, u_host, sizeof(double) * s->D * s->n_ref,
                     cudaMemcpyHostToDevice, s->stream), "upload u");
  Dims d = dims_of(s);
  k_fields_from_ref<<<dev_grid(d, 1), 256, 0, s->stream>>>(s->staging, s->rho, d, 1);
  k_fields_from_ref<<<dev_grid(d, s->D), 256, 0, s->stream>>>(s->staging + s->n_ref, s->u, d, s->D);
  CK(cudaGetLastError(), "macro upload kernel");
  s->launches += 2;
  return NAT_OK;
}

int nat_stream(nat_solver* s, double t, double* dt_out) {
  (void)t;
  if (!s) return NAT_ERR_INVALID_ARG;
  int rc = NAT_OK;
  if (s->mapped && !s->thermal) {
    rc = launch_mapped(s, false, 0);
    if (rc) return rc;
    if (dt_out) *dt_out = s->dt;
    return NAT_OK;
  }
  if (s->mapped) {
    // every row is a sparse row; the rest population stays
    s->cur = 1 - s->cur;
    const size_t es = s->spec.precision == NAT_FP64 ? 8 : 4;
    CK(cudaMemcpyAsync(s->f[s->cur], s->f[1 - s->cur], es * s->n_dev, cudaMemcpyDeviceToDevice, s->stream),
       "rest population");
    if (s->thermal)
      CK(cudaMemcpyAsync(s->g[s->cur], s->g[1 - s->cur], es * s->n_dev, cudaMemcpyDeviceToDevice, s->stream),
         "rest population");
  } else
    rc = s->thermal ? launch_thermal(s, false, 0) : launch_step(s, s->ks_stream, 0, 0);
  if (rc) return rc;
  rc = launch_walls(s);
  if (rc) return rc;
  if (dt_out) *dt_out = s->dt;
  return NAT_OK;
}

int nat_collide(nat_solver* s, int in_init) {
  if (!s) return NAT_ERR_INVALID_ARG;
  int rc = launch_collide(s, in_init);
  if (rc) return rc;
  return nat_status(s);
}

static int launch_collide(nat_solver* s, int in_init) {
  if (s->thermal) {
    if (s->spec.precision == NAT_FP64)
      CK(launch_thermal_collide(thermal_point_params<double>(s, in_init, s->tm), grid_for(s->n_dev), s->stream),
         "two-population collide launch");
    else
      CK(launch_thermal_collide(thermal_point_params<float>(s, in_init, s->tmf), grid_for(s->n_dev), s->stream),
         "two-population collide launch");
    s->launches++;
    return NAT_OK;
  }
  StepParams P = step_params(s, s->f[s->cur], s->f[s->cur], 1, 1, in_init);
  void* args[] = {&P};
  const void* fn = (s->force_scheme && s->ks_coll.collide_force) ? s->ks_coll.collide_force : s->ks_coll.collide;
  CK(cudaLaunchKernel(fn, dim3(grid_for(s->n_dev)), dim3(256), args, 0, s->stream),
     "collide launch");
  s->launches++;
  return NAT_OK;
}

// Fused step of the wall nodes, after the lattice-wide fused kernel of the
// same step (reads the pre-step buffer, overwrites the wall nodes).
static int launch_wall_nodes(nat_solver* s, int write_macro) {
  if ((!s->walls && !s->mapped) || s->nbn == 0) return NAT_OK;
  if (s->thermal && s->d_bn_bits) return NAT_OK;  // collided by the step kernel (launch_thermal)
  if (s->thermal) {
    // the step's buffers: launch_thermal toggled cur, so swap in and out
    cudaError_t e;
    if (s->spec.precision == NAT_FP64) {
      ThermalStepT<double> P = thermal_step_params<double>(s, write_macro, s->tt, s->tm);
      P.f_in = static_cast<const double*>(s->f[1 - s->cur]);
      P.g_in = static_cast<const double*>(s->g[1 - s->cur]);
      P.f_out = static_cast<double*>(s->f[s->cur]);
      P.g_out = static_cast<double*>(s->g[s->cur]);
      e = launch_thermal_wall_nodes(P, s->nbn, s->d_bn_node, s->d_br_ptr, s->d_br_col, s->d_br_w, s->d_br_c,
                                    true, s->stream);
    } else {
      ThermalStepT<float> P = thermal_step_params<float>(s, write_macro, s->ttf, s->tmf);
      P.f_in = static_cast<const float*>(s->f[1 - s->cur]);
      P.g_in = static_cast<const float*>(s->g[1 - s->cur]);
      P.f_out = static_cast<float*>(s->f[s->cur]);
      P.g_out = static_cast<float*>(s->g[s->cur]);
      e = launch_thermal_wall_nodes(P, s->nbn, s->d_bn_node, s->d_br_ptr, s->d_br_col, s->d_br_wf, s->d_br_c,
                                    true, s->stream);
    }
    if (e != cudaSuccess) return cuda_fail(s, e, "two-population wall nodes");
    s->launches += 2;  // rows, then the collision of the nodes
    return NAT_OK;
  }
  // the step's buffers: launch_* toggled cur, so the input is the other one;
  // the rows first (one thread per row), then the nodes' collision
  int rc = launch_wall_rows(s, s->f[1 - s->cur], s->f[s->cur], false);
  if (rc) return rc;
  StepParams P = step_params(s, s->f[1 - s->cur], s->f[s->cur], 1, write_macro, 0);
  void* args[2];
  WallNodes<double> W64;
  WallNodes<float> W32;
  args[0] = &P;
  if (s->spec.precision == NAT_FP64) {
    W64 = {s->nbn, s->d_bn_node};
    args[1] = &W64;
  } else {
    W32 = {s->nbn, s->d_bn_node};
    args[1] = &W32;
  }
  const void* fn = (s->force_scheme && s->ks_coll.wallnode_force) ? s->ks_coll.wallnode_force : s->ks_coll.wallnode;
  CK(cudaLaunchKernel(fn, dim3((s->nbn + 127) / 128), dim3(128), args, 0, s->stream),
     "wall nodes launch");
  s->launches++;
  return NAT_OK;
}

// The wall rows of the buffers just streamed (f, and g for the two-population model).
static int launch_walls(nat_solver* s) {
  if (!s->walls && !s->mapped) return NAT_OK;
  int rc = launch_wall_rows(s, s->f[1 - s->cur], s->f[s->cur], false);
  if (!rc && s->thermal) rc = launch_wall_rows(s, s->g[1 - s->cur], s->g[s->cur], true);
  return rc;
}

int nat_step_async(nat_solver* s, int n_steps, int write_macro) {
  if (!s || n_steps < 0) return NAT_ERR_INVALID_ARG;
  for (int k = 0; k < n_steps; ++k) {
    const int wm = (write_macro && k == n_steps - 1) ? 1 : 0;
    int rc = NAT_OK;
    if (s->mapped && !s->thermal) {
      rc = launch_mapped(s, true, wm);  // every node from its departure-point rows
      if (rc) return rc;
      continue;
    }
    if (s->mapped)
      s->cur = 1 - s->cur;  // every node is stepped from its sparse rows
    else
      rc = s->thermal ? launch_thermal(s, true, wm)
                      : (s->use_v2 ? launch_v2(s, wm) : launch_step(s, s->ks_coll, 1, wm));
    // wall nodes: redone from their sparse rows (fused stream + collide)
    if (!rc && (s->walls || s->mapped)) rc = launch_wall_nodes(s, wm);
    if (rc) return rc;
  }
  return NAT_OK;
}

int nat_step(nat_solver* s, int n_steps) {
  int rc = nat_step_async(s, n_steps, 1);
  if (rc) return rc;
  return nat_status(s);
}

int nat_set_wait_limit(nat_solver* s, uint32_t polls) {
  if (!s) return NAT_ERR_INVALID_ARG;
  s->wait_polls = polls;
  return NAT_OK;
}

int nat_status(nat_solver* s) {
  if (!s) return NAT_ERR_INVALID_ARG;
  int st = 0;
  CK(cudaMemcpyAsync(&st, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "status read");
  CK(cudaStreamSynchronize(s->stream), "status sync");
  if (st) {
    CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream), "status clear");
    return status_error(s, st);
  }
  return NAT_OK;
}

int nat_last_error(const nat_solver* s, char* buf, size_t len) {
  if (!buf || len == 0) return NAT_ERR_INVALID_ARG;
  const char* m = s ? s->err.c_str() : "null handle";
  snprintf(buf, len, "%s", m);
  return NAT_OK;
}

int nat_mass_energy(nat_solver* s, double* mass, double* ke) {
  if (!s) return NAT_ERR_INVALID_ARG;
  QuadW qw;
  memset(&qw, 0, sizeof(qw));
  const int p = s->spec.order;
  double xi[PMAX1 + 1], wq[PMAX1 + 1];
  gl_points(p, xi);
  gl_weights(p, xi, wq);
  qw.period = s->period;
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < s->period; ++c) {
      double w = wq[c];
      if (s->spec.topology == NAT_TOPO_FEQ && c == 0) w += wq[p];  // shared face node
      qw.w[a][c] = a < s->D ? w * s->h[a] : 1.0;
    }
  CK(cudaMemsetAsync(s->red, 0, 2 * sizeof(double), s->stream), "memset");
  k_mass_energy<<<grid_for(s->n_dev), 256, 0, s->stream>>>(s->rho, s->u, dims_of(s), s->D, qw, s->d_mw, s->red);
  CK(cudaGetLastError(), "reduction kernel");
  s->launches++;
  double h2[2];
  CK(cudaMemcpyAsync(h2, s->red, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream), "red read");
  CK(cudaStreamSynchronize(s->stream), "red sync");
  if (mass) *mass = h2[0];
  if (ke) *ke = h2[1];
  return NAT_OK;
}

int nat_device_f(nat_solver* s, void** f_dev) {
  if (!s || !f_dev) return NAT_ERR_INVALID_ARG;
  *f_dev = s->f[s->cur];
  return NAT_OK;
}

int64_t nat_launch_count(const nat_solver* s) { return s ? s->launches : -1; }

int nat_set_kernel_variant(nat_solver* s, int variant) {
  if (!s || variant < 0 || variant > 13 || variant == 5 || (variant >= 8 && variant <= 10)) return NAT_ERR_INVALID_ARG;
  if (s->mapped) {
    if (variant == 0) return NAT_OK;
    return fail(s, NAT_ERR_UNSUPPORTED, "mapped meshes run the departure-point kernel only");
  }
  if (s->thermal) {
    // one kernel serves the two-population model
    if (variant == 0) return NAT_OK;
    return fail(s, NAT_ERR_UNSUPPORTED, "the two-population model has a single fused kernel");
  }
  s->variant = variant;
  int smem_optin = 0;
  CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device),
     "device attribute");
  return select_v2(s, coll_selector(s->spec.collision), smem_optin);
}

// The two-population kernel's forms (sl_thermal.cuh) as kernel variants:
// 0 -> 5 (registers), 1 / 2 -> 9 / 10 (shared memory), 3 -> 14 (registers,
// staged rows); the forms an FP32 handle can choose from (form 3: order 2).
static int th_variant(int form) { return form == 0 ? 5 : (form == 3 ? 14 : 8 + form); }
static int th_forms(const nat_solver* s) { return s->ttf.p == 2 ? 4 : 3; }
static int th_threads(int form) { return 32 * ((form == 1 || form == 2) ? TH_WARPS_SS : TH_WARPS); }

int nat_kernel_variant(const nat_solver* s) {
  if (!s) return -1;
  if (s->mapped && !s->thermal) return 8;
  if (s->thermal) return th_variant(s->th_form);
  return s->use_v2 ? s->kind : 1;
}

// The kernels nat_autotune times, in its order: the specialised candidates
// that apply (filtered by the kernel variant setting), then the generic
// kernel unless a specialised one is required.
static int tune_candidates(nat_solver* s, std::vector<Cand>* cand, int* ncand) {
  int smem_optin = 0;
  CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device),
     "device attribute");
  const int coll_sel = coll_selector(s->spec.collision);
  *cand = s->variant == 1 ? std::vector<Cand>() : v2_candidates(s, coll_sel, smem_optin);
  if (s->variant >= 3) {
    std::vector<Cand> keep;
    for (const Cand& k : *cand)
      if (variant_kind(s->variant) == k.kind) keep.push_back(k);
    cand->swap(keep);
  }
  if (s->force_scheme) cand->clear();  // a body force runs in the generic kernel only
  *ncand = (int)cand->size() + (s->variant >= 2 ? 0 : 1);  // + the generic kernel
  return NAT_OK;
}

int nat_select_candidate(nat_solver* s, int index) {
  if (!s) return NAT_ERR_INVALID_ARG;
  if (s->thermal && s->spec.precision != NAT_FP64 && !s->mapped) {
    if (index < 0 || index >= th_forms(s))
      return fail(s, NAT_ERR_INVALID_ARG, "candidate %d of %d", index, th_forms(s));
    s->th_form = index;
    return NAT_OK;
  }
  if (s->thermal || s->mapped) return index == 0 ? NAT_OK : fail(s, NAT_ERR_INVALID_ARG, "one kernel only");
  std::vector<Cand> cand;
  int ncand = 0;
  int rc = tune_candidates(s, &cand, &ncand);
  if (rc) return rc;
  if (index < 0 || index >= ncand) return fail(s, NAT_ERR_INVALID_ARG, "candidate %d of %d", index, ncand);
  if (index < (int)cand.size()) return use_candidate(s, cand[index]);
  s->use_v2 = false;
  s->kind = 1;
  return NAT_OK;
}

// The two-population fused kernel in FP32: time its forms (three; four at
// order 2, which has the staged form), with f and g backed up in the staging
// buffer (Q n_ref doubles >= 2 Q n_dev floats), and keep the fastest.
static int autotune_thermal(nat_solver* s, int steps, int* n_candidates, int* chosen) {
  const size_t pop = sizeof(float) * (size_t)s->Q * s->n_dev;
  const int cur0 = s->cur, form0 = s->th_form;
  CK(cudaMemcpyAsync(s->staging, s->f[cur0], pop, cudaMemcpyDeviceToDevice, s->stream), "autotune backup");
  CK(cudaMemcpyAsync((char*)s->staging + pop, s->g[cur0], pop, cudaMemcpyDeviceToDevice, s->stream),
     "autotune backup");
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  s->at_ms.clear();
  s->at_desc.clear();
  float best = 1e30f;
  int best_i = -1, rc = NAT_OK;
  for (int form = 0; form < th_forms(s) && !rc; ++form) {
    s->th_form = form;
    rc = nat_step_async(s, 1, 0);
    if (rc) break;
    cudaEventRecord(e0, s->stream);
    rc = nat_step_async(s, steps, 0);
    cudaEventRecord(e1, s->stream);
    if (rc) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = cuda_fail(s, cudaGetLastError(), "autotune sync");
      break;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const int desc[5] = {th_variant(form), 32, 1, 1, th_threads(form)};
    s->at_ms.push_back(ms / steps);
    s->at_desc.insert(s->at_desc.end(), desc, desc + 5);
    if (ms < best) {
      best = ms;
      best_i = form;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s->cur = cur0;
  CK(cudaMemcpyAsync(s->f[cur0], s->staging, pop, cudaMemcpyDeviceToDevice, s->stream), "autotune restore");
  CK(cudaMemcpyAsync(s->g[cur0], (char*)s->staging + pop, pop, cudaMemcpyDeviceToDevice, s->stream),
     "autotune restore");
  CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream), "status clear");
  CK(cudaStreamSynchronize(s->stream), "autotune restore sync");
  if (rc) {
    s->th_form = form0;
    return rc;
  }
  s->th_form = best_i;
  if (n_candidates) *n_candidates = th_forms(s);
  if (chosen) *chosen = best_i;
  return NAT_OK;
}

int nat_autotune(nat_solver* s, int steps, int* n_candidates, int* chosen) {
  if (!s || steps < 1) return NAT_ERR_INVALID_ARG;
  if (s->thermal && s->spec.precision != NAT_FP64 && !s->mapped) return autotune_thermal(s, steps, n_candidates, chosen);
  if (s->thermal || s->mapped) {
    if (n_candidates) *n_candidates = 1;
    if (chosen) *chosen = 0;
    return NAT_OK;
  }
  std::vector<Cand> cand;
  int ncand = 0;
  int rc0 = tune_candidates(s, &cand, &ncand);
  if (rc0) return rc0;
  if (n_candidates) *n_candidates = ncand;
  if (ncand == 0) return fail(s, NAT_ERR_UNSUPPORTED, "no kernel applies");
  // keep the state: back it up in the staging buffer (Q * n_ref doubles >= f)
  const size_t es = s->spec.precision == NAT_FP64 ? 8 : 4;
  const size_t fbytes = es * (size_t)s->Q * s->n_dev;
  const int cur0 = s->cur;
  CK(cudaMemcpyAsync(s->staging, s->f[cur0], fbytes, cudaMemcpyDeviceToDevice, s->stream), "autotune backup");
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  float best = 1e30f;
  int best_i = -1;
  s->at_ms.clear();
  s->at_desc.clear();
  for (int i = 0; i < ncand; ++i) {
    int rc;
    if (i < (int)cand.size()) {
      rc = use_candidate(s, cand[i]);
    } else {
      s->use_v2 = false;
      rc = NAT_OK;
    }
    if (rc) break;
    int desc[5] = {0, 0, 0, 0, 0};
    {
      int tn[3], th = 0;
      int64_t sm = 0;
      nat_kernel_info(s, &desc[0], tn, &th, &sm);
      desc[1] = tn[0];
      desc[2] = tn[1];
      desc[3] = tn[2];
      desc[4] = th;
    }
    rc = nat_step_async(s, 1, 0);  // warm-up
    if (rc) break;
    cudaEventRecord(e0, s->stream);
    rc = nat_step_async(s, steps, 0);
    cudaEventRecord(e1, s->stream);
    if (rc) break;
    CK(cudaEventSynchronize(e1), "autotune sync");
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    s->at_ms.push_back(ms / steps);
    s->at_desc.insert(s->at_desc.end(), desc, desc + 5);
    if (ms < best) {
      best = ms;
      best_i = i;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // restore the state and the status word (the trial steps may have flagged
  // nothing of the caller's)
  s->cur = cur0;
  CK(cudaMemcpyAsync(s->f[cur0], s->staging, fbytes, cudaMemcpyDeviceToDevice, s->stream), "autotune restore");
  CK(cudaMemsetAsync(s->status, 0, sizeof(int), s->stream), "status clear");
  CK(cudaStreamSynchronize(s->stream), "autotune restore sync");
  if (best_i < 0) return fail(s, NAT_ERR_CUDA, "autotune: no candidate ran");
  if (chosen) *chosen = best_i;
  if (best_i < (int)cand.size()) return use_candidate(s, cand[best_i]);
  s->use_v2 = false;
  return NAT_OK;
}

int nat_autotune_report(const nat_solver* s, int max, float* ms_per_step, int* desc) {
  if (!s || max < 0) return -1;
  const int n = (int)s->at_ms.size();
  for (int i = 0; i < n && i < max; ++i) {
    if (ms_per_step) ms_per_step[i] = s->at_ms[i];
    if (desc)
      for (int k = 0; k < 5; ++k) desc[5 * i + k] = s->at_desc[5 * i + k];
  }
  return n;
}

int nat_kernel_info(const nat_solver* s, int* variant, int tile_nodes[3], int* threads, int64_t* smem_bytes) {
  if (!s) return NAT_ERR_INVALID_ARG;
  if (s->mapped && !s->thermal) {
    if (variant) *variant = 8;
    if (tile_nodes) tile_nodes[0] = tile_nodes[1] = tile_nodes[2] = 1;
    if (threads) *threads = 128;
    if (smem_bytes) *smem_bytes = 0;
    return NAT_OK;
  }
  if (s->thermal) {
    if (variant) *variant = nat_kernel_variant(s);
    if (tile_nodes) {
      tile_nodes[0] = 32;
      tile_nodes[1] = 1;
      tile_nodes[2] = 1;
    }
    if (threads) *threads = th_threads(s->th_form);
    if (smem_bytes) *smem_bytes = 0;
    return NAT_OK;
  }
  const int k = s->use_v2 ? s->kind : 1;
  if (variant) *variant = k;
  for (int a = 0; a < 3; ++a) {
    int t = k == 2 ? s->v2.B[a] : s->B[a];
    if (k == 3 || k == 6) t = a == 0 ? 32 : (a == 1 ? s->row.wy : s->row.wz);
    if (k == 7) t = a == 0 ? 32 * s->row.g : (a == 1 ? s->row.wy : 1);
    if (k >= 11 && k <= 13) t = a == 0 ? s->row.g * s->period : (a == 1 ? s->row.wy : 1);
    if (tile_nodes) tile_nodes[a] = t;
  }
  const bool row = k == 3 || k == 6 || k == 7 || (k >= 11 && k <= 13);
  if (threads)
    *threads = k == 2 ? s->v2.nth
                      : (k == 7 ? 32 * s->row.g * s->row.wy
                                : (k >= 11 && k <= 13 ? 32 * s->row.warps
                                                      : (row ? 32 * s->row.wy * s->row.wz : STEP_THREADS)));
  if (smem_bytes) *smem_bytes = (int64_t)(k == 2 ? s->v2.smem : (row ? s->row.smem : s->smem_step));
  return NAT_OK;
}

int nat_set_force(nat_solver* s, int scheme, const double force[3]) {
  if (!s || scheme < NAT_FORCE_NONE || scheme > NAT_FORCE_GUO || (scheme && !force))
    return NAT_ERR_INVALID_ARG;
  if (scheme && (s->thermal || s->spec.collision != NAT_BGK_STANDARD))
    return fail(s, NAT_ERR_UNSUPPORTED, "a body force acts in the BGK_STANDARD collision only");
  if (scheme == NAT_FORCE_GUO && s->spec.stencil != NAT_D2Q9 && s->spec.stencil != NAT_D3Q19)
    return fail(s, NAT_ERR_UNSUPPORTED,
                "the GUO scheme exists for D2Q9 and D3Q19 only (the legacy BGKStandard collision)");
  s->force_scheme = scheme;
  for (int a = 0; a < 3; ++a) s->force[a] = (scheme && a < s->D) ? force[a] : 0.0;
  if (scheme) {
    // the specialised kernels have no force term: the generic kernel runs
    s->use_v2 = false;
    s->kind = 1;
  }
  return NAT_OK;
}

int nat_set_boundary(nat_solver* s, int face, int kind, const double u_wall[3]) {
  if (!s || face < 0 || face >= 2 * s->D) return NAT_ERR_INVALID_ARG;
  if (s->spec.periodic[face / 2])
    return fail(s, NAT_ERR_INVALID_ARG, "face %d belongs to a periodic axis", face);
  if (kind != NAT_BC_VELOCITY_BOUNCE_BACK && kind != NAT_BC_DO_NOTHING)
    return fail(s, NAT_ERR_INVALID_ARG, "unknown boundary kind %d", kind);
  s->bc[face] = kind;
  for (int a = 0; a < 3; ++a) s->uw[face][a] = (u_wall && kind == NAT_BC_VELOCITY_BOUNCE_BACK) ? u_wall[a] : 0.0;
  return build_wall_rows(s);
}

int nat_set_thermal(nat_solver* s, const nat_thermal* t) {
  if (!s || !t) return NAT_ERR_INVALID_ARG;
  if (!s->thermal) return fail(s, NAT_ERR_UNSUPPORTED, "not a NAT_BGK_COMPRESSIBLE handle");
  if (!(t->gamma > 1.0) || !(t->prandtl > 0.0) ||
      (t->equilibrium != NAT_EQ_QUARTIC && t->equilibrium != NAT_EQ_BGK))
    return fail(s, NAT_ERR_INVALID_ARG, "gamma must be > 1, prandtl > 0, equilibrium NAT_EQ_QUARTIC or NAT_EQ_BGK");
  s->th = *t;
  fill_thermal_model(s);
  return NAT_OK;
}

int nat_get_thermal(const nat_solver* s, nat_thermal* t) {
  if (!s || !t) return NAT_ERR_INVALID_ARG;
  if (!s->thermal) return NAT_ERR_UNSUPPORTED;
  *t = s->th;
  return NAT_OK;
}

int nat_upload_g(nat_solver* s, const double* g_host) {
  if (!s || !g_host) return NAT_ERR_INVALID_ARG;
  if (!s->thermal) return fail(s, NAT_ERR_UNSUPPORTED, "not a NAT_BGK_COMPRESSIBLE handle");
  CK(cudaMemcpyAsync(s->staging, g_host, sizeof(double) * s->Q * s->n_ref, cudaMemcpyHostToDevice, s->stream),
     "upload g");
  if (s->spec.precision == NAT_FP64)
    k_upload<double><<<dev_grid(dims_of(s), s->Q), 256, 0, s->stream>>>(s->staging, (double*)s->g[s->cur], dims_of(s), s->Q, s->red + 2 + 32);
  else
    k_upload<float><<<dev_grid(dims_of(s), s->Q), 256, 0, s->stream>>>(s->staging, (float*)s->g[s->cur], dims_of(s), s->Q, s->red + 2 + 32);
  CK(cudaGetLastError(), "upload kernel");
  s->launches++;
  return NAT_OK;
}

int nat_download_g(nat_solver* s, double* g_host) {
  if (!s || !g_host) return NAT_ERR_INVALID_ARG;
  if (!s->thermal) return fail(s, NAT_ERR_UNSUPPORTED, "not a NAT_BGK_COMPRESSIBLE handle");
  if (s->spec.precision == NAT_FP64)
    k_download<double><<<ref_grid(dims_of(s), s->Q), 256, 0, s->stream>>>((const double*)s->g[s->cur], s->staging, dims_of(s), s->Q,
                                                  s->red + 2 + 32);
  else
    k_download<float><<<ref_grid(dims_of(s), s->Q), 256, 0, s->stream>>>((const float*)s->g[s->cur], s->staging, dims_of(s), s->Q,
                                                 s->red + 2 + 32);
  CK(cudaGetLastError(), "download kernel");
  s->launches++;
  CK(cudaMemcpyAsync(g_host, s->staging, sizeof(double) * s->Q * s->n_ref, cudaMemcpyDeviceToHost, s->stream),
     "download g");
  CK(cudaStreamSynchronize(s->stream), "download sync");
  return NAT_OK;
}

int nat_download_thermal(nat_solver* s, double* T_host, double* mask_host) {
  if (!s || !T_host || !mask_host) return NAT_ERR_INVALID_ARG;
  if (!s->thermal) return fail(s, NAT_ERR_UNSUPPORTED, "not a NAT_BGK_COMPRESSIBLE handle");
  Dims d = dims_of(s);
  k_fields_to_ref<<<ref_grid(d, 1), 256, 0, s->stream>>>(s->T, s->staging, d, 1);
  k_fields_to_ref<<<ref_grid(d, 1), 256, 0, s->stream>>>(s->mask, s->staging + s->n_ref, d, 1);
  CK(cudaGetLastError(), "thermal fields kernel");
  s->launches += 2;
  CK(cudaMemcpyAsync(T_host, s->staging, sizeof(double) * s->n_ref, cudaMemcpyDeviceToHost, s->stream),
     "download T");
  CK(cudaMemcpyAsync(mask_host, s->staging + s->n_ref, sizeof(double) * s->n_ref, cudaMemcpyDeviceToHost,
                     s->stream), "download mask");
  CK(cudaStreamSynchronize(s->stream), "download sync");
  return NAT_OK;
}

int nat_init_thermal(nat_solver* s, const double* rho_host, const double* u_host, const double* T_host) {
  if (!s || !rho_host || !u_host || !T_host) return NAT_ERR_INVALID_ARG;
  if (!s->thermal) return fail(s, NAT_ERR_UNSUPPORTED, "not a NAT_BGK_COMPRESSIBLE handle");
  int rc = nat_upload_macro(s, rho_host, u_host);
  if (rc) return rc;
  // the staging buffer is reused once the copies above are done (same stream)
  CK(cudaMemcpyAsync(s->staging + (1 + s->D) * s->n_ref, T_host, sizeof(double) * s->n_ref,
                     cudaMemcpyHostToDevice, s->stream), "upload T");
  k_fields_from_ref<<<dev_grid(dims_of(s), 1), 256, 0, s->stream>>>(s->staging + (1 + s->D) * s->n_ref, s->T,
                                                                     dims_of(s), 1);
  CK(cudaGetLastError(), "T upload kernel");
  s->launches++;
  CK(launch_thermal_init(thermal_point_params<double>(s, 0, s->tm), s->f[s->cur], s->g[s->cur],
                         s->spec.precision != NAT_FP64, grid_for(s->n_dev), s->stream),
     "two-population init launch");
  s->launches++;
  CK(cudaStreamSynchronize(s->stream), "init sync");
  return NAT_OK;
}

}  // extern "C"

// ============================================================================
// Checkpoint and output (the reference's solver/Checkpoint.cpp and the
// solution output of CFDSolver.cpp:1001-1069)
// ============================================================================
