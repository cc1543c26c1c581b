// Host departure-path tracker of libnatgpu.so (restates the tracker of
// SemiLagrangian::fillSparseObject, advection/SemiLagrangian.cpp:145-522):
//  - the face search on Cartesian and on MappingQ1 cells
//    (SemiLagrangian.cpp:525-757), wall hits and periodic translations;
//  - the sparse rows of the wall nodes (k_wall_rows streams them);
//  - the departure-point rows of mapped meshes (sl_mapped.cuh) and the mapped
//    mesh's setup (period vectors, Jacobian quadrature weights).
// The departure-point rows of mapped meshes are searched on the device
// (k_track_rows, one thread per row) with the same tracker functions as the
// host (track.cuh; this file is compiled without floating-point
// contraction, so both give the same rows bit for bit); the host search on
// all host threads remains for wall rows, two-population mapped meshes and
// as the reference the test compares the device rows with.  Runs once per
// time step size.
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
#include "track.cuh"

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

// The tracker's view of a solver (track.cuh), its vertex pointer `vtx` in
// host or device memory.
TrackGeom make_geom(const nat_solver* s, const double* vtx) {
  TrackGeom g;
  memset(&g, 0, sizeof g);
  HostStencil hs;
  get_host_stencil(s->spec.stencil, &hs, s->spec.scaling);
  g.D = s->D;
  g.Q = s->Q;
  g.p = s->spec.order;
  g.PER = s->period;
  g.mapped = s->mapped ? 1 : 0;
  g.n = s->n_dev;
  g.dt = s->dt;
  g.cs2_scaled = s->cs2_scaled;
  gl_points(g.p, g.xi);
  for (int a = 0; a < 3; ++a) {
    g.n_ax[a] = s->n_ax[a];
    g.N[a] = s->spec.cells[a];
    g.periodic[a] = s->spec.periodic[a];
    g.h[a] = s->h[a];
    for (int b = 0; b < 3; ++b) g.pv[a][b] = s->pv[a][b];
  }
  for (int f = 0; f < 6; ++f) {
    g.bc[f] = s->bc[f];
    for (int a = 0; a < 3; ++a) g.uw[f][a] = s->uw[f][a];
  }
  for (int i = 0; i < g.Q; ++i) {
    for (int a = 0; a < 3; ++a) g.es[i][a] = a < g.D ? hs.e[i][a] * s->spec.scaling : 0.0;
    g.w[i] = hs.w[i];
    g.rest[i] = s->rest[i];
  }
  for (int i = 0; i < g.Q; ++i) {
    g.opp[i] = 0;
    for (int j = 0; j < g.Q; ++j)
      if (g.es[j][0] == -g.es[i][0] && g.es[j][1] == -g.es[i][1] && g.es[j][2] == -g.es[i][2]) g.opp[i] = j;
  }
  g.vtx = vtx;
  return g;
}

// the vertex grid alone (cell maps of setup and output)
TrackGeom vertex_geom(const nat_solver* s) {
  TrackGeom g;
  memset(&g, 0, sizeof g);
  g.D = s->D;
  g.mapped = s->mapped ? 1 : 0;
  for (int a = 0; a < 3; ++a) {
    g.N[a] = s->spec.cells[a];
    g.h[a] = s->h[a];
  }
  g.vtx = s->vtx.data();
  return g;
}

const double* grid_vertex(const nat_solver* s, int i, int j, int k) {
  const TrackGeom g = vertex_geom(s);
  return tg_vertex(g, i, j, k);
}

// Position of the node at Gauss-Lobatto point (xi[l0], xi[l1], xi[l2]) of cell c.
void node_point(const nat_solver* s, const int* c, const int* l, const double* xi, double* x) {
  x[0] = x[1] = x[2] = 0.0;
  if (s->mapped) {
    const TrackGeom g = vertex_geom(s);
    double u[3] = {0, 0, 0};
    for (int a = 0; a < s->D; ++a) u[a] = xi[l[a]];
    tg_q1_map(g, c, u, x, nullptr);
    return;
  }
  for (int a = 0; a < s->D; ++a) x[a] = c[a] * s->h[a] + xi[l[a]] * s->h[a];
}

// Departure-point rows of a mapped mesh on the device: one thread per (node,
// direction) row, the same tracker as the host (track.cuh), rows written in
// the solve's arithmetic type.  err[0]: bit 0 an inverse map failed (err[1]
// gets the smallest such row), bit 1 a gathered index left the Q x n state.
template <bool F64>
__global__ void __launch_bounds__(128, 1) k_track_rows(const TrackGeom g, int* __restrict__ base,
                                                       void* __restrict__ uout, void* __restrict__ cout,
                                                       unsigned char* __restrict__ flags, int* __restrict__ err) {
  const long long nr = (long long)(g.Q - 1) * g.n;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < nr;
       r += (long long)gridDim.x * blockDim.x) {
    const int alpha = (int)(r / g.n) + 1;
    const long long node = r % g.n;
    TrackRow R;
    if (tg_row(g, node, alpha, R)) {
      atomicOr(err, 1);
      atomicMin(err + 1, (int)(r < 0x7fffffffLL ? r : 0x7fffffffLL));
      continue;
    }
    // every gathered index must address the Q x n state
    const long long st[3] = {1, g.n_ax[0], (long long)g.n_ax[0] * g.n_ax[1]};
    long long lo = R.base, hi = R.base;
    for (int a = 0; a < g.D; ++a) {
      if (R.flags & (1u << a)) {
        lo += (long long)(g.p - g.n_ax[a]) * st[a];
        hi += (long long)(g.p - 1) * st[a];
      } else {
        hi += (long long)g.p * st[a];
      }
    }
    if (lo < 0 || hi >= (long long)g.Q * g.n) atomicOr(err, 2);
    base[r] = (int)R.base;
    flags[r] = R.flags;
    if constexpr (F64) {
      double* u = static_cast<double*>(uout);
      for (int a = 0; a < g.D; ++a)
        for (int j = 0; j <= g.p; ++j) u[(((long long)(alpha - 1) * g.D + a) * (g.p + 1) + j) * g.n + node] = R.l1[a][j];
      static_cast<double*>(cout)[r] = R.c_plain;
    } else {
      float* u = static_cast<float*>(uout);
      for (int a = 0; a < g.D; ++a) u[((long long)(alpha - 1) * g.D + a) * g.n + node] = (float)R.uu[a];
      static_cast<float*>(cout)[r] = (float)R.c_dev;
    }
  }
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

// Departure-point rows built on the host (already in the device layout and
// type) to the device.
int upload_mapped_rows(nat_solver* s, const std::vector<int>& base, const std::vector<unsigned char>& ub,
                       const std::vector<unsigned char>& cb, const std::vector<unsigned char>& flags) {
  const size_t nr = base.size();
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

// Departure-point rows of every (node, direction) of a mapped mesh, by the
// host tracker on all host threads, into host vectors in the layout of the
// device arrays (FP32: unit coordinates and the deviation-storage constant
// as float; FP64: the 1-D Lagrange values and the plain constant).
int host_mapped_rows(nat_solver* s, std::vector<int>& mp_base, std::vector<unsigned char>& mp_u,
                     std::vector<unsigned char>& mp_c, std::vector<unsigned char>& mp_flags) {
  const TrackGeom g = make_geom(s, s->vtx.data());
  const bool f64 = s->spec.precision == NAT_FP64;
  const int D = s->D, Q = s->Q, p = s->spec.order;
  const long long n = s->n_dev;
  const size_t es = f64 ? 8 : 4, nr = (size_t)(Q - 1) * n;
  mp_base.assign(nr, 0);
  mp_u.assign(nr * D * (f64 ? p + 1 : 1) * es, 0);
  mp_c.assign(nr * es, 0);
  mp_flags.assign(nr, 0);
  struct Err {
    int rc = NAT_OK;
    long long row = -1;
  };
  const int nthr = (int)std::max<long long>(1, std::min<long long>(std::thread::hardware_concurrency(), n / 256));
  std::vector<Err> errs(nthr);
  auto work = [&](long long n0, long long n1, Err& E) {
    for (long long node = n0; node < n1; ++node)
      for (int alpha = 1; alpha < Q; ++alpha) {
        const long long r = (long long)(alpha - 1) * n + node;
        TrackRow R;
        if (tg_row(g, node, alpha, R)) {
          if (E.row < 0 || r < E.row) E.row = r;
          E.rc = NAT_ERR_UNSUPPORTED;
          return;
        }
        mp_base[r] = (int)R.base;
        mp_flags[r] = R.flags;
        if (f64) {
          for (int a = 0; a < D; ++a)
            for (int j = 0; j <= p; ++j)
              memcpy(&mp_u[8 * ((((long long)(alpha - 1) * D + a) * (p + 1) + j) * n + node)], &R.l1[a][j], 8);
          memcpy(&mp_c[8 * r], &R.c_plain, 8);
        } else {
          for (int a = 0; a < D; ++a) {
            const float v = (float)R.uu[a];
            memcpy(&mp_u[4 * (((long long)(alpha - 1) * D + a) * n + node)], &v, 4);
          }
          const float c = (float)R.c_dev;
          memcpy(&mp_c[4 * r], &c, 4);
        }
      }
  };
  {
    std::vector<std::thread> th;
    for (int t = 0; t < nthr; ++t) th.emplace_back(work, n * t / nthr, n * (t + 1) / nthr, std::ref(errs[t]));
    for (auto& t : th) t.join();
  }
  for (const Err& E : errs)
    if (E.rc) {
      TrackRow R;
      tg_row(g, E.row % n, (int)(E.row / n) + 1, R);
      return fail(s, NAT_ERR_UNSUPPORTED,
                  "the inverse map of cell (%d %d %d) failed at a departure point; the mesh is too distorted for "
                  "this time step",
                  R.cell[0], R.cell[1], R.cell[2]);
    }
  // every gathered index must address the Q x n_dev state
  const long long qn = (long long)Q * n;
  const long long st[3] = {1, s->n_ax[0], (long long)s->n_ax[0] * s->n_ax[1]};
  for (size_t r = 0; r < nr; ++r) {
    long long lo = mp_base[r], hi = mp_base[r];
    for (int a = 0; a < D; ++a) {
      if (mp_flags[r] & (1u << a)) {
        lo += (long long)(p - s->n_ax[a]) * st[a];
        hi += (long long)(p - 1) * st[a];
      } else {
        hi += (long long)p * st[a];
      }
    }
    if (lo < 0 || hi >= qn)
      return fail(s, NAT_ERR_CUDA, "internal error: departure-point row %zu addresses %lld..%lld", r, lo, hi);
  }
  return NAT_OK;
}

// The same rows by the device tracker (k_track_rows) into device arrays
// (allocated here); the vertex grid is copied to the device for the call.
int device_mapped_rows(nat_solver* s, int** d_base, void** d_u, void** d_c, unsigned char** d_flags) {
  const bool f64 = s->spec.precision == NAT_FP64;
  const int D = s->D, Q = s->Q, p = s->spec.order;
  const long long n = s->n_dev;
  const size_t es = f64 ? 8 : 4, nr = (size_t)(Q - 1) * n;
  double* d_vtx = nullptr;
  int* d_err = nullptr;
  *d_base = nullptr;
  *d_u = *d_c = nullptr;
  *d_flags = nullptr;
  auto alloc = [&](void** ptr, size_t bytes) -> bool {
    if (cudaMalloc(ptr, bytes) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return true;
  };
  auto release = [&]() {
    cudaFree(d_vtx);
    cudaFree(d_err);
  };
  if (!alloc((void**)&d_vtx, sizeof(double) * s->vtx.size()) || !alloc((void**)&d_err, 2 * sizeof(int)) ||
      !alloc((void**)d_base, sizeof(int) * nr) || !alloc(d_u, nr * D * (f64 ? p + 1 : 1) * es) ||
      !alloc(d_c, nr * es) || !alloc((void**)d_flags, nr)) {
    release();
    cudaFree(*d_base);
    cudaFree(*d_u);
    cudaFree(*d_c);
    cudaFree(*d_flags);
    *d_base = nullptr;
    *d_u = *d_c = nullptr;
    *d_flags = nullptr;
    return fail(s, NAT_ERR_OOM, "cudaMalloc of the departure-point rows failed");
  }
  const TrackGeom g = make_geom(s, d_vtx);
  const int h_err0[2] = {0, 0x7fffffff};
  cudaError_t e = cudaMemcpyAsync(d_vtx, s->vtx.data(), sizeof(double) * s->vtx.size(), cudaMemcpyHostToDevice,
                                  s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_err, h_err0, sizeof(h_err0), cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess) {
    const long long blocks = std::min<long long>(((long long)nr + 127) / 128, 152LL * 16);
    if (f64)
      k_track_rows<true><<<(int)blocks, 128, 0, s->stream>>>(g, *d_base, *d_u, *d_c, *d_flags, d_err);
    else
      k_track_rows<false><<<(int)blocks, 128, 0, s->stream>>>(g, *d_base, *d_u, *d_c, *d_flags, d_err);
    e = cudaGetLastError();
    s->launches++;
  }
  int h_err[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_err, d_err, sizeof(h_err), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  release();
  if (e != cudaSuccess) return cuda_fail(s, e, "device departure-point search");
  if (h_err[0] & 1) {
    const TrackGeom gh = make_geom(s, s->vtx.data());
    TrackRow R;
    tg_row(gh, h_err[1] % n, h_err[1] / n + 1, R);
    return fail(s, NAT_ERR_UNSUPPORTED,
                "the inverse map of cell (%d %d %d) failed at a departure point; the mesh is too distorted for "
                "this time step",
                R.cell[0], R.cell[1], R.cell[2]);
  }
  if (h_err[0] & 2) return fail(s, NAT_ERR_CUDA, "internal error: a departure-point row addresses outside the state");
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
  cudaFree(s->d_bn_bits);
  s->d_bn_bits = nullptr;
  s->d_br_dst = s->d_br_ptr = s->d_br_col = s->d_bn_node = nullptr;
  s->d_br_w = s->d_br_c = nullptr;
  s->d_br_wf = nullptr;
  s->nbr = 0;
  s->nbn = 0;
  free_mapped_rows(s);
  if (!s->walls && !s->mapped) return NAT_OK;
  const long long n = s->n_dev;
  // mapped meshes (one population): departure-point rows of every node
  // (sl_mapped.cuh), searched on the device
  if (s->mapped && !s->thermal) {
    if ((long long)s->Q * n > INT32_MAX) return fail(s, NAT_ERR_UNSUPPORTED, "Q x nodes exceeds 2^31");
    if (s->track_on_host) {
      std::vector<int> base;
      std::vector<unsigned char> u, c, flags;
      int rc = host_mapped_rows(s, base, u, c, flags);
      if (rc) return rc;
      return upload_mapped_rows(s, base, u, c, flags);
    }
    return device_mapped_rows(s, &s->d_mp_base, &s->d_mp_u, &s->d_mp_c, &s->d_mp_flags);
  }
  const TrackGeom g = make_geom(s, s->vtx.data());
  const int D = s->D, Q = s->Q, p = s->spec.order, PER = s->period;
  double grest[32];
  for (int q = 0; q < Q; ++q) grest[q] = s->rest[q] * s->gref;
  // sparse rows of the wall nodes (and of every node of a two-population
  // mapped mesh), node range [n0, n1) into one chunk on a host thread
  struct Chunk {
    std::vector<int> dst, ptr, col, bnodes;
    std::vector<double> w, cst;
    int rc = NAT_OK;
    char err[256] = {0};
  };
  auto work = [&](long long n0, long long n1, Chunk& C) {
    for (long long node = n0; node < n1; ++node) {
      const int idx[3] = {(int)(node % s->n_ax[0]), (int)((node / s->n_ax[0]) % s->n_ax[1]),
                          (int)(node / ((long long)s->n_ax[0] * s->n_ax[1]))};
      int own[3] = {0, 0, 0}, loc[3] = {0, 0, 0};
      for (int a = 0; a < D; ++a) {
        own[a] = idx[a] / PER;
        loc[a] = idx[a] % PER;
      }
      double x[3];
      tg_node_point(g, own, loc, x);
      // a node is a wall node when one of its paths meets a wall; all its rows
      // are then evaluated as sparse rows
      TrackPath paths[32];
      int hits[32];
      bool wall_node = false;
      for (int alpha = 1; alpha < Q; ++alpha) {
        hits[alpha] = tg_trace(g, x, own, alpha, paths[alpha]);
        if (hits[alpha] != 0) wall_node = true;
      }
      if (!wall_node && !s->mapped) continue;
      C.bnodes.push_back((int)node);
      for (int alpha = 1; alpha < Q; ++alpha) {
        const TrackPath& P = paths[alpha];
        const bool identity = hits[alpha] < 0;
        const int sdir = identity ? alpha : P.sdir;
        int cell[3] = {own[0], own[1], own[2]};
        if (!identity)
          for (int a = 0; a < D; ++a) cell[a] = P.cell[a];
        double l1[3][PMAX1];
        for (int a = 0; a < 3; ++a)
          for (int j = 0; j < PMAX1; ++j) l1[a][j] = (a >= D && j == 0) ? 1.0 : 0.0;
        double ud[3] = {0, 0, 0};
        if (!identity && s->mapped && P.udep_ok) {
          for (int a = 0; a < 3; ++a) ud[a] = P.udep[a];
        } else if (!identity && s->mapped && !tg_q1_inverse(g, cell, P.dep, ud)) {
          C.rc = NAT_ERR_UNSUPPORTED;
          snprintf(C.err, sizeof(C.err),
                   "the inverse map of cell (%d %d %d) failed at a departure point; the mesh is too distorted "
                   "for this time step",
                   cell[0], cell[1], cell[2]);
          return;
        }
        for (int a = 0; a < D; ++a) {
          if (identity) {
            cell[a] = own[a];
            for (int j = 0; j <= p; ++j) l1[a][j] = (j == idx[a] % PER) ? 1.0 : 0.0;
            continue;
          }
          double ul = s->mapped ? ud[a] : (P.dep[a] - cell[a] * s->h[a]) / s->h[a];
          if (fabs(ul) < 1e-10) ul = 0.0;
          if (fabs(ul - 1.0) < 1e-10) ul = 1.0;
          for (int j = 0; j <= p; ++j) l1[a][j] = tg_lagrange(p, g.xi, j, ul);
        }
        const int np1 = p + 1;
        const int nloc = D == 3 ? np1 * np1 * np1 : np1 * np1;
        double wrest = 0.0, wgrest = 0.0;
        for (int li = 0; li < nloc; ++li) {
          const int lx = li % np1, ly = (li / np1) % np1, lz = D == 3 ? li / (np1 * np1) : 0;
          const double v = l1[0][lx] * l1[1][ly] * (D == 3 ? l1[2][lz] : 1.0);
          if (fabs(v) < 1e-10) continue;  // SemiLagrangian.cpp:483
          wrest += v * s->rest[sdir];
          wgrest += v * grest[sdir];
          // the FE_Q node p of the last cell of a periodic axis is node 0
          const int ix = (cell[0] * PER + lx) % s->n_ax[0], iy = (cell[1] * PER + ly) % s->n_ax[1],
                    iz = (cell[2] * PER + lz) % s->n_ax[2];
          const long long src = ((long long)iz * s->n_ax[1] + iy) * s->n_ax[0] + ix;
          C.col.push_back((int)(sdir * n + src));
          C.w.push_back(v);
        }
        if (C.col.size() > (size_t)INT32_MAX) {
          C.rc = NAT_ERR_UNSUPPORTED;
          snprintf(C.err, sizeof(C.err), "sparse rows exceed 2^31 entries; use fewer nodes");
          return;
        }
        const double c = P.c;
        C.dst.push_back((int)(alpha * n + node));
        C.ptr.push_back((int)C.col.size());
        C.cst.push_back(c);                           // plain f
        C.cst.push_back(c + wrest - s->rest[alpha]);  // f - w_i storage
        C.cst.push_back(0.0);                         // plain g: no wall term
        C.cst.push_back(wgrest - grest[alpha]);       // g - w_i g_ref storage
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
  if (s->thermal && !s->mapped && !bnodes.empty()) {
    // the two-population step collides the wall nodes itself: mark them per
    // 32-node x segment of a row (node = y nx + x)
    const int nx = s->n_ax[0], nseg = (nx + 31) / 32;
    std::vector<unsigned> bits((size_t)nseg * s->n_ax[1], 0u);
    for (int v : bnodes) {
      const int y = v / nx, x = v % nx;
      if (v < 0 || y >= s->n_ax[1]) return fail(s, NAT_ERR_CUDA, "internal error: wall node %d out of range", v);
      bits[(size_t)y * nseg + x / 32] |= 1u << (x % 32);
    }
    if (cudaMalloc((void**)&s->d_bn_bits, sizeof(unsigned) * bits.size()) != cudaSuccess) {
      cudaGetLastError();
      return fail(s, NAT_ERR_OOM, "cudaMalloc(%zu) failed", sizeof(unsigned) * bits.size());
    }
    CK(cudaMemcpy(s->d_bn_bits, bits.data(), sizeof(unsigned) * bits.size(), cudaMemcpyHostToDevice),
       "wall node bits");
  }
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
  const TrackGeom vg = vertex_geom(s);
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
          tg_q1_map(vg, c, u, x, J);
          if (!(tg_det(D, J) > 0))
            return fail(s, NAT_ERR_INVALID_ARG, "cell (%d %d %d) is inverted or degenerate", cx, cy, cz);
        }
        const int nloc = D == 3 ? np1 * np1 * np1 : np1 * np1;
        for (int li = 0; li < nloc; ++li) {
          const int l[3] = {li % np1, (li / np1) % np1, D == 3 ? li / (np1 * np1) : 0};
          const double u[3] = {xi[l[0]], xi[l[1]], D == 3 ? xi[l[2]] : 0.0};
          double x[3], J[3][3];
          tg_q1_map(vg, c, u, x, J);
          double w = tg_det(D, J);
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

using namespace natgpu::api;

extern "C" int nat_mapped_rows(nat_solver* s, int where, int32_t* base, void* u, void* c, uint8_t* flags) {
  if (!s || (where != 0 && where != 1)) return NAT_ERR_INVALID_ARG;
  if (!s->mapped || s->thermal)
    return fail(s, NAT_ERR_UNSUPPORTED, "departure-point rows exist for mapped one-population meshes only");
  const bool f64 = s->spec.precision == NAT_FP64;
  const size_t es = f64 ? 8 : 4, nr = (size_t)(s->Q - 1) * s->n_dev;
  const size_t ub = nr * s->D * (f64 ? s->spec.order + 1 : 1) * es, cb = nr * es;
  if (where == 0) {
    std::vector<int> b;
    std::vector<unsigned char> uu, cc, fl;
    const int rc = host_mapped_rows(s, b, uu, cc, fl);
    if (rc) return rc;
    if (base) memcpy(base, b.data(), sizeof(int) * nr);
    if (u) memcpy(u, uu.data(), ub);
    if (c) memcpy(c, cc.data(), cb);
    if (flags) memcpy(flags, fl.data(), nr);
    return NAT_OK;
  }
  int* d_base;
  void *d_u, *d_c;
  unsigned char* d_flags;
  int rc = device_mapped_rows(s, &d_base, &d_u, &d_c, &d_flags);
  if (rc == NAT_OK) {
    cudaError_t e = cudaSuccess;
    if (base && e == cudaSuccess) e = cudaMemcpy(base, d_base, sizeof(int) * nr, cudaMemcpyDeviceToHost);
    if (u && e == cudaSuccess) e = cudaMemcpy(u, d_u, ub, cudaMemcpyDeviceToHost);
    if (c && e == cudaSuccess) e = cudaMemcpy(c, d_c, cb, cudaMemcpyDeviceToHost);
    if (flags && e == cudaSuccess) e = cudaMemcpy(flags, d_flags, nr, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_fail(s, e, "departure-point rows read-back");
  }
  cudaFree(d_base);
  cudaFree(d_u);
  cudaFree(d_c);
  cudaFree(d_flags);
  return rc;
}
