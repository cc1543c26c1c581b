// Checkpoint and solution output of libnatgpu.so (the reference's
// Checkpoint.cpp:74-112 and CFDSolver::output, CFDSolver.cpp:1001-1069, in
// the flat forms declared in include/natgpu.h).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "solver.h"

using namespace natgpu;
using namespace natgpu::api;

namespace {

constexpr char CKPT_MAGIC[8] = {'N', 'A', 'T', 'C', 'K', 'P', 'T', '1'};

// Fixed-size header of a checkpoint file; the reference's status file holds
// iteration, time, stencil scaling and FE order (Checkpoint.cpp:74-112).
struct CkptHeader {
  char magic[8];
  int32_t version;
  int32_t stencil, order, topology, collision, precision, Q, D;
  int32_t cells[3];
  int32_t thermal;
  int64_t n_ref;
  int64_t iteration;
  double time, scaling, dt, length[3];
  int32_t mapped;     // MappingQ1 vertex grid and a hash of its bytes
  uint64_t vtx_hash;  // (a resume on a different grid is refused)
};

// FNV-1a over the bytes of the vertex array: exact, and free of the
// floating-point contraction choices a sum would depend on
uint64_t vertex_hash(const nat_solver* s) {
  uint64_t h = 1469598103934665603ull;
  const unsigned char* b = reinterpret_cast<const unsigned char*>(s->vtx.data());
  for (size_t i = 0; i < s->vtx.size() * sizeof(double); ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

}  // namespace

extern "C" {

int nat_checkpoint_save(nat_solver* s, const char* path, int64_t iteration, double time) {
  if (!s || !path) return NAT_ERR_INVALID_ARG;
  CkptHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, CKPT_MAGIC, 8);
  h.version = 2;
  h.stencil = s->spec.stencil;
  h.order = s->spec.order;
  h.topology = s->spec.topology;
  h.collision = s->spec.collision;
  h.precision = s->spec.precision;
  h.Q = s->Q;
  h.D = s->D;
  for (int a = 0; a < 3; ++a) {
    h.cells[a] = s->spec.cells[a];
    h.length[a] = s->spec.length[a];
  }
  h.thermal = s->thermal ? 1 : 0;
  h.n_ref = s->n_ref;
  h.iteration = iteration;
  h.time = time;
  h.scaling = s->spec.scaling;
  h.dt = s->dt;
  h.mapped = s->mapped ? 1 : 0;
  h.vtx_hash = vertex_hash(s);
  std::vector<double> buf((size_t)s->Q * s->n_ref);
  FILE* fp = fopen(path, "wb");
  if (!fp) return fail(s, NAT_ERR_INVALID_ARG, "cannot open %s for writing", path);
  bool ok = fwrite(&h, sizeof(h), 1, fp) == 1;
  int rc = ok ? nat_download_f(s, buf.data()) : NAT_OK;
  if (ok && rc == NAT_OK) ok = fwrite(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
  if (ok && rc == NAT_OK && s->thermal) {
    rc = nat_download_g(s, buf.data());
    if (rc == NAT_OK) ok = fwrite(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
  }
  if (fclose(fp) != 0) ok = false;
  if (rc != NAT_OK) return rc;
  if (!ok) return fail(s, NAT_ERR_INVALID_ARG, "writing %s failed", path);
  return NAT_OK;
}

int nat_checkpoint_load(nat_solver* s, const char* path, int64_t* iteration, double* time) {
  if (!s || !path) return NAT_ERR_INVALID_ARG;
  FILE* fp = fopen(path, "rb");
  if (!fp) return fail(s, NAT_ERR_INVALID_ARG, "cannot open %s", path);
  CkptHeader h;
  if (fread(&h, sizeof(h), 1, fp) != 1 || memcmp(h.magic, CKPT_MAGIC, 8) != 0 || h.version != 2) {
    fclose(fp);
    return fail(s, NAT_ERR_INVALID_ARG, "%s is not a checkpoint of this library", path);
  }
  // the lattice must be the same; the reference likewise refuses a changed
  // FE order or stencil scaling (Checkpoint.cpp:126-160)
  const char* what = nullptr;
  if (h.stencil != s->spec.stencil || h.Q != s->Q || h.D != s->D) what = "stencil";
  else if (h.order != s->spec.order || h.topology != s->spec.topology) what = "FE order or node topology";
  else if (h.n_ref != s->n_ref || h.cells[0] != s->spec.cells[0] || h.cells[1] != s->spec.cells[1] ||
           h.cells[2] != s->spec.cells[2]) what = "lattice";
  else if (h.thermal != (s->thermal ? 1 : 0)) what = "collision model (one or two populations)";
  else if (h.scaling != s->spec.scaling) what = "stencil scaling";
  else if (h.mapped != (s->mapped ? 1 : 0) || h.vtx_hash != vertex_hash(s)) what = "vertex grid";
  if (what) {
    fclose(fp);
    return fail(s, NAT_ERR_INVALID_ARG, "checkpoint %s: different %s", path, what);
  }
  std::vector<double> buf((size_t)s->Q * s->n_ref);
  bool ok = fread(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
  int rc = ok ? nat_upload_f(s, buf.data()) : NAT_OK;
  if (ok && rc == NAT_OK && s->thermal) {
    ok = fread(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
    if (ok) rc = nat_upload_g(s, buf.data());
  }
  fclose(fp);
  if (rc != NAT_OK) return rc;
  if (!ok) return fail(s, NAT_ERR_INVALID_ARG, "checkpoint %s is truncated", path);
  if (iteration) *iteration = h.iteration;
  if (time) *time = h.time;
  CK(cudaStreamSynchronize(s->stream), "checkpoint upload sync");
  return NAT_OK;
}

int nat_write_vtu(nat_solver* s, const char* path) {
  if (!s || !path) return NAT_ERR_INVALID_ARG;
  const int D = s->D, p = s->spec.order;
  const bool dg = s->spec.topology == NAT_TOPO_DG;
  const long long n = s->n_ref;
  std::vector<double> rho(n), u((size_t)D * n), T, mask;
  int rc = nat_download_macro(s, rho.data(), u.data());
  if (rc) return rc;
  if (s->thermal) {
    T.resize(n);
    mask.resize(n);
    rc = nat_download_thermal(s, T.data(), mask.data());
    if (rc) return rc;
  }
  double xi[PMAX1 + 1];
  gl_points(p, xi);
  // node coordinates per axis, reference layout (Cartesian box)
  std::vector<double> ax[3];
  for (int a = 0; a < 3; ++a) {
    if (a >= D) {
      ax[a].assign(1, 0.0);
      continue;
    }
    const double h = s->h[a];
    for (int c = 0; c < s->spec.cells[a]; ++c)
      for (int l = 0; l < (dg ? p + 1 : p); ++l) ax[a].push_back(c * h + xi[l] * h);
    if (!dg) ax[a].push_back(s->spec.cells[a] * h);
  }
  const int nr[3] = {(int)ax[0].size(), (int)ax[1].size(), (int)ax[2].size()};
  // sub-cells: neighbouring nodes inside each finite-element cell (p^D per cell)
  std::vector<long long> conn;
  auto nid = [&](int i, int j, int k) { return ((long long)k * nr[1] + j) * nr[0] + i; };
  const int stride = dg ? p + 1 : p;
  long long ncell = 0;
  for (int cz = 0; cz < (D == 3 ? s->spec.cells[2] : 1); ++cz)
    for (int cy = 0; cy < s->spec.cells[1]; ++cy)
      for (int cx = 0; cx < s->spec.cells[0]; ++cx)
        for (int lz = 0; lz < (D == 3 ? p : 1); ++lz)
          for (int ly = 0; ly < p; ++ly)
            for (int lx = 0; lx < p; ++lx) {
              const int i = cx * stride + lx, j = cy * stride + ly, k = D == 3 ? cz * stride + lz : 0;
              conn.push_back(nid(i, j, k));
              conn.push_back(nid(i + 1, j, k));
              conn.push_back(nid(i + 1, j + 1, k));
              conn.push_back(nid(i, j + 1, k));
              if (D == 3) {
                conn.push_back(nid(i, j, k + 1));
                conn.push_back(nid(i + 1, j, k + 1));
                conn.push_back(nid(i + 1, j + 1, k + 1));
                conn.push_back(nid(i, j + 1, k + 1));
              }
              ++ncell;
            }
  FILE* fp = fopen(path, "w");
  if (!fp) return fail(s, NAT_ERR_INVALID_ARG, "cannot open %s for writing", path);
  const int nv = D == 3 ? 8 : 4;
  fprintf(fp, "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
  fprintf(fp, "<UnstructuredGrid>\n<Piece NumberOfPoints=\"%lld\" NumberOfCells=\"%lld\">\n", n, ncell);
  fprintf(fp, "<Points>\n<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n");
  for (int k = 0; k < nr[2]; ++k)
    for (int j = 0; j < nr[1]; ++j)
      for (int i = 0; i < nr[0]; ++i) {
        if (!s->mapped) {
          fprintf(fp, "%.17g %.17g %.17g\n", ax[0][i], ax[1][j], ax[2][k]);
          continue;
        }
        // mapped cell: the cell map at the node's Gauss-Lobatto point
        const int ii[3] = {i, j, k};
        int c[3] = {0, 0, 0}, l[3] = {0, 0, 0};
        for (int a = 0; a < D; ++a) {
          if (dg) {
            c[a] = ii[a] / (p + 1);
            l[a] = ii[a] % (p + 1);
          } else {
            c[a] = std::min(ii[a] / p, s->spec.cells[a] - 1);
            l[a] = ii[a] - c[a] * p;
          }
        }
        double x[3];
        node_point(s, c, l, xi, x);
        fprintf(fp, "%.17g %.17g %.17g\n", x[0], x[1], x[2]);
      }
  fprintf(fp, "</DataArray>\n</Points>\n<Cells>\n<DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">\n");
  for (size_t q = 0; q < conn.size(); ++q) fprintf(fp, "%lld%c", conn[q], (q % nv == (size_t)nv - 1) ? '\n' : ' ');
  fprintf(fp, "</DataArray>\n<DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">\n");
  for (long long c = 1; c <= ncell; ++c) fprintf(fp, "%lld\n", c * nv);
  fprintf(fp, "</DataArray>\n<DataArray type=\"UInt8\" Name=\"types\" format=\"ascii\">\n");
  for (long long c = 0; c < ncell; ++c) fprintf(fp, "%d\n", D == 3 ? 12 : 9);  // VTK_HEXAHEDRON / VTK_QUAD
  fprintf(fp, "</DataArray>\n</Cells>\n<PointData Scalars=\"rho\">\n");
  auto field = [&](const char* name, const double* v) {
    fprintf(fp, "<DataArray type=\"Float64\" Name=\"%s\" format=\"ascii\">\n", name);
    for (long long i = 0; i < n; ++i) fprintf(fp, "%.17g\n", v[i]);
    fprintf(fp, "</DataArray>\n");
  };
  field("rho", rho.data());
  const char* un[3] = {"ux", "uy", "uz"};
  for (int a = 0; a < D; ++a) field(un[a], u.data() + (size_t)a * n);
  if (s->thermal) {
    field("T", T.data());
    field("shock_sensor", mask.data());
  }
  fprintf(fp, "</PointData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n");
  if (fclose(fp) != 0) return fail(s, NAT_ERR_INVALID_ARG, "writing %s failed", path);
  return NAT_OK;
}

}  // extern "C"
