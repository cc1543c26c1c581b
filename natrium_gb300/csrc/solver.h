// Internal to libnatgpu.so: the solver handle and the helpers its
// translation units share.
//   natgpu_api.cu  creation, stepping, transfers, reductions, kernel choice;
//   tracker.cu     the host departure-path tracker: wall rows, mapped-mesh
//                  (MappingQ1) rows and mesh setup;
//   io.cu          checkpoint and solution output.
// Not part of the C ABI (include/natgpu.h).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/natgpu.h"
#include "launch.h"
#include "natgpu_common.h"
#include "sl_step_v2.cuh"

struct nat_solver {
  nat_spec spec;
  int D = 0, Q = 0;
  int period = 0;
  int n_ax[3] = {1, 1, 1};      // device lattice per axis
  int n_ref_ax[3] = {1, 1, 1};  // reference layout per axis
  long long n_dev = 0, n_ref = 0;
  double dt = 0, tau = 0, h[3] = {1, 1, 1};
  double cs2_scaled = 0;
  cudaStream_t stream = nullptr;
  int device = 0;
  void* f[2] = {nullptr, nullptr};
  int cur = 0;
  double* rho = nullptr;
  double* u = nullptr;
  double* staging = nullptr;  // Q * n_ref doubles
  double* red = nullptr;      // reduction results (2 doubles)
  int* status = nullptr;
  natgpu::SLTables* d_tab = nullptr;
  natgpu::SLTables h_tab;
  int B[3] = {1, 1, 1};
  int ntiles = 0;
  size_t smem_step = 0;
  natgpu::KernelSet ks_coll, ks_stream;
  std::string err;
  long long launches = 0;
  double rest[32];
  // specialised kernel (sl_step_v2.cuh)
  int variant = 0;  // 0 auto, 1 generic only, 2 specialised required
  bool use_v2 = false;  // a specialised kernel (tile or row) is in use
  int kind = 1;         // 1 generic, 2 tile, 3 row
  natgpu::V2Launch v2;
  natgpu::RowLaunch row;
  natgpu::SpecWeights<double> w64;
  natgpu::SpecWeights<float> w32;
  // compressible two-population model (D2Q25H)
  bool thermal = false;
  nat_thermal th;
  void* g[2] = {nullptr, nullptr};  // second population, same layout and type as f
  double* T = nullptr;              // temperature
  double* mask = nullptr;           // shock sensor (Knudsen estimate)
  double gref = 3.0;                // FP32 deviation storage of g: g - w_i gref
  natgpu::ThermalModelT<double> tm;
  natgpu::ThermalModelT<float> tmf;
  natgpu::ThermalTablesT<double> tt;
  natgpu::ThermalTablesT<float> ttf;
  int th_form = 0;  // fused kernel form: 0 registers, 1 / 2 shared memory (FP32)
  // constant body force (NAT_FORCE_*), F in scaled units
  int force_scheme = 0;
  double force[3] = {0, 0, 0};
  // wall boundaries (non-periodic axes): per face kind and wall velocity, and
  // the rows of the streaming operator whose departure path meets a wall
  bool walls = false;
  int bc[6] = {0, 0, 0, 0, 0, 0};
  double uw[6][3] = {{0}};
  int nbr = 0;                   // boundary rows
  int* d_br_dst = nullptr;       // destination index dir * n_dev + node
  int* d_br_ptr = nullptr;       // nbr + 1 offsets into col / w
  int* d_br_col = nullptr;       // source index dir * n_dev + node
  double* d_br_w = nullptr;      // Lagrange weights (FP64)
  float* d_br_wf = nullptr;      // the same in float
  double* d_br_c = nullptr;      // per row: f const, f const (deviation form), g const, g const (deviation)
  int nbn = 0;                   // wall nodes: nodes with a row that meets a wall; their
  int* d_bn_node = nullptr;      // Q - 1 rows are rows k (Q-1) .. k (Q-1) + Q - 2 above
  unsigned* d_bn_bits = nullptr; // two-population Cartesian lattice: the wall nodes as bits,
                                 // one word per 32-node x segment of a row (ThermalStepT)
  // MappingQ1 cells: every node is a "wall node" (all rows sparse), the
  // Cartesian fused kernels are not used
  bool mapped = false;
  std::vector<double> vtx;       // grid vertices, x fastest, 3 doubles each
  double pv[3][3] = {{0}};       // periodic translation of each axis
  double* d_mw = nullptr;        // per-node quadrature weight (mass / energy)
  // departure-point rows (sl_mapped.cuh), one population only
  int* d_mp_base = nullptr;
  void* d_mp_u = nullptr;        // Real
  void* d_mp_c = nullptr;        // Real
  unsigned char* d_mp_flags = nullptr;
  bool track_on_host = false;    // departure-point rows by the host tracker (else the device's)
  const void* mp_step = nullptr;    // kernels for this stencil / model / order / precision
  const void* mp_stream = nullptr;
  const void* mp_step_force = nullptr;  // BGK with the body-force term
  // report of the last nat_autotune: per candidate ms per step, kind, nodes
  // per CTA along x, y, z and threads per CTA
  std::vector<float> at_ms;
  std::vector<int> at_desc;  // 5 ints per candidate
  // Pipelined host transfers.  nat_upload_f copies into one of two input
  // staging buffers on its own stream (h2d), and a conversion stream turns
  // it into the device layout in a spare state buffer (a third f buffer);
  // the solver's stream waits for the conversion, and the spare and the
  // current buffer swap roles (host-side pointers).  The next copy into the
  // same staging buffer waits for its conversion, and the next conversion
  // into the spare waits for the spare's last use on the solver's stream.
  // So the copy and the conversion of the next state run while the current
  // one is stepped and read back.  Created on first use.
  cudaStream_t h2d = nullptr;
  cudaStream_t conv = nullptr;
  double* in_stage[2] = {nullptr, nullptr};  // Q * n_ref doubles each
  cudaEvent_t in_full[2] = {nullptr, nullptr};
  cudaEvent_t in_free[2] = {nullptr, nullptr};
  int in_slot = 0;
  void* f_spare = nullptr;            // Q * n_dev values (the state's precision)
  cudaEvent_t spare_free = nullptr;   // the spare's last use on the solver stream
  // Asynchronous read-backs (nat_download_macro_async): ticket t uses slot
  // t % NTICKET, an event on the solver's stream and a page-locked copy of
  // the device status word taken right before it.  Reusing a slot first
  // waits for its old ticket and keeps that ticket's status in tk_lost.
  static constexpr int NTICKET = 8;
  cudaEvent_t tk_ev[NTICKET] = {};
  unsigned long long tk_held[NTICKET] = {};  // ticket issued in each slot (0 none)
  int* tk_status = nullptr;                  // page-locked, NTICKET words
  // The device-to-host copies of an asynchronous read-back run on their own
  // stream (d2h) from one of two read-back staging slots (rb_stage, (1 + D)
  // n_ref doubles each), so they overlap the next step on the handle's
  // stream; rb_done[b] marks when slot b's copies have finished.
  cudaStream_t d2h = nullptr;
  double* rb_stage[2] = {nullptr, nullptr};
  cudaEvent_t rb_done[2] = {nullptr, nullptr};
  cudaEvent_t rb_ready = nullptr;
  unsigned long long tk_next = 1;            // next ticket; 0 is never issued
  int tk_lost = 0;
  // limit of each wait of the bulk-copy kernels for a copy (polls of the
  // mbarrier); 0 makes every such wait run out at once
  unsigned wait_polls = natgpu::MBAR_MAX_POLLS;
};

namespace natgpu {
namespace api {

// error text into the handle, returns the code
int fail(nat_solver* s, int code, const char* fmt, ...);
int cuda_fail(nat_solver* s, cudaError_t e, const char* what);

// stencil metadata (host)
struct HostStencil {
  int D, Q;
  double e[32][3];  // unscaled velocities
  double w[32];
  // per-axis displacement classes: count and scaled speed of each (the
  // departure point is x - dt * cls along the axis)
  int nd;
  double cls[ND_MAX];
};

bool get_host_stencil(int id, HostStencil* out, double scaling);
// Gauss-Lobatto points on [0, 1], Lagrange basis value l_j(x), GL weights
void gl_points(int p, double* xi);
double lagrange(int p, const double* xi, int j, double x);
void gl_weights(int p, const double* xi, double* wq);

struct Dims {
  int nx, ny, nz;    // device lattice
  int rx, ry, rz;    // reference lattice
};

// tracker.cu
int build_wall_rows(nat_solver* s);
int launch_wall_rows(nat_solver* s, const void* in, void* out, bool g_pop);
void free_mapped_rows(nat_solver* s);
int setup_mapping(nat_solver* s, const double* vertices, double* hmin);
int host_mapped_rows(nat_solver* s, std::vector<int>& base, std::vector<unsigned char>& u,
                     std::vector<unsigned char>& c, std::vector<unsigned char>& flags);
int device_mapped_rows(nat_solver* s, int** d_base, void** d_u, void** d_c, unsigned char** d_flags);
void node_point(const nat_solver* s, const int* c, const int* l, const double* xi, double* x);

}  // namespace api
}  // namespace natgpu

#define CK(call, what)                              \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_fail(s, e_, what); \
  } while (0)
