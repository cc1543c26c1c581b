// Continuous-batching server for independent 2-D semi-Lagrangian solves.
//
// Requests (D2Q9, BGK or KBC, FE_Q order 1-6, any cell count, own Ma / Re /
// step count) are admitted by their HBM footprint into slots of a device
// memory pool; every live solve advances one time step per server step.  A
// server step is one CUDA graph: one kernel per (order, collision) group of
// the live solves, as parallel branches, each specialised for its order and
// model and walking its part of a device work list of (slot, row, 32-node
// segment) items with the row body of sl_row.cuh.  The step counter lives in
// device memory and the last CTA of the step advances it, so the graph needs
// no separate tick.  Admissions and retirements rebuild the work list
// (uploaded asynchronously from double-buffered page-locked memory) and the
// graph; steps in between relaunch the same graph.  A solve's last step
// writes rho / u; the host copies them out after an event and frees the slot.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <chrono>
#include <deque>
#include <map>
#include <string>
#include <vector>

#include "../../include/natgpu.h"
#include "launch.h"
#include "sl_row.cuh"

using namespace natgpu;

namespace {

constexpr int SERVE_WARPS = 8;  // warps per CTA of the batched kernel
constexpr int SERVE_MINB = 3;   // resident CTAs per SM it is compiled for

struct SlotDesc {
  float* f[2];  // ping-pong distribution buffers (FP32 deviation)
  double* rho;
  double* u;
  int* status;
  int n, nx, ny, nseg;
  int P, coll;
  int active;
  long long start_step;  // server step at admission (step parity origin)
  long long last_step;   // server step of the solve's final step
  double tau, scaling;
  float W[3][2][PER_MAX][PMAX1];
};

struct WorkItem {
  int slot, row, seg;
};

template <int P, int COLL>
__device__ __forceinline__ void serve_item(const SlotDesc& d, const float* sw, float* buf, float* fs, int row,
                                           int seg, int lane, long long step) {
  const int par = (int)((step - d.start_step) & 1);
  RowArgs<float> a;
  a.f_in = d.f[par];
  a.f_out = d.f[1 - par];
  a.rho = d.rho;
  a.u = d.u;
  a.status = d.status;
  a.n = d.n;
  a.nx = d.nx;
  a.ny = d.ny;
  a.nz = 1;
  a.tau = d.tau;
  a.scaling = d.scaling;
  a.write_macro = step == d.last_step;
  row_body<SD2Q9, float, COLL, P, false, true>(a, sw, buf, row, 0, seg * 32, lane, fs);
  __syncwarp();
}

// group g = (order - 1) * 2 + (collision is KBC)
constexpr int NGROUPS = 2 * PMAX;
__host__ __device__ constexpr int serve_group(int P, int coll) { return (P - 1) * 2 + (coll == COLL_KBC ? 1 : 0); }

struct GroupRange {
  int begin, count;  // items of the group in the work list
};

// The batched step of one (order, collision) group.  Each warp takes a
// contiguous chunk of the group's items (items of one solve are adjacent, so
// the weight table of the solve is filled once per chunk, not per item).
// The CTA that finishes last among all CTAs of the step's kernels
// (total_ctas, counted on *ticket) advances the device step counter: every
// CTA has read the counter before that.
// The streamed values of a segment wait in the warp's shared array (the row
// kernel's shared-state form): at most 80 registers, three resident CTAs
// per SM (24 warps) instead of two at 128.
template <int P, int COLL>
__global__ void __launch_bounds__(32 * SERVE_WARPS, SERVE_MINB)
    k_serve_group(const SlotDesc* __restrict__ slots, const WorkItem* __restrict__ work,
                  const GroupRange* __restrict__ groups, long long* step_ctr, unsigned* ticket,
                  unsigned total_ctas) {
  constexpr int TAB = row_table_size<P, false>();
  constexpr int BW = 32 + P + P + 1;
  __shared__ float s_tab[SERVE_WARPS][TAB];
  __shared__ float s_buf[SERVE_WARPS][2 * (BW + 1)];
  __shared__ float s_fs[SERVE_WARPS][SD2Q9::Q * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const GroupRange gr = groups[serve_group(P, COLL)];
  const long long step = *step_ctr;
  const int nwarps = gridDim.x * SERVE_WARPS;
  const int chunk = (gr.count + nwarps - 1) / nwarps;
  const int w0 = (blockIdx.x * SERVE_WARPS + warp) * chunk;
  const int w1 = min(w0 + chunk, gr.count);
  int cur = -1;
  for (int w = w0; w < w1; ++w) {
    const WorkItem it = work[gr.begin + w];
    const SlotDesc& d = slots[it.slot];
    if (!d.active || step > d.last_step) continue;
    if (it.slot != cur) {
      __syncwarp();
      fill_row_table<float, P, false>(s_tab[warp], d.W, lane, 32);
      __syncwarp();
      cur = it.slot;
    }
    serve_item<P, COLL>(d, s_tab[warp], s_buf[warp], s_fs[warp], it.row, it.seg, lane, step);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned t = atomicAdd(ticket, 1u);
    if (t == total_ctas - 1) {
      *ticket = 0u;
      *step_ctr = step + 1;
      __threadfence();
    }
  }
}

using GroupKernel = void (*)(const SlotDesc*, const WorkItem*, const GroupRange*, long long*, unsigned*, unsigned);

GroupKernel group_kernel(int g) {
  switch (g) {
#define NAT_SERVE_G(PP)                                         \
  case serve_group(PP, COLL_BGK): return k_serve_group<PP, COLL_BGK>; \
  case serve_group(PP, COLL_KBC): return k_serve_group<PP, COLL_KBC>;
    NAT_SERVE_G(1)
    NAT_SERVE_G(2)
    NAT_SERVE_G(3)
    NAT_SERVE_G(4)
    NAT_SERVE_G(5)
    NAT_SERVE_G(6)
#undef NAT_SERVE_G
    default: return nullptr;
  }
}

// Equilibrium initial state of one slot (CFDSolver::initializeDistributions,
// EQUILIBRIUM option, solver/CFDSolver.cpp:1103-1130), FE_Q lattice with the
// periodic duplicates folded.  kind 0: Taylor-Green vortex
// (benchmarks/TaylorGreenVortex2D.cpp:36-59), 1: double shear layer
// (benchmarks/ShearLayer2D.cpp:39-53).
struct InitArgs {
  float* f;
  int n, nx, ny, P, kind;
  double hx, hy, Lx, Ly, scaling, Ma, u0, kappa, delta;
  double xi[PMAX1 + 1];
};

__global__ void k_serve_init(InitArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int ix = i % a.nx, iy = i / a.nx;
  const double x = ((ix / a.P) + a.xi[ix % a.P]) * a.hx;
  const double y = ((iy / a.P) + a.xi[iy % a.P]) * a.hy;
  double rho, ux, uy;  // scaled velocity
  if (a.kind == 0) {
    const double kx = 2.0 * M_PI / a.Lx, ky = 2.0 * M_PI / a.Ly;
    ux = a.u0 * sin(kx * x) * cos(ky * y);
    uy = -a.u0 * cos(kx * x) * sin(ky * y);
    rho = 1.0 + a.Ma * a.Ma * 0.25 * (cos(2.0 * kx * x) + cos(2.0 * ky * y));
  } else {
    const double yy = y / a.Ly, xx = x / a.Lx;
    ux = a.u0 * (yy <= 0.5 ? tanh(a.kappa * (yy - 0.25)) : tanh(a.kappa * (0.75 - yy)));
    uy = a.delta * a.u0 * sin(2.0 * M_PI * (xx + 0.25));
    rho = 1.0;
  }
  const double u = ux / a.scaling, v = uy / a.scaling;
  const double uu = 1.5 * (u * u + v * v);
  for (int q = 0; q < 9; ++q) {
    const double ue = 3.0 * (SD2Q9::e(q, 0) * u + SD2Q9::e(q, 1) * v);
    const double w = SD2Q9::w(q);
    const double feq = w * rho * (1.0 + ue * (1.0 + 0.5 * ue) - uu);
    a.f[(size_t)q * a.n + i] = (float)(feq - w);
  }
}

// first-fit allocator over the device pool (offsets in bytes)
struct Pool {
  std::map<size_t, size_t> free_;  // offset -> size
  size_t used = 0;
  void init(size_t bytes) {
    free_.clear();
    free_[0] = bytes;
    used = 0;
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = (bytes + 255) & ~size_t(255);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes;
        const size_t o = it->first;
        free_.erase(it);
        if (rest) free_[o + bytes] = rest;
        used += bytes;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    used -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

struct Live {
  int64_t id;
  int slot;
  size_t off, bytes;
  long long last_step;
};

struct Completing {
  Live live;
  cudaEvent_t ev;
  std::vector<double> rho, u;
  int status;
};

}  // namespace

struct nat_server {
  cudaStream_t stream = nullptr;
  int device = 0;
  char* pool_base = nullptr;
  size_t pool_bytes = 0;
  Pool pool;
  int max_slots = 0;
  SlotDesc* d_slots = nullptr;
  std::vector<SlotDesc> h_slots;
  std::vector<int> slot_used;
  WorkItem* d_work = nullptr;
  GroupRange* d_groups = nullptr;
  long long* d_step = nullptr;
  unsigned* d_ticket = nullptr;
  int* d_status = nullptr;  // one per slot
  int max_work = 0;
  int group_count[NGROUPS] = {};
  // page-locked staging of the work list, group ranges and slot table, two
  // sets used in turn; an event marks when a set's copies have been read
  // a ring of NSTAGE page-locked staging sets for the work list uploads: a
  // set is refilled once its copies (an event) are done, which with several
  // sets rarely waits even when the device runs many steps behind
  static constexpr int NSTAGE = 8;
  WorkItem* stage_work[NSTAGE] = {};
  GroupRange* stage_groups[NSTAGE] = {};
  SlotDesc* stage_slots[NSTAGE] = {};
  int stage_cap[NSTAGE] = {};
  cudaEvent_t stage_ev[NSTAGE] = {};
  int stage_k = 0;
  // bound on the host running ahead of the device: an event every
  // RUNAHEAD_EVERY steps in a ring of RUNAHEAD_RING
  cudaEvent_t ahead_ev[4] = {nullptr, nullptr, nullptr, nullptr};
  bool ahead_used[4] = {false, false, false, false};
  int ahead_k = 0;
  unsigned graph_ctas = 0;
  int graph_nodes = 0;
  int sms = 0;
  std::deque<std::pair<int64_t, nat_request>> pending;
  std::vector<Live> live;
  std::vector<Completing*> completing;
  std::map<int64_t, Completing*> done;
  long long host_step = 0;
  int64_t next_id = 1;
  bool dirty = true;
  // the step graph, its template and kernel nodes (one per non-empty group,
  // graph_mask); a new live set with the same non-empty groups updates the
  // nodes' grids and arguments in place instead of instantiating again
  cudaGraphExec_t graph = nullptr;
  cudaGraph_t graph_tmpl = nullptr;
  cudaGraphNode_t gnodes[NGROUPS] = {};
  unsigned graph_mask = 0;
  bool graph_stale = true;
  long long graph_builds = 0, graph_updates = 0, rebuild_ns = 0;
  std::string err;
  // statistics
  long long steps_run = 0, node_updates = 0, launches = 0;
  double* h_stage = nullptr;  // pinned staging for results
  size_t h_stage_bytes = 0;
};

namespace {

int sfail(nat_server* s, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (s) s->err = buf;
  return code;
}

#define SCK(call, what)                                                         \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) return sfail(s, NAT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_)); \
  } while (0)

size_t footprint(const nat_request& r, int* nx, int* ny) {
  *nx = r.cells[0] * r.order;
  *ny = r.cells[1] * r.order;
  const size_t n = (size_t)(*nx) * (*ny);
  return 2 * 9 * n * sizeof(float) + 3 * n * sizeof(double);
}

int validate(nat_server* s, const nat_request& r) {
  if (r.stencil != NAT_D2Q9) return sfail(s, NAT_ERR_UNSUPPORTED, "the server runs D2Q9 solves");
  if (r.collision != NAT_BGK_STANDARD && r.collision != NAT_KBC_STANDARD)
    return sfail(s, NAT_ERR_UNSUPPORTED, "the server runs BGK or KBC");
  if (r.order < 1 || r.order > PMAX) return sfail(s, NAT_ERR_INVALID_ARG, "order must be 1..6");
  if (r.cells[0] < 1 || r.cells[1] < 1) return sfail(s, NAT_ERR_INVALID_ARG, "cells must be >= 1");
  if (!(r.length[0] > 0) || !(r.length[1] > 0)) return sfail(s, NAT_ERR_INVALID_ARG, "length must be > 0");
  if (!(r.scaling > 0) || !(r.viscosity > 0)) return sfail(s, NAT_ERR_INVALID_ARG, "scaling, viscosity > 0");
  if (r.steps < 1) return sfail(s, NAT_ERR_INVALID_ARG, "steps must be >= 1");
  if (r.init != NAT_INIT_TAYLOR_GREEN && r.init != NAT_INIT_SHEAR_LAYER)
    return sfail(s, NAT_ERR_INVALID_ARG, "unknown initial state");
  return NAT_OK;
}

constexpr int RUNAHEAD_EVERY = 16;
constexpr int RUNAHEAD_RING = 4;

// rebuild the device work list from the live slots, grouped by (order,
// collision); uploaded asynchronously from one of the two staging sets
int upload_state(nat_server* s) {
  std::vector<WorkItem> per[NGROUPS];
  for (const Live& L : s->live) {
    const SlotDesc& d = s->h_slots[L.slot];
    std::vector<WorkItem>& v = per[serve_group(d.P, d.coll)];
    for (int y = 0; y < d.ny; ++y)
      for (int g = 0; g < d.nseg; ++g) v.push_back({L.slot, y, g});
  }
  int nw = 0;
  for (int g = 0; g < NGROUPS; ++g) nw += (int)per[g].size();
  if (nw > s->max_work) {
    // in-flight steps may still read the old list: drain them first (rare)
    SCK(cudaStreamSynchronize(s->stream), "work list drain");
    cudaFree(s->d_work);
    s->max_work = nw * 2;
    SCK(cudaMalloc(&s->d_work, sizeof(WorkItem) * s->max_work), "work list");
  }
  const int k = s->stage_k;
  SCK(cudaEventSynchronize(s->stage_ev[k]), "staging reuse");  // its last copies are done
  if (nw > s->stage_cap[k]) {
    cudaFreeHost(s->stage_work[k]);
    s->stage_cap[k] = nw * 2;
    SCK(cudaHostAlloc(&s->stage_work[k], sizeof(WorkItem) * s->stage_cap[k], cudaHostAllocDefault), "staging");
  }
  int off = 0;
  for (int g = 0; g < NGROUPS; ++g) {
    s->stage_groups[k][g] = {off, (int)per[g].size()};
    s->group_count[g] = (int)per[g].size();
    if (!per[g].empty()) memcpy(s->stage_work[k] + off, per[g].data(), sizeof(WorkItem) * per[g].size());
    off += (int)per[g].size();
  }
  memcpy(s->stage_slots[k], s->h_slots.data(), sizeof(SlotDesc) * s->max_slots);
  if (nw)
    SCK(cudaMemcpyAsync(s->d_work, s->stage_work[k], sizeof(WorkItem) * nw, cudaMemcpyHostToDevice, s->stream),
        "work upload");
  SCK(cudaMemcpyAsync(s->d_groups, s->stage_groups[k], sizeof(GroupRange) * NGROUPS, cudaMemcpyHostToDevice,
                      s->stream),
      "group upload");
  SCK(cudaMemcpyAsync(s->d_slots, s->stage_slots[k], sizeof(SlotDesc) * s->max_slots, cudaMemcpyHostToDevice,
                      s->stream),
      "slot upload");
  SCK(cudaEventRecord(s->stage_ev[k], s->stream), "staging event");
  s->stage_k = (k + 1) % nat_server::NSTAGE;
  s->dirty = false;
  s->graph_stale = true;  // the groups or their sizes changed
  return NAT_OK;
}

// The step graph of the live set: a kernel node per non-empty group, no
// dependencies between them (independent solves), each with a grid of about
// one item per warp (a short serial chain per step), at most SERVE_MINB CTAs
// per SM.  When the set of non-empty
// groups is the one the graph was built for, the nodes' grids and the CTA
// total are updated in the instantiated graph; otherwise it is built anew.
int capture(nat_server* s) {
  int grid[NGROUPS] = {};
  unsigned total = 0, mask = 0;
  for (int g = 0; g < NGROUPS; ++g) {
    if (!s->group_count[g]) continue;
    const int want = (s->group_count[g] + SERVE_WARPS - 1) / SERVE_WARPS;  // one item per warp
    grid[g] = want < 1 ? 1 : (want > SERVE_MINB * s->sms ? SERVE_MINB * s->sms : want);
    total += (unsigned)grid[g];
    mask |= 1u << g;
  }
  if (!total) return NAT_OK;
  void* args[] = {(void*)&s->d_slots, (void*)&s->d_work, (void*)&s->d_groups, (void*)&s->d_step,
                  (void*)&s->d_ticket, (void*)&total};
  auto params = [&](int g) {
    cudaKernelNodeParams kp;
    memset(&kp, 0, sizeof kp);
    kp.func = (void*)group_kernel(g);
    kp.gridDim = dim3(grid[g]);
    kp.blockDim = dim3(32 * SERVE_WARPS);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    return kp;
  };
  if (s->graph && mask == s->graph_mask) {
    bool ok = true;
    for (int g = 0; g < NGROUPS && ok; ++g) {
      if (!grid[g]) continue;
      const cudaKernelNodeParams kp = params(g);
      ok = cudaGraphExecKernelNodeSetParams(s->graph, s->gnodes[g], &kp) == cudaSuccess;
    }
    if (ok) {
      s->graph_ctas = total;
      s->graph_updates++;
      return NAT_OK;
    }
    cudaGetLastError();  // an update the driver refused: build anew
  }
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->graph_tmpl) cudaGraphDestroy(s->graph_tmpl);
  s->graph = nullptr;
  s->graph_tmpl = nullptr;
  SCK(cudaGraphCreate(&s->graph_tmpl, 0), "graph create");
  for (int g = 0; g < NGROUPS; ++g) {
    s->gnodes[g] = nullptr;
    if (!grid[g]) continue;
    const cudaKernelNodeParams kp = params(g);
    cudaError_t e = cudaGraphAddKernelNode(&s->gnodes[g], s->graph_tmpl, nullptr, 0, &kp);
    if (e != cudaSuccess) return sfail(s, NAT_ERR_CUDA, "graph node: %s", cudaGetErrorString(e));
  }
  cudaError_t e = cudaGraphInstantiate(&s->graph, s->graph_tmpl, 0);
  if (e != cudaSuccess) return sfail(s, NAT_ERR_CUDA, "instantiate: %s", cudaGetErrorString(e));
  s->graph_mask = mask;
  s->graph_ctas = total;
  s->graph_nodes = 0;
  for (int g = 0; g < NGROUPS; ++g) s->graph_nodes += grid[g] ? 1 : 0;
  s->graph_builds++;
  return NAT_OK;
}

int admit(nat_server* s) {
  while (!s->pending.empty()) {
    const nat_request& r = s->pending.front().second;
    int slot = -1;
    for (int i = 0; i < s->max_slots; ++i)
      if (!s->slot_used[i]) {
        slot = i;
        break;
      }
    if (slot < 0) return NAT_OK;
    int nx, ny;
    const size_t bytes = footprint(r, &nx, &ny);
    size_t off;
    if (!s->pool.alloc(bytes, &off)) return NAT_OK;  // admit in order; wait for memory
    // operator tables for this request
    nat_spec sp;
    memset(&sp, 0, sizeof sp);
    sp.dim = 2;
    sp.stencil = NAT_D2Q9;
    sp.order = r.order;
    sp.topology = NAT_TOPO_FEQ;
    sp.cells[0] = r.cells[0];
    sp.cells[1] = r.cells[1];
    sp.cells[2] = 1;
    sp.length[0] = r.length[0];
    sp.length[1] = r.length[1];
    sp.length[2] = 1;
    sp.periodic[0] = sp.periodic[1] = sp.periodic[2] = 1;
    sp.scaling = r.scaling;
    sp.viscosity = r.viscosity;
    sp.cfl = r.cfl;
    sp.dt = r.dt;
    sp.collision = r.collision;
    sp.precision = NAT_FP32_DEV;
    double hmin = fmin(r.length[0] / r.cells[0], r.length[1] / r.cells[1]);
    double dt = r.dt > 0 ? r.dt : r.cfl * hmin / (sqrt(2.0) * r.scaling * r.order * r.order);
    SLTables T;
    std::string e;
    int rc = build_solver_tables(&sp, dt, &T, &e);
    if (rc) {
      s->pool.release(off, bytes);
      const int64_t id = s->pending.front().first;
      s->pending.pop_front();
      // a request that cannot run completes at once with its error status
      Completing* c = new Completing();
      c->live = {id, -1, 0, 0, s->host_step};
      c->ev = nullptr;
      c->status = rc;
      s->done[id] = c;
      continue;
    }
    SlotDesc d;
    memset(&d, 0, sizeof d);
    char* base = s->pool_base + off;
    const size_t n = (size_t)nx * ny;
    d.f[0] = reinterpret_cast<float*>(base);
    d.f[1] = d.f[0] + 9 * n;
    d.rho = reinterpret_cast<double*>(base + 2 * 9 * n * sizeof(float));
    d.u = d.rho + n;
    d.status = s->d_status + slot;
    d.n = (int)n;
    d.nx = nx;
    d.ny = ny;
    d.nseg = (nx + 31) / 32;
    d.P = r.order;
    d.coll = r.collision == NAT_BGK_STANDARD ? COLL_BGK : COLL_KBC;
    d.active = 1;
    d.start_step = s->host_step;
    d.last_step = s->host_step + r.steps - 1;
    d.tau = r.viscosity / (dt * r.scaling * r.scaling / 3.0) + 0.5;
    d.scaling = r.scaling;
    for (int a = 0; a < 3; ++a)
      for (int sd = 0; sd < 2; ++sd)
        for (int c = 0; c < PER_MAX; ++c)
          for (int j = 0; j < PMAX1; ++j) d.W[a][sd][c][j] = (float)T.w[a][sd][c][j];
    s->h_slots[slot] = d;
    s->slot_used[slot] = 1;
    SCK(cudaMemsetAsync(d.status, 0, sizeof(int), s->stream), "status clear");
    InitArgs ia;
    memset(&ia, 0, sizeof ia);
    ia.f = d.f[0];
    ia.n = (int)n;
    ia.nx = nx;
    ia.ny = ny;
    ia.P = r.order;
    ia.kind = r.init == NAT_INIT_TAYLOR_GREEN ? 0 : 1;
    ia.hx = r.length[0] / r.cells[0];
    ia.hy = r.length[1] / r.cells[1];
    ia.Lx = r.length[0];
    ia.Ly = r.length[1];
    ia.scaling = r.scaling;
    ia.Ma = r.Ma;
    ia.u0 = r.u0;
    ia.kappa = r.kappa;
    ia.delta = r.delta;
    gl_points_host(r.order, ia.xi);
    k_serve_init<<<(int)((n + 255) / 256), 256, 0, s->stream>>>(ia);
    SCK(cudaGetLastError(), "init launch");
    s->launches++;
    s->live.push_back({s->pending.front().first, slot, off, bytes, d.last_step});
    s->pending.pop_front();
    s->dirty = true;
  }
  return NAT_OK;
}

// solves whose last step is the one just enqueued: copy their results out
int retire(nat_server* s, long long step) {
  std::vector<Live> keep;
  for (const Live& L : s->live) {
    if (L.last_step != step) {
      keep.push_back(L);
      continue;
    }
    SlotDesc& d = s->h_slots[L.slot];
    Completing* c = new Completing();
    c->live = L;
    c->rho.resize(d.n);
    c->u.resize(2 * (size_t)d.n);
    c->status = 0;
    SCK(cudaMemcpyAsync(c->rho.data(), d.rho, sizeof(double) * d.n, cudaMemcpyDeviceToHost, s->stream), "result");
    SCK(cudaMemcpyAsync(c->u.data(), d.u, sizeof(double) * 2 * d.n, cudaMemcpyDeviceToHost, s->stream), "result");
    SCK(cudaMemcpyAsync(&c->status, d.status, sizeof(int), cudaMemcpyDeviceToHost, s->stream), "result");
    SCK(cudaEventCreateWithFlags(&c->ev, cudaEventDisableTiming), "event");
    SCK(cudaEventRecord(c->ev, s->stream), "event record");
    d.active = 0;
    s->completing.push_back(c);
    s->dirty = true;
  }
  s->live.swap(keep);
  return NAT_OK;
}

int harvest(nat_server* s, bool wait) {
  std::vector<Completing*> keep;
  for (Completing* c : s->completing) {
    cudaError_t q = wait ? cudaEventSynchronize(c->ev) : cudaEventQuery(c->ev);
    if (q == cudaErrorNotReady) {
      keep.push_back(c);
      continue;
    }
    if (q != cudaSuccess) return sfail(s, NAT_ERR_CUDA, "result event: %s", cudaGetErrorString(q));
    cudaEventDestroy(c->ev);
    c->ev = nullptr;
    s->pool.release(c->live.off, c->live.bytes);
    s->slot_used[c->live.slot] = 0;
    int st = c->status;
    c->status = st == 0 ? NAT_OK : ((st & ST_NAN) ? NAT_ERR_NAN : NAT_ERR_DENSITY_UNDERFLOW);
    s->done[c->live.id] = c;
  }
  s->completing.swap(keep);
  return NAT_OK;
}

}  // namespace

extern "C" {

int nat_server_create(size_t pool_bytes, int max_slots, nat_server** out) {
  if (!out || pool_bytes < (1u << 20) || max_slots < 1) return NAT_ERR_INVALID_ARG;
  nat_server* s = new nat_server();
  *out = s;
  SCK(cudaGetDevice(&s->device), "device");
  SCK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "stream");
  cudaError_t e = cudaMalloc(&s->pool_base, pool_bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return sfail(s, NAT_ERR_OOM, "pool of %zu bytes: %s", pool_bytes, cudaGetErrorString(e));
  }
  s->pool_bytes = pool_bytes;
  s->pool.init(pool_bytes);
  s->max_slots = max_slots;
  s->h_slots.assign(max_slots, SlotDesc());
  memset(s->h_slots.data(), 0, sizeof(SlotDesc) * max_slots);
  s->slot_used.assign(max_slots, 0);
  SCK(cudaMalloc(&s->d_slots, sizeof(SlotDesc) * max_slots), "slots");
  SCK(cudaMalloc(&s->d_status, sizeof(int) * max_slots), "status");
  SCK(cudaMalloc(&s->d_groups, sizeof(GroupRange) * NGROUPS), "groups");
  SCK(cudaMalloc(&s->d_step, sizeof(long long)), "step");
  SCK(cudaMemsetAsync(s->d_step, 0, sizeof(long long), s->stream), "step clear");
  SCK(cudaMalloc(&s->d_ticket, sizeof(unsigned)), "ticket");
  SCK(cudaMemsetAsync(s->d_ticket, 0, sizeof(unsigned), s->stream), "ticket clear");
  s->max_work = 1 << 16;
  SCK(cudaMalloc(&s->d_work, sizeof(WorkItem) * s->max_work), "work list");
  for (int k = 0; k < nat_server::NSTAGE; ++k) {
    s->stage_cap[k] = s->max_work;
    SCK(cudaHostAlloc(&s->stage_work[k], sizeof(WorkItem) * s->stage_cap[k], cudaHostAllocDefault), "staging");
    SCK(cudaHostAlloc(&s->stage_groups[k], sizeof(GroupRange) * NGROUPS, cudaHostAllocDefault), "staging");
    SCK(cudaHostAlloc(&s->stage_slots[k], sizeof(SlotDesc) * max_slots, cudaHostAllocDefault), "staging");
    SCK(cudaEventCreateWithFlags(&s->stage_ev[k], cudaEventDisableTiming), "staging event");
  }
  for (int k = 0; k < RUNAHEAD_RING; ++k)
    SCK(cudaEventCreateWithFlags(&s->ahead_ev[k], cudaEventDisableTiming), "run-ahead event");
  SCK(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device), "sm count");
  return NAT_OK;
}

int nat_server_destroy(nat_server* s) {
  if (!s) return NAT_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (Completing* c : s->completing) {
    if (c->ev) cudaEventDestroy(c->ev);
    delete c;
  }
  for (auto& kv : s->done) delete kv.second;
  if (s->graph) cudaGraphExecDestroy(s->graph);
  if (s->graph_tmpl) cudaGraphDestroy(s->graph_tmpl);
  cudaFree(s->pool_base);
  cudaFree(s->d_slots);
  cudaFree(s->d_status);
  cudaFree(s->d_groups);
  cudaFree(s->d_step);
  cudaFree(s->d_ticket);
  cudaFree(s->d_work);
  for (int k = 0; k < nat_server::NSTAGE; ++k) {
    cudaFreeHost(s->stage_work[k]);
    cudaFreeHost(s->stage_groups[k]);
    cudaFreeHost(s->stage_slots[k]);
    if (s->stage_ev[k]) cudaEventDestroy(s->stage_ev[k]);
  }
  for (int k = 0; k < RUNAHEAD_RING; ++k)
    if (s->ahead_ev[k]) cudaEventDestroy(s->ahead_ev[k]);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return NAT_OK;
}

int nat_server_submit(nat_server* s, const nat_request* r, int64_t* id) {
  if (!s || !r || !id) return NAT_ERR_INVALID_ARG;
  int rc = validate(s, *r);
  if (rc) return rc;
  int nx, ny;
  if (footprint(*r, &nx, &ny) > s->pool_bytes) return sfail(s, NAT_ERR_OOM, "request larger than the pool");
  *id = s->next_id++;
  s->pending.push_back({*id, *r});
  return NAT_OK;
}

}  // extern "C"

namespace {

// One server step: collect finished results, admit queued requests, advance
// every live solve by one time step (one graph launch).  *ran = 0 when no
// solve was live.
int server_step(nat_server* s, int* ran) {
  *ran = 0;
  int rc = harvest(s, false);
  if (rc) return rc;
  rc = admit(s);
  if (rc) return rc;
  if (s->live.empty()) return NAT_OK;
  if (s->dirty || s->graph_stale || !s->graph) {
    const auto t0 = std::chrono::steady_clock::now();
    if (s->dirty) {
      rc = upload_state(s);
      if (rc) return rc;
    }
    rc = capture(s);
    if (rc) return rc;
    s->graph_stale = false;
    s->rebuild_ns +=
        std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
  }
  SCK(cudaGraphLaunch(s->graph, s->stream), "graph launch");
  s->launches += s->graph_nodes;  // the graph's kernels, one per group
  const long long step = s->host_step++;
  s->steps_run++;
  for (const Live& L : s->live) s->node_updates += s->h_slots[L.slot].n;
  // keep the host at most RUNAHEAD_EVERY * RUNAHEAD_RING steps ahead of the device
  if (s->host_step % RUNAHEAD_EVERY == 0) {
    const int k = s->ahead_k;
    if (s->ahead_used[k]) SCK(cudaEventSynchronize(s->ahead_ev[k]), "run-ahead wait");
    SCK(cudaEventRecord(s->ahead_ev[k], s->stream), "run-ahead event");
    s->ahead_used[k] = true;
    s->ahead_k = (k + 1) % RUNAHEAD_RING;
  }
  *ran = 1;
  return retire(s, step);
}

}  // namespace

extern "C" {

int nat_server_step(nat_server* s) {
  if (!s) return NAT_ERR_INVALID_ARG;
  int ran;
  return server_step(s, &ran);
}

int nat_server_run(nat_server* s, int max_steps, int* steps_done) {
  if (!s || max_steps < 0) return NAT_ERR_INVALID_ARG;
  int k = 0;
  for (; k < max_steps; ++k) {
    int ran = 0;
    const int rc = server_step(s, &ran);
    if (rc) {
      if (steps_done) *steps_done = k;
      return rc;
    }
    if (!ran) break;
  }
  if (steps_done) *steps_done = k;
  return NAT_OK;
}

int nat_server_poll(nat_server* s, int64_t* ids, int max_ids, int* n_done, int wait) {
  if (!s || !n_done) return NAT_ERR_INVALID_ARG;
  int rc = harvest(s, wait != 0);
  if (rc) return rc;
  int k = 0;
  for (auto& kv : s->done) {
    if (k >= max_ids) break;
    if (ids) ids[k] = kv.first;
    ++k;
  }
  *n_done = k;
  return NAT_OK;
}

int nat_server_result(nat_server* s, int64_t id, double* rho, double* u, int64_t* n_nodes, int* status) {
  if (!s) return NAT_ERR_INVALID_ARG;
  auto it = s->done.find(id);
  if (it == s->done.end()) return sfail(s, NAT_ERR_INVALID_ARG, "request %lld is not finished", (long long)id);
  Completing* c = it->second;
  if (n_nodes) *n_nodes = (int64_t)c->rho.size();
  if (status) *status = c->status;
  if (rho && !c->rho.empty()) memcpy(rho, c->rho.data(), sizeof(double) * c->rho.size());
  if (u && !c->u.empty()) memcpy(u, c->u.data(), sizeof(double) * c->u.size());
  delete c;
  s->done.erase(it);
  return NAT_OK;
}

int nat_server_stats(const nat_server* s, nat_server_stats_t* st) {
  if (!s || !st) return NAT_ERR_INVALID_ARG;
  st->pending = (int64_t)s->pending.size();
  st->live = (int64_t)s->live.size();
  st->completing = (int64_t)s->completing.size();
  st->finished = (int64_t)s->done.size();
  st->steps = s->steps_run;
  st->node_updates = s->node_updates;
  st->pool_used = (int64_t)s->pool.used;
  st->pool_bytes = (int64_t)s->pool_bytes;
  st->launches = s->launches;
  st->graph_builds = s->graph_builds;
  st->graph_updates = s->graph_updates;
  st->rebuild_ns = s->rebuild_ns;
  return NAT_OK;
}

int nat_server_last_error(const nat_server* s, char* buf, size_t len) {
  if (!buf || !len) return NAT_ERR_INVALID_ARG;
  snprintf(buf, len, "%s", s ? s->err.c_str() : "null server");
  return NAT_OK;
}

}  // extern "C"
