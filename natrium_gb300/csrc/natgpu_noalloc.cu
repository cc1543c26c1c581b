// Allocation-free FP64 mass / kinetic-energy reduction.
//
// Some callers cannot allocate device memory at the point where they need
// these global diagnostics: code that records its work into a CUDA graph
// (cudaMalloc is not allowed while a stream is being captured), embeddings
// where a host framework owns every device byte through its own pool, and
// latency-bound loops that cannot afford cudaMalloc's implicit device
// synchronisation.  nat_mass_energy_noalloc serves them: the caller passes
// the input fields and a device output, and the only scratch the reduction
// needs -- one partial sum pair per block -- lives in the file-scope array
// g_partials below, which every GPU that loads the library holds until the
// process exits.
//
// Contract:
//   * at most NAT_NOALLOC_MAX_NODES lattice nodes per call (larger inputs are
//     rejected with NAT_ERR_INVALID_ARG and a message);
//   * every axis holds whole cells (a multiple of p nodes for FE_Q with the
//     periodic duplicates folded, of p + 1 for DG), else NAT_ERR_INVALID_ARG;
//   * the first call on a device looks up the device address of g_partials
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before capturing any stream, later calls do no set-up (a call after a
//     cudaDeviceReset sees a new context id and looks the address up again);
//   * every call shares g_partials: calls whose kernels overlap on the GPU
//     (different streams, or different host threads) race on it and must be
//     serialised by the caller;
//   * nothing in g_partials has to start at zero: the first kernel writes
//     every partial the second one reads, so the last call's contents are
//     simply overwritten;
//   * no cudaMalloc, cudaFree or allocating library routine is called.
// The reduction order is fixed (one contiguous chunk per block, then one
// block over the partials), so repeated calls on the same input give
// bitwise identical results.
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "../../include/natgpu.h"
#include "natgpu_common.h"
#include "solver.h"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_NODES_PER_BLOCK = NA_THREADS * 16;  // one contiguous chunk per block
constexpr int NA_MAX_BLOCKS = 4096;                  // partials held by g_partials
static_assert((long long)NA_MAX_BLOCKS * NA_NODES_PER_BLOCK == NAT_NOALLOC_MAX_NODES,
              "header limit must match the scratch size");

// the scratch: mass and energy partial of every block (64 KiB)
static __device__ __align__(256) double g_partials[2 * NA_MAX_BLOCKS];

struct NaQuad {
  double w[3][natgpu::PER_MAX];  // per axis, per node class: quadrature weight * cell size
  int period;
  int nx, ny, nz, dim;
  long long n;
};

__device__ __forceinline__ void block_sum2(double& a, double& b, double (*sm)[NA_THREADS / 32]) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sm[0][wid] = a;
    sm[1][wid] = b;
  }
  __syncthreads();
  if (wid == 0) {
    a = lane < NA_THREADS / 32 ? sm[0][lane] : 0.0;
    b = lane < NA_THREADS / 32 ? sm[1][lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
  }
}

// pass 1: block b reduces nodes [b * NA_NODES_PER_BLOCK, ...) into partials
__global__ void __launch_bounds__(NA_THREADS) k_me_partials(const double* __restrict__ rho,
                                                           const double* __restrict__ u, NaQuad q,
                                                           double* __restrict__ partials) {
  __shared__ double sm[2][NA_THREADS / 32];
  double m = 0.0, e = 0.0;
  const long long begin = (long long)blockIdx.x * NA_NODES_PER_BLOCK;
  const long long end = min(begin + NA_NODES_PER_BLOCK, q.n);
  for (long long i = begin + threadIdx.x; i < end; i += NA_THREADS) {
    const int x = (int)(i % q.nx);
    const int y = (int)((i / q.nx) % q.ny);
    const int z = (int)(i / ((long long)q.nx * q.ny));
    double wgt = q.w[0][x % q.period] * q.w[1][y % q.period];
    if (q.dim == 3) wgt *= q.w[2][z % q.period];
    double uu = u[i] * u[i] + u[q.n + i] * u[q.n + i];
    if (q.dim == 3) uu += u[2 * q.n + i] * u[2 * q.n + i];
    m += wgt * rho[i];
    e += wgt * rho[i] * uu;
  }
  block_sum2(m, e, sm);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = m;
    partials[2 * blockIdx.x + 1] = e;
  }
}

// pass 2: one block over the partials, result to the caller's output
__global__ void __launch_bounds__(NA_THREADS) k_me_final(const double* __restrict__ partials, int nb,
                                                        double* __restrict__ out) {
  __shared__ double sm[2][NA_THREADS / 32];
  double m = 0.0, e = 0.0;
  for (int b = threadIdx.x; b < nb; b += NA_THREADS) {
    m += partials[2 * b];
    e += partials[2 * b + 1];
  }
  block_sum2(m, e, sm);
  if (threadIdx.x == 0) {
    out[0] = m;
    out[1] = 0.5 * e;
  }
}

// Device address of g_partials, looked up once per device and CUDA context.
// The context id is part of the key so that a cudaDeviceReset between calls
// (which destroys the context and the module holding g_partials) leads to a
// fresh look-up instead of a stale address.
struct AddrEntry {
  unsigned long long ctx_id;
  double* addr;
};
std::mutex g_mtx;
AddrEntry g_addr[64] = {};

// id of the current CUDA context (cuCtxGetCurrent / cuCtxGetId, reached through
// the runtime's driver entry points so the library does not link libcuda);
// 0 when unavailable, which disables the reset check but not the cache
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

}  // namespace

extern "C" int nat_mass_energy_noalloc(const double* rho_dev, const double* u_dev, int dim, const int n_axis[3],
                                       int order, int topology, const double cell_size[3], double* out_dev,
                                       void* cuda_stream) {
  if (!rho_dev || !u_dev || !n_axis || !cell_size || !out_dev) return NAT_ERR_INVALID_ARG;
  if (dim != 2 && dim != 3) return NAT_ERR_INVALID_ARG;
  if (order < 1 || order > natgpu::PMAX) return NAT_ERR_INVALID_ARG;
  if (topology != NAT_TOPO_FEQ && topology != NAT_TOPO_DG) return NAT_ERR_INVALID_ARG;
  // node classes repeat with the period of a cell: p (FE_Q, periodic
  // duplicates folded) or p + 1 (DG); an axis must hold whole cells
  const int period = topology == NAT_TOPO_DG ? order + 1 : order;
  long long n = 1;
  for (int a = 0; a < dim; ++a) {
    if (n_axis[a] < 1 || n_axis[a] % period != 0) return NAT_ERR_INVALID_ARG;
    n *= n_axis[a];
  }
  if (n > NAT_NOALLOC_MAX_NODES) return NAT_ERR_INVALID_ARG;  // beyond the scratch in g_partials
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return NAT_ERR_CUDA;
  double* partials;
  {
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lk(g_mtx);
    AddrEntry& e = g_addr[dev];
    if (!e.addr || (ctx != 0 && e.ctx_id != ctx)) {
      // set-up, once per device (and again after a reset of its context),
      // with that device current
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_partials) != cudaSuccess || !p) return NAT_ERR_CUDA;
      e.addr = static_cast<double*>(p);
      e.ctx_id = current_context_id();  // the look-up made the context current
    }
    partials = e.addr;
  }
  NaQuad q;
  double xi[natgpu::PMAX1 + 1], wq[natgpu::PMAX1 + 1];
  natgpu::api::gl_points(order, xi);  // the rule nat_mass_energy uses
  natgpu::api::gl_weights(order, xi, wq);
  q.period = period;
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < natgpu::PER_MAX; ++c) {
      double w = c < q.period ? wq[c] : 0.0;
      if (topology == NAT_TOPO_FEQ && c == 0) w += wq[order];  // node shared by two cells
      q.w[a][c] = a < dim ? w * cell_size[a] : 1.0;
    }
  q.nx = n_axis[0];
  q.ny = dim >= 2 ? n_axis[1] : 1;
  q.nz = dim == 3 ? n_axis[2] : 1;
  q.dim = dim;
  q.n = n;
  int nb = (int)((n + NA_NODES_PER_BLOCK - 1) / NA_NODES_PER_BLOCK);
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  // each launch's own status (an earlier, unrelated error of the caller's
  // thread is neither reported nor cleared here)
  void* a1[] = {(void*)&rho_dev, (void*)&u_dev, (void*)&q, (void*)&partials};
  if (cudaLaunchKernel((const void*)k_me_partials, dim3(nb), dim3(NA_THREADS), a1, 0, st) != cudaSuccess)
    return NAT_ERR_CUDA;
  const double* pc = partials;
  void* a2[] = {(void*)&pc, (void*)&nb, (void*)&out_dev};
  if (cudaLaunchKernel((const void*)k_me_final, dim3(1), dim3(NA_THREADS), a2, 0, st) != cudaSuccess)
    return NAT_ERR_CUDA;
  return NAT_OK;
}
