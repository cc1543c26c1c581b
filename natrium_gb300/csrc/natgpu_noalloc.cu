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
//   * the first call on a device looks up the device address of g_partials
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before capturing any stream, later calls do no set-up;
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

// per-device address of g_partials, looked up once per device
std::mutex g_mtx;
double* g_addr[64] = {nullptr};

// Gauss-Lobatto points on [0, 1] and their quadrature weights (host, no
// allocation)
void gl_rule(int p, double* xi, double* wq) {
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
      long double dx = d1 / ((2 * x * d1 - p * (p + 1) * p1) / (1 - x * x));
      x -= dx;
      if (fabsl(dx) < 1e-22L) break;
    }
    xi[j] = (double)((x + 1.0L) / 2.0L);
  }
  for (int j = 0; j <= p; ++j) {
    long double x = 2.0L * xi[j] - 1.0L, p0 = 1, p1 = x;
    for (int k = 2; k <= p; ++k) {
      long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    wq[j] = (double)(1.0L / ((long double)p * (p + 1) * p1 * p1));
  }
}

}  // namespace

extern "C" int nat_mass_energy_noalloc(const double* rho_dev, const double* u_dev, int dim, const int n_axis[3],
                                       int order, int topology, const double cell_size[3], double* out_dev,
                                       void* cuda_stream) {
  if (!rho_dev || !u_dev || !n_axis || !cell_size || !out_dev) return NAT_ERR_INVALID_ARG;
  if (dim != 2 && dim != 3) return NAT_ERR_INVALID_ARG;
  if (order < 1 || order > natgpu::PMAX) return NAT_ERR_INVALID_ARG;
  if (topology != NAT_TOPO_FEQ && topology != NAT_TOPO_DG) return NAT_ERR_INVALID_ARG;
  long long n = 1;
  for (int a = 0; a < dim; ++a) {
    if (n_axis[a] < 1) return NAT_ERR_INVALID_ARG;
    n *= n_axis[a];
  }
  if (n > NAT_NOALLOC_MAX_NODES) return NAT_ERR_INVALID_ARG;  // beyond the scratch in g_partials
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return NAT_ERR_CUDA;
  double* partials;
  {
    std::lock_guard<std::mutex> lk(g_mtx);
    if (!g_addr[dev]) {
      // set-up, once per device, with that device current
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_partials) != cudaSuccess || !p) {
        cudaGetLastError();
        return NAT_ERR_CUDA;
      }
      g_addr[dev] = static_cast<double*>(p);
    }
    partials = g_addr[dev];
  }
  NaQuad q;
  double xi[natgpu::PMAX1 + 1], wq[natgpu::PMAX1 + 1];
  gl_rule(order, xi, wq);
  q.period = topology == NAT_TOPO_DG ? order + 1 : order;
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
  const int nb = (int)((n + NA_NODES_PER_BLOCK - 1) / NA_NODES_PER_BLOCK);
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  k_me_partials<<<nb, NA_THREADS, 0, st>>>(rho_dev, u_dev, q, partials);
  k_me_final<<<1, NA_THREADS, 0, st>>>(partials, nb, out_dev);
  return cudaGetLastError() == cudaSuccess ? NAT_OK : NAT_ERR_CUDA;
}
