// Launcher table shared by the per-stencil translation units and the API.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/natgpu.h"
#include "natgpu_common.h"

namespace natgpu {

// collision selector values (match sl_step.cuh)
enum { L_COLL_NONE = 0, L_COLL_BGK = 1, L_COLL_BGK_INC = 2, L_COLL_KBC = 3 };

struct KernelSet {
  const void* step;      // fused stream(+collide) kernel, NULL if unsupported
  const void* collide;   // collide-only kernel, NULL for COLL_NONE
  const void* wallnode;  // fused step of the wall nodes (k_wall_nodes), NULL for COLL_NONE
  // the same three with the body-force term (BGK only, else NULL)
  const void* step_force = nullptr;
  const void* collide_force = nullptr;
  const void* wallnode_force = nullptr;
};

// prec: 0 = FP64, 1 = FP32 deviation
KernelSet kernels_d2q9(int coll, int prec);
KernelSet kernels_d3q19(int coll, int prec);
KernelSet kernels_d3q27(int coll, int prec);

// departure-point kernels of mapped meshes (sl_mapped.cuh) for order p;
// NULL when the combination is not instantiated.  coll L_COLL_BGK_FORCE: the
// BGK form with the body-force term.
constexpr int L_COLL_BGK_FORCE = 100;
const void* mapped_kernel_d2q9(int coll, int prec, int p);
const void* mapped_kernel_d3q19(int coll, int prec, int p);
const void* mapped_kernel_d3q27(int coll, int prec, int p);

// threads per CTA of the fused kernel and nodes per thread
constexpr int STEP_THREADS = 256;
constexpr int STEP_NPT = 2;

// dynamic shared memory of the fused kernel
size_t step_smem_bytes(int prec, const int Rmax[3], const int B[3]);

// Specialised fused kernel (sl_step_v2.cuh): compile-time order, topology
// and tile shape.
struct V2Launch {
  int stencil, coll, prec, P;
  bool dg;
  int cells[3];  // tile shape in cells
  int B[3];      // tile shape in nodes
  int nth;       // threads per CTA
  const void* fn;
  size_t smem;
};
// operator tables of a solve (natgpu_api.cu), for the server's slots
int build_solver_tables(const struct ::nat_spec* spec, double dt, SLTables* T, std::string* err);
void gl_points_host(int p, double* xi);

// every instantiation that applies, in order of preference
std::vector<V2Launch> find_v2(int stencil, int coll, int prec, int P, bool dg, const int cells[3], int dim,
                              int nx);

// Row-segment fused kernel (sl_row.cuh): one warp per 32 x-nodes at a fixed
// (y, z); CTA = WY x WZ warps.
struct RowLaunch {
  int stencil, coll, prec, P;
  bool dg;
  int wy, wz;
  const void* fn;
  int kind = 3;      // 3: row kernel (sl_row.cuh), 6: bulk-copy row kernel (sl_rowt.cuh),
                     // 7: row-group kernel (sl_rowg.cuh; wy = rows per CTA),
                     // 11: cell-row kernel (sl_cell.cuh; wy = rows per CTA),
                     // 12: the same with the D3Q27 corner directions on the tensor cores,
                     // 13: the same with z sharing of the yz-diagonal directions
  int g = 0;         // kind 7: warps per x row (32 (g - 1) < nx <= 32 g); kind 11-13: cells per x row
  int warps = 0;     // kind 11-13: warps per CTA
  size_t smem = 0;   // dynamic shared memory (kind 6)
  int align = 1;     // nx must be a multiple of this (kind 6: aligned row copies)
  int min_nx = 0;    // and at least this (kind 6: at most two pieces per row)
};
void row_kernels_d2q9(std::vector<RowLaunch>& v);
void row_kernels_d3q19(std::vector<RowLaunch>& v);
void row_kernels_d3q27(std::vector<RowLaunch>& v);
void row_ss_kernels_d3q19(std::vector<RowLaunch>& v);
void rowg_kernels_d3q19(std::vector<RowLaunch>& v);
void rowg_kernels_d3q27(std::vector<RowLaunch>& v);
void row_ss_kernels_d3q27(std::vector<RowLaunch>& v);
void rowt_kernels_d3q19(std::vector<RowLaunch>& v);
void rowt_kernels_d3q27_bgk(std::vector<RowLaunch>& v);
void rowt_kernels_d3q27_kbc(std::vector<RowLaunch>& v);
void cell_kernels(std::vector<RowLaunch>& v);

// Compressible two-population model on D2Q25H (k_thermal.cu): fused
// stream(f, g) (+ relaxWithG), collision only, equilibrium initialisation;
// FP64 and FP32-deviation forms.
// form: 0 register form, 1 / 2 shared-memory forms (FP32 only)
cudaError_t launch_thermal_step(const ThermalStepT<double>& P, bool collide, cudaStream_t st, int form);
cudaError_t launch_thermal_step(const ThermalStepT<float>& P, bool collide, cudaStream_t st, int form);
cudaError_t launch_thermal_collide(const ThermalPointT<double>& P, int grid, cudaStream_t st);
cudaError_t launch_thermal_collide(const ThermalPointT<float>& P, int grid, cudaStream_t st);
cudaError_t launch_thermal_init(const ThermalPointT<double>& P, void* f, void* g, bool fp32, int grid,
                                cudaStream_t st);
// fused step of the wall nodes of the two-population model: rows as
// k_wall_nodes, f and g through the same rows (constant slots f, g);
// collide = false: the rows only (the step kernel then collides the nodes)
cudaError_t launch_thermal_wall_nodes(const ThermalStepT<double>& P, int nbn, const int* node, const int* ptr,
                                      const int* col, const double* w, const double* cst, bool collide,
                                      cudaStream_t st);
cudaError_t launch_thermal_wall_nodes(const ThermalStepT<float>& P, int nbn, const int* node, const int* ptr,
                                      const int* col, const float* w, const double* cst, bool collide,
                                      cudaStream_t st);

}  // namespace natgpu
