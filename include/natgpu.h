/*
 * natgpu.h -- C ABI of the GB300-native semi-Lagrangian stream + collide
 * engine (libnatgpu.so).
 *
 * The entry points replace, for one CFDSolver-style time loop, the two
 * operator interfaces of NATriuM that carry the hot path:
 *
 *   advection/AdvectionOperator.h:151-152 (virtual double stream(f_old, f, t)),
 *   implemented by advection/SemiLagrangian.h:150-161 and inlined in
 *   solver/CFDSolver.cpp:658-754 (copy f, BlockSparseMatrix::vmult, boundaries);
 *
 *   collision/CollisionModel.h:74-78 (virtual void collideAll(f, rho, u,
 *   owned, inInitializationProcedure)), run in the time loop through
 *   collision_advanced/CollisionSelection.h:60-232 -> CollisionOperator.h:26-111.
 *
 * Plain C: plain pointers and sizes, no C++ or torch types.  Every call
 * returns an int status (NAT_OK == 0); no exception crosses the ABI.  The
 * text of the last error of a handle is available from nat_last_error().
 * A handle is thread-compatible, not thread-safe: one CUDA stream per handle.
 *
 * Distribution-function layout on the host (reference layout): Q blocks of
 * n_ref doubles, block 0 = f_0 (the rest population, never streamed), blocks
 * 1..Q-1 = the streamed directions in the stencil's own order (this is the
 * order of DistributionFunctions::at(i), solver/DistributionFunctions.h:47-300).
 * Inside a block the nodes are numbered lexicographically over the node
 * lattice of the Cartesian mesh, x fastest:
 *   NAT_TOPO_FEQ: (N_a * p + 1) nodes per axis (continuous FE_Q on
 *                 Gauss-Lobatto points, the reference's semi-Lagrangian element,
 *                 advection/SemiLagrangian.cpp:43-44; periodic duplicates kept);
 *   NAT_TOPO_DG:  N_a * (p + 1) nodes per axis (FE_DGQArbitraryNodes).
 * Macroscopic fields: rho[n_ref], u[D][n_ref] with u scaled (u_lattice *
 * scaling), as the reference stores them (CollisionOperator.h:79-82).
 */
#ifndef NATGPU_H
#define NATGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define NAT_OK 0
#define NAT_ERR_INVALID_ARG 1
#define NAT_ERR_OOM 2
/* rho < 1e-10 in a collision: the reference throws CollisionException /
 * DensityZeroException (collision_advanced/AuxiliaryCollisionFunctions.h:53-56,
 * CollisionOperator.h:106-109) */
#define NAT_ERR_DENSITY_UNDERFLOW 3
#define NAT_ERR_NAN 4
#define NAT_ERR_TIMEOUT 5
#define NAT_ERR_CUDA 6
#define NAT_ERR_UNSUPPORTED 7

/* ---- stencils (the stencils/ directory of the reference) --------------- */
#define NAT_D2Q9 0
#define NAT_D3Q19 1
#define NAT_D3Q27 2
#define NAT_D2Q25H 3

/* ---- collision models (utilities/ConfigNames.h CollisionSchemeName) ---- */
#define NAT_BGK_STANDARD 0      /* BGKCollision + BGKEquilibrium */
#define NAT_BGK_INCOMPRESSIBLE 1 /* collision/BGKIncompressible.cpp (D2Q9) */
#define NAT_KBC_STANDARD 2      /* collision/KBCStandard.cpp (D2Q9); D3Q27 extension */
/* Compressible two-population BGK of CompressibleCFDSolver on D2Q25H: f and g
 * streamed by the same operator (solver/CompressibleCFDSolver.h:181-314),
 * collideAll(f, g, rho, u, T, mask) (collision_advanced/CollisionOperator.h:113-224)
 * with BGKCollision::relaxWithG (collision_advanced/CollisionSchemes.h:43-118).
 * Requires stencil NAT_D2Q25H (and D2Q25H requires this model).  Precision
 * NAT_FP64, or NAT_FP32_DEV: f - w_i and g - w_i g_ref (g_ref = 3, the
 * rest-state g^eq / f^eq for gamma = 1.4) stored and computed in float. */
#define NAT_BGK_COMPRESSIBLE 3

/* ---- node topology ----------------------------------------------------- */
#define NAT_TOPO_FEQ 0
#define NAT_TOPO_DG 1

/* ---- storage precision ------------------------------------------------- */
#define NAT_FP64 0     /* plain: f stored and computed in double */
#define NAT_FP32_DEV 1 /* f - w_i stored in float, float arithmetic,
                          compensated moment sums */

/* Solver description.  Replaces the subset of SolverConfiguration /
 * ProblemDescription that the stream + collide path reads. */
typedef struct nat_spec {
  int dim;          /* 2 or 3 */
  int stencil;      /* NAT_D2Q9 ... */
  int order;        /* FE order p (1..6) */
  int topology;     /* NAT_TOPO_FEQ or NAT_TOPO_DG */
  int cells[3];     /* uniform Cartesian cells per axis (unused axes: 1) */
  double length[3]; /* box edge lengths; the box is [0, L_a) */
  int periodic[3];  /* 1: periodic axis; 0: two wall faces (DG topology only),
                       bounce-back at rest until nat_set_boundary changes them */
  double scaling;   /* stencil scaling (e = scaling * unit vectors) */
  double viscosity; /* kinematic viscosity nu */
  double cfl;       /* used when dt <= 0: dt = CFL h_min / (sqrt(2) scaling p^2)
                       (utilities/CFDSolverUtilities.cpp:92-100) */
  double dt;        /* time step; <= 0 selects the CFL rule */
  int collision;    /* NAT_BGK_STANDARD ... */
  int precision;    /* NAT_FP64 or NAT_FP32_DEV */
  /* MappingQ1 cells (advection/AdvectionOperator.cpp:59-63 picks MappingQ1
   * when the problem is not Cartesian): NULL = the Cartesian box of `length`;
   * else the vertices of the structured grid of cells[] cells, x fastest,
   * (cells[0]+1)(cells[1]+1)[(cells[2]+1)] points of 3 doubles each (z
   * ignored in 2-D), copied at creation.  Every cell is the multilinear
   * image of the unit cell; a periodic axis needs one translation vector
   * between the vertices of its two faces (PeriodicBoundary.cpp:184-270).
   * The CFL time step then uses the smallest distance between two vertices
   * of a cell (utilities/CFDSolverUtilities.cpp:69-84). */
  const double* vertices;
} nat_spec;

typedef struct nat_solver nat_solver;

/* Create a solver: allocates device buffers on the current CUDA device and
 * assembles the streaming operator for dt (SemiLagrangian::setDeltaT ->
 * updateSparsityPattern/reassemble, advection/SemiLagrangian.h:175-179).
 * Q x nodes must stay below 2^31 (32-bit indexing in the kernels; e.g.
 * 113 M nodes of D3Q19): larger lattices get NAT_ERR_UNSUPPORTED. */
int nat_create(const nat_spec* spec, nat_solver** out);
int nat_destroy(nat_solver* s);

/* Sizes: n_ref = nodes per block in the reference layout; n_dev = nodes per
 * block on the device (periodic duplicates folded); Q, D. */
int nat_sizes(const nat_solver* s, int64_t* n_ref, int64_t* n_dev, int* Q,
              int* D);
/* Time step and relaxation time tau = nu / (dt c_s^2) + 1/2
 * (collision_advanced/AuxiliaryCollisionFunctions.h:63-68). */
int nat_get_dt(const nat_solver* s, double* dt, double* tau);

/* setDeltaT: rebuild the operator for a new time step
 * (advection/SemiLagrangian.h:175-179). */
int nat_set_dt(nat_solver* s, double dt);

/* Bind the handle to a CUDA stream (cudaStream_t passed as void*); NULL =
 * the legacy default stream.  Work already enqueued on the previous stream
 * is ordered before work enqueued on the new one. */
int nat_set_stream(nat_solver* s, void* cuda_stream);

/* Copy f (host, reference layout, Q * n_ref doubles) to the device.
 * Enqueued without waiting: the copy runs on the handle's own copy stream
 * into one of two input staging buffers, and the conversion to the device
 * layout on the handle's stream waits for it.  Work enqueued later on the
 * handle's stream sees the new f.  With page-locked f_host the copy is
 * asynchronous: keep f_host unchanged until a later synchronising call
 * (nat_status, nat_wait, a blocking download) returns. */
int nat_upload_f(nat_solver* s, const double* f_host);
/* Copy f back to the host (reference layout; periodic duplicates filled). */
int nat_download_f(nat_solver* s, double* f_host);
/* Copy rho (n_ref) and u (D * n_ref, scaled) of the last collision. */
int nat_download_macro(nat_solver* s, double* rho_host, double* u_host);
/* The read-back of nat_download_macro, enqueued without waiting.  *ticket
 * receives a number for nat_wait; rho_host and u_host (page-locked for an
 * asynchronous copy) must stay valid and are filled once nat_wait(ticket)
 * returns.  The device status word is read and cleared with it, so the
 * ticket carries the status of the steps enqueued since the previous read of
 * it.  The conversion to the reference layout runs on the handle's stream,
 * the copies to the host on the handle's own read-back stream, so they
 * overlap the steps enqueued after this call.
 * Used to pipeline host I/O: the upload of the next f runs while this
 * read-back is in flight. */
int nat_download_macro_async(nat_solver* s, double* rho_host, double* u_host,
                             uint64_t* ticket);
/* Wait until the read-back of a ticket is on the host; returns its status
 * (NAT_OK, NAT_ERR_DENSITY_UNDERFLOW, NAT_ERR_NAN, NAT_ERR_TIMEOUT).  Up to 8 tickets are
 * tracked; issuing a ninth waits for the oldest, and its status, if nobody
 * waited for it, is returned by the next nat_wait. */
int nat_wait(nat_solver* s, uint64_t ticket);
/* Copy rho and scaled u from the host to the device (the input of a
 * collision with in_init != 0). */
int nat_upload_macro(nat_solver* s, const double* rho_host,
                     const double* u_host);

/* AdvectionOperator::stream(f_old, f, t): f <- A f (semi-Lagrangian
 * streaming of directions 1..Q-1, f_0 unchanged); writes dt to *dt_out when
 * dt_out != NULL (the interface returns dt). */
int nat_stream(nat_solver* s, double t, double* dt_out);

/* CollisionModel::collideAll(f, rho, u, owned, inInitializationProcedure):
 * in-place collision of every node; writes rho and (unless in_init) u.  With
 * in_init != 0 the velocity is taken from the device copy of u. */
int nat_collide(nat_solver* s, int in_init);

/* n_steps of the CFDSolver loop body {stream(); collide();} fused into one
 * kernel per step.  rho and u are written by the last step only.  Checks the
 * device status word once at the end (synchronises the stream). */
int nat_step(nat_solver* s, int n_steps);

/* Same as nat_step but only enqueues the work (no synchronisation, no status
 * check); pair with nat_status(). */
int nat_step_async(nat_solver* s, int n_steps, int write_macro);

/* Synchronise the handle's stream and return the device status
 * (NAT_OK, NAT_ERR_DENSITY_UNDERFLOW, NAT_ERR_NAN, or NAT_ERR_TIMEOUT when
 * a bulk-copy kernel's wait for a copy ran out and a step is incomplete);
 * clears it. */
int nat_status(nat_solver* s);

/* Limit of every wait of the bulk-copy kernels (tile and bulk-copy row
 * kernels) for a copy, in polls of its mbarrier; default 2^24.  A wait that
 * runs out sets NAT_ERR_TIMEOUT in the status, waits (bounded) for the
 * copies it still has in flight and stops its tile, so a lost copy cannot
 * hang the GPU.  0 makes every such wait run out at once: the way to test
 * that path without a fault. */
int nat_set_wait_limit(nat_solver* s, uint32_t polls);

/* Copy the text of the last error into buf (always NUL terminated). */
int nat_last_error(const nat_solver* s, char* buf, size_t len);

/* FP64 global reductions over the device state (mass = sum of rho over the
 * lattice nodes with Gauss-Lobatto quadrature weights; kinetic energy
 * 0.5 sum rho |u|^2 with the same weights, solver/PhysicalProperties.cpp:29-79);
 * they use the macroscopic fields of the last collision. */
int nat_mass_energy(nat_solver* s, double* mass, double* kinetic_energy);

/* Allocation-free variant of nat_mass_energy.  No counterpart in the
 * reference.  For callers that cannot allocate device memory where they need
 * the diagnostics: work recorded into a CUDA graph (cudaMalloc is not allowed
 * during stream capture), hosts whose framework owns all device memory
 * through its own pool, and loops that cannot pay for cudaMalloc's implicit
 * synchronisation.  Inputs: rho (n) and u (dim * n) in device memory, in the
 * device lattice order (n_axis[a] nodes per axis, periodic FE_Q duplicates
 * folded: N_a p per axis, DG: N_a (p+1)); output: out_dev[0] = mass,
 * out_dev[1] = kinetic energy, in device memory, written on cuda_stream.
 * The only scratch is a 64 KiB file-scope device array that every GPU
 * loading the library holds until exit; inputs above NAT_NOALLOC_MAX_NODES
 * nodes are rejected (NAT_ERR_INVALID_ARG), and so is an axis whose node count
 * is not a whole number of cells (a multiple of p for FE_Q, of p + 1 for DG).
 * The first call on a device looks up the array's device address (make it
 * before any stream capture; after a cudaDeviceReset the next call looks it
 * up again); calls whose kernels overlap on the GPU share the array and race.
 * Calls no cudaMalloc / cudaFree.  Deterministic: fixed reduction order.  The node
 * weights are those of the Cartesian box (cell_size); a mapped mesh's
 * weights depend on its cells' Jacobians: use nat_mass_energy there. */
#define NAT_NOALLOC_MAX_NODES 16777216LL
int nat_mass_energy_noalloc(const double* rho_dev, const double* u_dev, int dim, const int n_axis[3],
                            int order, int topology, const double cell_size[3], double* out_dev,
                            void* cuda_stream);

/* ---- wall boundaries ----------------------------------------------------
 * Faces of a non-periodic axis: 0 x-, 1 x+, 2 y-, 3 y+, 4 z-, 5 z+.  A
 * departure path that meets a wall is handled as SemiLagrangian::
 * fillSparseObject does (advection/SemiLagrangian.cpp:354-399):
 *   NAT_BC_VELOCITY_BOUNCE_BACK (boundaries/VelocityNeqBounceBack.h): the path
 *     reverses at the wall and takes the opposite population; the wall adds
 *     2 w_alpha rho_w (e_alpha . u_wall) / c_s^2 with rho_w = 1, scaled units
 *     (VelocityNeqBounceBack.cpp:137-194);
 *   NAT_BC_DO_NOTHING (boundaries/DoNothingBoundary.h): the population is taken
 *     from x + dt e_alpha instead.
 * The two-population model streams g through the same rows, without the
 * wall term.  Those rows are evaluated after the interior streaming. */
#define NAT_BC_VELOCITY_BOUNCE_BACK 1
#define NAT_BC_DO_NOTHING 2
int nat_set_boundary(nat_solver* s, int face, int kind, const double u_wall[3]);

/* Constant body force (ProblemDescription::setExternalForce with
 * ConstantExternalForce; SolverConfiguration::setForcingScheme), applied by
 * the advanced collision of the time loop (collision_advanced/
 * CollisionOperator.h:76-90, AuxiliaryCollisionFunctions.h:332-414):
 *   NAT_FORCE_SHIFTING_VELOCITY: equilibrium velocity u + tau dt F / rho;
 *   NAT_FORCE_EXACT_DIFFERENCE: after relaxation
 *     f += f^eq(rho, u + dt F / rho) - f^eq(rho, u);
 *   NAT_FORCE_GUO: the legacy BGKStandard::collideAll scheme
 *     (collision/BGKStandard.cpp:128-133, 222-225 for D2Q9; :374-380,
 *     470-473 for D3Q19; the advanced path throws for it): equilibrium velocity
 *     u' = u + dt F / (2 rho), then f_i += dt w_i (1 - omega/2) (p (e_i.F - u'.F)
 *     + p^2 (e_i.u')(e_i.F)), p = scaling / c_s^2, with unit e_i and scaled u',
 *     F (collision/ExternalForceFunctions.h:119-200).  D2Q9 and D3Q19 only
 *     (the reference sends D3Q27 to the generic BGK::collideAll, which has no
 *     force).  For D3Q19 the reference adds the source term to a copy that it
 *     does not store, so only the shifted equilibrium acts: kept as written.
 * All report u + dt F / (2 rho).  force[0..D-1] in scaled units (like u).
 * BGK_STANDARD only (NAT_ERR_UNSUPPORTED otherwise).  Not applied with
 * a prescribed velocity (nat_collide with in_init).  With a force the step
 * runs in the generic fused kernel.  NAT_FORCE_NONE switches it off. */
#define NAT_FORCE_NONE 0
#define NAT_FORCE_SHIFTING_VELOCITY 1
#define NAT_FORCE_EXACT_DIFFERENCE 2
#define NAT_FORCE_GUO 3
int nat_set_force(nat_solver* s, int scheme, const double force[3]);

/* ---- compressible two-population model (NAT_BGK_COMPRESSIBLE) ---------- */
/* Equilibrium of the collision (SolverConfiguration equilibrium scheme). */
#define NAT_EQ_BGK 0     /* second order, collision_advanced/Equilibria.h:66-83 */
#define NAT_EQ_QUARTIC 1 /* quartic with temperature, Equilibria.h:88-267 (default) */

/* Model settings; the defaults are the reference's SolverConfiguration
 * defaults (solver/SolverConfiguration.cpp:21-31): gamma 1.4, Prandtl 1.0 with
 * the Prandtl correction off, Sutherland law off; quartic equilibrium. */
typedef struct nat_thermal {
  double gamma;       /* heat capacity ratio; C_v = 1 / (gamma - 1) */
  double prandtl;     /* Prandtl number, used when prandtl_set != 0 */
  int prandtl_set;    /* apply the f*, g* correction (CollisionSchemes.h:63-79, 103-116) */
  int sutherland_set; /* tau_visc scaled by (T / 0.85)^0.7 (CollisionSchemes.h:81-88) */
  int equilibrium;    /* NAT_EQ_QUARTIC or NAT_EQ_BGK */
} nat_thermal;

/* Set / read the model settings of a NAT_BGK_COMPRESSIBLE handle. */
int nat_set_thermal(nat_solver* s, const nat_thermal* t);
int nat_get_thermal(const nat_solver* s, nat_thermal* t);

/* Second population g (CompressibleCFDSolver::m_g): same layout as f. */
int nat_upload_g(nat_solver* s, const double* g_host);
int nat_download_g(nat_solver* s, double* g_host);

/* Temperature T (n_ref) and shock-sensor mask (n_ref, the Knudsen estimate of
 * AuxiliaryCollisionFunctions.h:474-481) written by the last collision. */
int nat_download_thermal(nat_solver* s, double* T_host, double* mask_host);

/* CompressibleCFDSolver::initializeDistributions (CompressibleCFDSolver.h:849-899),
 * EQUILIBRIUM scheme: f = f^eq(rho, u, T) of the quartic equilibrium and
 * g = f^eq T (2 C_v - D) at every node, computed on the device from host
 * fields rho (n_ref), u (D * n_ref, scaled) and T (n_ref); also stores rho, u
 * and T on the device. */
int nat_init_thermal(nat_solver* s, const double* rho_host, const double* u_host, const double* T_host);

/* nat_stream on such a handle streams f and g (stream() + gStream());
 * nat_collide runs collideAll(f, g, rho, u, T, mask) (with in_init the
 * velocity comes from the device copy of u, as set by nat_upload_macro);
 * nat_step fuses stream(f), stream(g) and collide into one kernel per step. */

/* ---- checkpoint and output ----------------------------------------------
 * Checkpoint (solver/Checkpoint.cpp:74-112 writes a status file with
 * iteration, time, stencil scaling and FE order, and the f vectors): one
 * binary file with a header (those fields plus the lattice) and f (and g for
 * NAT_BGK_COMPRESSIBLE) in the reference layout, FP64.  Loading checks that
 * lattice, stencil, order and scaling are the handle's, and for a mapped
 * mesh its vertex grid (by a hash of the vertex array's bytes). */
int nat_checkpoint_save(nat_solver* s, const char* path, int64_t iteration, double time);
int nat_checkpoint_load(nat_solver* s, const char* path, int64_t* iteration, double* time);

/* Solution output (CFDSolver.cpp:1001-1069 writes rho, ux, uy[, uz] with
 * deal.II's DataOut): an ASCII VTK unstructured-grid file whose points are
 * the lattice nodes (reference layout) and whose cells are the p^D sub-cells
 * between neighbouring nodes of every element; point data rho, ux, uy[, uz]
 * and, for NAT_BGK_COMPRESSIBLE, T and shock_sensor, from the last collision. */
int nat_write_vtu(nat_solver* s, const char* path);

/* Departure-point rows of a mapped one-population mesh (no counterpart in
 * the reference, whose tracker fills the sparse matrix directly,
 * SemiLagrangian.cpp:145-522): searched again by the host tracker (where = 0,
 * all host threads) or the device tracker (where = 1, one GPU thread per
 * row; the one nat_create uses), without changing the handle's own rows, and
 * copied to the host arrays that are not NULL.  Rows are direction-major,
 * node-minor: (Q-1) n_dev of them.  base: int32 per row; flags: uint8 per row;
 * u: per row D unit coordinates (float, NAT_FP32_DEV) or D (p+1) 1-D Lagrange
 * values (double, NAT_FP64), stored [row direction][axis][j][node]; c: per row
 * the additive constant (float deviation form / double plain).  Both trackers
 * use the same code without floating-point contraction and give the same rows
 * bit for bit.  NAT_ERR_UNSUPPORTED for other handles. */
int nat_mapped_rows(nat_solver* s, int where, int32_t* base, void* u, void* c, uint8_t* flags);

/* Device pointers of the current distribution buffer (Q blocks of n_dev
 * values, double for NAT_FP64 and float (f - w_i) for NAT_FP32_DEV).  The
 * buffer changes with every step and every nat_upload_f (which converts into
 * a spare buffer on its own streams and then makes it the current one), so
 * the pointer is valid until the next of those calls. */
int nat_device_f(nat_solver* s, void** f_dev);

/* Kernel choice for the fused step: 0 = automatic (a specialised kernel --
 * row-segment or tile -- when an instantiation for this stencil / model /
 * order / topology exists and every departure point lies in the node's own
 * or the adjacent upwind cell, the generic kernel otherwise), 1 = generic
 * kernel only, 2 = specialised kernel required (NAT_ERR_UNSUPPORTED when
 * none applies), 3 = tile kernel required, 4 = row-segment kernel required,
 * 6 = bulk-copy row-segment kernel required (3-D stencils; per-warp
 * cp.async.bulk pipeline of the source rows), 7 = row-group kernel required
 * (3-D, FP32: 2-4 warps own a whole x row, no halo recomputation), 11 =
 * cell-row kernel required (3-D: a lane owns one cell's nodes along x, p + 1
 * in DG, p in FE_Q, a warp whole periodic x rows of 16 or 32 cells, or two
 * (four) warps a row of 64 (128); vector
 * loads of cell rows, the x window by warp shuffles), 12 = the cell-row kernel with the 8
 * corner directions of D3Q27 (FP32 deviation storage, DG p = 3, 32 cells per
 * x row) applied as dense per-cell operator tiles on the tensor cores
 * (mma.sync m16n8k8, operands split into two TF32 halves, FP32
 * accumulation; slower than 11 and short of its accuracy, so only taken
 * when asked for), 13 = the cell-row kernel with z sharing: the z-window sums
 * of the yz-diagonal directions computed once per CTA for all its rows. */
int nat_set_kernel_variant(nat_solver* s, int variant);
/* The fused-step kernel in use: 1 generic, 2 tile, 3 row-segment,
 * 5 two-population row-segment kernel (NAT_BGK_COMPRESSIBLE; 9 and 10: its
 * FP32 forms with f and g in shared memory, 20 / 24 resident warps per SM;
 * 14: its FP32 register form at order 2 with the window rows copied into
 * shared memory asynchronously, one direction ahead),
 * 6 bulk-copy row-segment kernel, 7 row-group kernel, 8 departure-point
 * kernel of mapped (MappingQ1) meshes, 11 cell-row kernel, 12 cell-row
 * kernel with tensor-core corner directions, 13 cell-row kernel with z
 * sharing.  nat_autotune chooses among 5, 9 and 10 (and 14 at order 2) for
 * an FP32 two-population handle; nat_select_candidate takes their index
 * 0-2 (3). */
int nat_kernel_variant(const nat_solver* s);

/* Autotuner: times `steps` fused steps with every kernel that applies to
 * this configuration (each specialised tile shape and the generic kernel),
 * keeps the fastest, and restores f and the status word afterwards.  Writes
 * the number of candidates and the index of the chosen one (the generic
 * kernel is the last) when the pointers are not NULL.  Synchronises.  The
 * trial steps run on the solver's own buffers (no allocation). */
int nat_autotune(nat_solver* s, int steps, int* n_candidates, int* chosen);

/* Report of the last nat_autotune (no counterpart in the reference): returns
 * the number of candidates timed and writes, for the first `max` of them,
 * the mean ms per step (L2-warm, back-to-back steps) and five ints each in
 * desc: kernel variant, nodes per CTA along x, y, z, threads per CTA.
 * Either pointer may be NULL; -1 for a NULL handle. */
int nat_autotune_report(const nat_solver* s, int max, float* ms_per_step, int* desc);

/* Use candidate `index` of the list nat_autotune times (same order, same
 * variant filter; no counterpart in the reference): a fixed, reproducible
 * kernel choice without timing, and the way the tests reach every kernel. */
int nat_select_candidate(nat_solver* s, int index);

/* The fused-step kernel in use: variant (1 generic, 2 tile, 3 row-segment),
 * nodes per CTA along each axis, threads per CTA, dynamic shared memory. */
int nat_kernel_info(const nat_solver* s, int* variant, int tile_nodes[3], int* threads,
                    int64_t* smem_bytes);

/* Number of kernels this handle has launched (for launch accounting). */
int64_t nat_launch_count(const nat_solver* s);

/* ---- continuous-batching server (independent 2-D solves) ---------------
 * Serving workload of the spec: many independent periodic D2Q9 solves
 * of uneven size, order and model, admitted by their HBM footprint into a
 * device pool and advanced together, one persistent graph-captured launch
 * per server step.  No reference counterpart: the reference runs one solve
 * per process (solver/CFDSolver.cpp). */
#define NAT_INIT_TAYLOR_GREEN 0 /* benchmarks/TaylorGreenVortex2D.cpp:36-59 */
#define NAT_INIT_SHEAR_LAYER 1  /* benchmarks/ShearLayer2D.cpp:39-53 */

typedef struct nat_request {
  int stencil;      /* NAT_D2Q9 */
  int collision;    /* NAT_BGK_STANDARD or NAT_KBC_STANDARD */
  int order;        /* FE_Q order 1..6 */
  int cells[2];
  double length[2];
  double scaling;   /* stencil scaling (sqrt(3)/Ma for unit velocity) */
  double viscosity;
  double cfl;       /* dt = CFL h_min / (sqrt(2) scaling p^2) when dt <= 0 */
  double dt;
  int steps;        /* time steps to run */
  int init;         /* NAT_INIT_TAYLOR_GREEN or NAT_INIT_SHEAR_LAYER */
  double Ma;        /* density amplitude of the Taylor-Green state */
  double u0;        /* velocity amplitude (scaled units) */
  double kappa;     /* shear layer: tanh steepness */
  double delta;     /* shear layer: perturbation amplitude */
} nat_request;

typedef struct nat_server_stats_t {
  int64_t pending, live, completing, finished;
  int64_t steps, node_updates;
  int64_t pool_used, pool_bytes;
  int64_t launches;
  /* step graphs instantiated, step graphs updated in place (same non-empty
   * groups), and host time spent rebuilding work lists and graphs (ns) */
  int64_t graph_builds, graph_updates, rebuild_ns;
} nat_server_stats_t;

typedef struct nat_server nat_server;

/* Create a server with a device pool of pool_bytes and at most max_slots
 * live solves on the current device. */
int nat_server_create(size_t pool_bytes, int max_slots, nat_server** out);
int nat_server_destroy(nat_server* s);
/* Queue a request; admitted in submission order as slots and pool memory
 * free up. */
int nat_server_submit(nat_server* s, const nat_request* r, int64_t* id);
/* One server step: collect finished results, admit queued requests, advance
 * every live solve by one time step (one graph launch: a kernel per group of
 * live solves with the same order and collision model). */
int nat_server_step(nat_server* s);
/* Up to max_steps server steps in one call (no counterpart in the
 * reference); stops early when no solve is live.  *steps_done (may be NULL)
 * receives the number run.  The host runs at most 64 steps ahead of the
 * device. */
int nat_server_run(nat_server* s, int max_steps, int* steps_done);
/* Ids of finished requests (up to max_ids); wait != 0 blocks until every
 * solve that has run its last step is copied out. */
int nat_server_poll(nat_server* s, int64_t* ids, int max_ids, int* n_done, int wait);
/* Copy a finished request's rho (n_nodes) and scaled u (2 * n_nodes) out
 * (device lattice order, periodic duplicates folded) and release it; status
 * is the solve's own (NAT_OK or NAT_ERR_DENSITY_UNDERFLOW / NAT_ERR_NAN /
 * NAT_ERR_UNSUPPORTED). rho / u may be NULL to query n_nodes. */
int nat_server_result(nat_server* s, int64_t id, double* rho, double* u, int64_t* n_nodes, int* status);
int nat_server_stats(const nat_server* s, nat_server_stats_t* st);
int nat_server_last_error(const nat_server* s, char* buf, size_t len);

/* Library version string. */
const char* nat_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NATGPU_H */
