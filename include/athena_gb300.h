/* athena_gb300.h -- C ABI of the GB300-native finite-volume (M)HD stage update and
 * multigrid Poisson solve.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes (0 = ok, <0 =
 * error, message from athg_last_error()). No exceptions cross this boundary. All
 * MeshBlock state lives in one device pool owned by the context; host code holds
 * handles and exchanges arrays in the reference's AthenaArray layout (n,k,j,i), i
 * fastest, ghosts included, so problem generators and outputs keep working.
 *
 * Every entry point names the reference interface it replaces (paths are relative to
 * the reference's src/). The reference calls these per MeshBlock from its TaskList;
 * here one call covers every block of the pool, stream-ordered on the context's CUDA
 * stream. One host thread per context.
 */
#ifndef ATHENA_GB300_H_
#define ATHENA_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ATHG_OK 0
#define ATHG_ERR_ARG (-1)    /* invalid argument or unsupported configuration */
#define ATHG_ERR_CUDA (-2)   /* CUDA runtime error */
#define ATHG_ERR_STATE (-3)  /* call out of order (e.g. no blocks yet) */
#define ATHG_ERR_DEVICE (-4) /* a kernel reported an error through the device error word
                                (a TMA load that timed out, a time step that is not a
                                positive finite number, a non-finite density or pressure);
                                reported by the next call that synchronises the context's
                                stream: athg_get_time, athg_synchronize */

/* Riemann solvers (configure.py --flux) */
enum { ATHG_HLLE = 0, ATHG_HLLC = 1, ATHG_HLLD = 2, ATHG_LHLLC = 3, ATHG_LHLLD = 4 };
/* time integrators (<time> integrator) */
enum { ATHG_VL2 = 0, ATHG_RK1 = 1, ATHG_RK2 = 2, ATHG_RK3 = 3 };
/* arithmetic of reconstruction/Riemann fluxes: FP64 (the reference's, bit for bit); FP32
 * with FP64 state + CT (mixed); or double-float (pairs of FP32 values, ~48 bits, on the FP32
 * pipe) with FP64 state (on uniform periodic meshes without source terms the update,
 * primitive recovery and time step in double-float too, each new state value FP64 base
 * minus a double-float increment): the FP64 path's accuracy, including for waves near the
 * FP32 resolution of their background (donor cell or PLM; HLLC/HLLE hydro, HLLD/HLLE MHD).
 * ATHG_DFLOAT has no counterpart in the reference. */
enum { ATHG_FP64 = 0, ATHG_MIXED = 1, ATHG_DFLOAT = 2 };
/* arrays exchanged with the host, per block, AthenaArray layout with ghosts:
 * CONS (5,nc3,nc2,nc1)  B1F (nc3,nc2,nc1+1)  B2F (nc3,nc2+1,nc1)  B3F (nc3+1,nc2,nc1)
 * PRIM (5,nc3,nc2,nc1)  BCC (3,nc3,nc2,nc1)  PHI (nc3,nc2,nc1)   nc = nx + 2*nghost */
enum {
  ATHG_VAR_CONS = 0, ATHG_VAR_B1F = 1, ATHG_VAR_B2F = 2, ATHG_VAR_B3F = 3,
  ATHG_VAR_PRIM = 4, ATHG_VAR_BCC = 5, ATHG_VAR_PHI = 6
};

typedef struct athg_ctx athg_ctx;

/* Compile-time physics of the reference (configure.py, src/defs.hpp.in) plus the
 * runtime keys of <time>/<hydro> the stage needs. */
typedef struct {
  int nx1, nx2, nx3;  /* MeshBlock interior size (<meshblock> nx1..nx3); same for all blocks */
  int nghost;         /* NGHOST (2 for PLM, >= 3 for PPM) */
  int magnetic;       /* MAGNETIC_FIELDS_ENABLED */
  int rsolver;        /* ATHG_HLLE; ATHG_HLLC / ATHG_LHLLC (hydro); ATHG_HLLD / ATHG_LHLLD (MHD).
                         The L- solvers are the fork's low-dissipation variants with the
                         velocity-difference shock detector */
  int xorder;         /* <time> xorder: 1 donor cell, 2 PLM, 3 PPM */
  int integrator;     /* ATHG_VL2 / ATHG_RK1 / ATHG_RK2 / ATHG_RK3 */
  int precision;      /* ATHG_FP64 or ATHG_MIXED */
  double gamma;       /* <hydro> gamma */
  double dfloor, pfloor; /* <hydro> dfloor, pfloor (default sqrt(1024*FLT_MIN)) */
  double cfl_number;  /* <time> cfl_number, already limited to the integrator's limit */
  double tlim;        /* <time> tlim: the last dt is clamped to reach it */
} athg_config;

/* One MeshBlock: reference MeshBlock::loc, block_size and the neighbour table of
 * BoundaryBase (src/bvals/bvals_base.cpp). */
typedef struct {
  int64_t lx1, lx2, lx3;
  int32_t level;
  double dx1, dx2, dx3;          /* uniform cell widths (coordinates.cpp:127-145) */
  const double *x1f, *x2f, *x3f; /* host arrays of face positions incl. ghosts, nc+1 each */
  int32_t neighbor[27];          /* same-level neighbour block id, -1 if none; index
                                    (ox3+1)*9 + (ox2+1)*3 + (ox1+1) */
} athg_block;

/* A uniform single-level mesh (<mesh> and <meshblock>), built the way the reference's
 * Mesh constructor lays out a root grid (src/mesh/mesh.cpp:1664-1760 block sizes,
 * src/coordinates/coordinates.cpp:88-150 face positions). */
typedef struct {
  int nx1, nx2, nx3;                         /* <mesh> nx1..nx3 */
  double x1min, x1max, x2min, x2max, x3min, x3max;
  int periodic[3];                           /* per axis: 1 periodic (ix/ox_bc = periodic);
                                                0 outflow on both sides (ix/ox_bc = outflow,
                                                bvals/cc/outflow_cc.cpp, bvals/fc/
                                                outflow_fc.cpp; precision ATHG_FP64 or
                                                ATHG_DFLOAT, uniform meshes). Other
                                                values are rejected with ATHG_ERR_ARG */
} athg_mesh;

/* A static-refinement region (<refinementN> x1min..x3max, level >= 1). */
typedef struct {
  double x1min, x1max, x2min, x2max, x3min, x3max;
  int level;
} athg_region;

/* ---- context and pool ---------------------------------------------------------- */
int athg_create(const athg_config* cfg, athg_ctx** out);
int athg_destroy(athg_ctx* ctx);
/* Replaces the per-block allocation of Hydro/Field/EOS (hydro/hydro.cpp:31,
 * field/field.cpp, mesh/meshblock.cpp:47): allocates every block in one device pool. */
int athg_set_blocks(athg_ctx* ctx, int nblocks, const athg_block* blocks);
/* Builds the blocks of a uniform mesh (Mesh::Mesh block layout, SetBlockSizeAndBoundaries
 * mesh/mesh.cpp:1668, Coordinates ctor) and calls athg_set_blocks. Blocks are ordered
 * with lx1 fastest, then lx2, then lx3. */
int athg_set_uniform_mesh(athg_ctx* ctx, const athg_mesh* mesh);
/* Static mesh refinement (<mesh> refinement = static): the root grid of `mesh`, refined
 * where `regions` say, with the leaves and their 2:1 balance of Mesh::Mesh
 * (mesh/mesh.cpp:334-462, mesh/meshblock_tree.cpp) and the level-boundary work of
 * bvals/bvals_refine.cpp, bvals/cc/flux_correction_cc.cpp and bvals/fc/flux_correction_fc.cpp
 * done on the device (ghost fill through coarse buffers, prolongation, flux and EMF
 * correction). Periodic boundaries only; FP64 or mixed precision (on the mixed path the
 * level-boundary flux and EMF corrections are FP32, conservative to FP32 rounding of the
 * boundary fluxes). Blocks are ordered by level,
 * then lx3, lx2, lx1 (athg_block_location gives each one). */
int athg_set_refined_mesh(athg_ctx* ctx, const athg_mesh* mesh, int nregions,
                          const athg_region* regions);
/* The same for an explicit list of leaves, as the reference's MeshBlockTree holds them:
 * locs[4*b .. 4*b+3] = level (relative to the root grid), lx1, lx2, lx3 of block b. */
int athg_set_multilevel_blocks(athg_ctx* ctx, const athg_mesh* mesh, int nblocks,
                               const int64_t* locs);
/* Adaptive refinement (<mesh> refinement = adaptive) with the blast's criterion
 * (pgen/blast.cpp:413-442): a block is flagged for refinement where max |grad p| / p over
 * its cells exceeds `threshold`, for derefinement below deref_fraction * threshold;
 * MeshRefinement::CheckRefinementCondition (derefinement counters, no derefinement next to
 * finer blocks), Mesh::UpdateMeshBlockTree / MeshBlockTree::Refine / Derefine and the data
 * of new blocks (FillSameRankCoarseToFineAMR / FineToCoarseAMR) follow the reference. */
typedef struct {
  double threshold;       /* <problem> thr */
  double deref_fraction;  /* 0.25 in the reference's blast */
  int max_level;          /* levels above the root: <mesh> numlevel - 1 */
  int derefine_count;     /* <mesh> derefine_count (the reference's default is 10) */
} athg_amr_config;
/* Turns adaptive refinement on (FP64, periodic); a uniform mesh keeps its state. From
 * then on athg_cycles checks the criterion after every cycle and regrids (the main loop's
 * LoadBalancingAndAdaptiveMeshRefinement + NewTimeStep); blocks may change order and
 * number (athg_num_blocks, athg_block_location). */
int athg_amr_enable(athg_ctx* ctx, const athg_amr_config* cfg);
/* One refinement check and regrid on the current state, with Mesh::Initialize(2) after a
 * change (the initial refinement loop of Mesh::Initialize): *changed = 1 if the mesh
 * changed. */
int athg_amr_regrid(athg_ctx* ctx, int* changed);
/* ---- FFT over the whole uniform periodic mesh (cuFFT) ------------------------------ */
/* Turbulence driving (fft/turbulence.cpp, <problem> turb_flag and the <turbulence> block):
 * a power-law spectrum with Gaussian amplitudes and uniform phases from std::mt19937_64
 * (the same sequence as the reference for a given rseed >= 0), optional projection onto
 * compressive/shear parts, Ornstein-Uhlenbeck smoothing in time, transformed to a velocity
 * perturbation that is mean-free in momentum and scaled to inject dedt (per unit time for
 * driven turbulence) into the kinetic energy. */
typedef struct {
  int turb_flag;   /* 1 decaying (once at athg_initialize), 2 impulsive every dtdrive,
                      3 continuous (every cycle) */
  int64_t rseed;   /* <turbulence> rseed; < 0 seeds from std::random_device */
  int nlow, nhigh; /* <turbulence> nlow (0), nhigh (mesh nx1 / 2): kept shells */
  double dtdrive;  /* <turbulence> dtdrive (turb_flag 2) */
  double tcorr;    /* <turbulence> tcorr: OU correlation time (turb_flag > 1) */
  double f_shear;  /* <turbulence> f_shear: shear fraction; < 0 no projection */
  double expo;     /* <turbulence> expo (2) */
  double dedt;     /* <turbulence> dedt */
} athg_turb_config;
/* Attaches the driver (uniform single-level mesh whose blocks tile `mesh`; FP64 state).
 * athg_initialize then drives once for turb_flag 1 and 2 (mesh/mesh.cpp:1383-1384) and
 * athg_cycles drives before every cycle for turb_flag > 1 (main.cpp:457). cfg NULL detaches. */
int athg_turb_attach(athg_ctx* ctx, const athg_mesh* mesh, const athg_turb_config* cfg);
/* One TurbulenceDriver::Driving at the current time and dt. */
int athg_turb_drive(athg_ctx* ctx);
/* FFT self-gravity (SELF_GRAVITY_ENABLED == 1, gravity/fft_gravity.cpp): Poisson's equation
 * with the 7-point Laplacian's eigenvalues, periodic, solved after every stage and in
 * athg_initialize like the multigrid coupling (replaces it); four_pi_G = 0 detaches. */
int athg_attach_fft_gravity(athg_ctx* ctx, const athg_mesh* mesh, double four_pi_G);
/* Sizes of the multi-level work lists (all 0 on a single-level mesh): out[0..7] = ghost-fill
 * elements, same-level restrictions, flux corrections, EMF corrections, coarse cells
 * converted to primitives, prolongated cells, internal-field cells, fine cells rebuilt. */
int athg_smr_stats(athg_ctx* ctx, int64_t* out8);
int athg_num_blocks(const athg_ctx* ctx, int* nblocks);
/* logical location of block b: out[0..3] = lx1, lx2, lx3, level */
int athg_block_location(const athg_ctx* ctx, int block, int64_t* out);
/* Number of doubles one block holds for var (see ATHG_VAR_*). */
int athg_var_size(const athg_ctx* ctx, int var, size_t* count);
/* Host <-> device copies of one block (block >= 0) or of all blocks back to back
 * (block = -1). count is the number of doubles in host. */
int athg_upload(athg_ctx* ctx, int block, int var, const double* host, size_t count);
int athg_download(athg_ctx* ctx, int block, int var, double* host, size_t count);

/* ---- the stage (TaskList) --------------------------------------------------------- */
/* Tail of Mesh::Initialize (mesh/mesh.cpp:1405-1649): ghost exchange, W(U) over interior
 * and ghosts, first NewBlockTimeStep and Mesh::NewTimeStep. */
int athg_initialize(athg_ctx* ctx);
/* Mesh::Initialize after a restart (res_flag = 1, mesh/mesh.cpp:1367-1656): the same, but
 * time, dt and ncycle keep the values set by athg_set_time (read from the restart file),
 * and the first Mesh::NewTimeStep starts from that dt. */
int athg_resume(athg_ctx* ctx);
/* One stage (1-based) of TimeIntegratorTaskList::DoTaskListOneStage
 * (task_list/task_list.cpp:66) over every block: CalculateHydroFlux (donor cell on the
 * first VL2 stage), CalculateEMF, IntegrateHydro, IntegrateField, ghost exchange,
 * Primitives, and on the last stage NewBlockTimeStep (time_integrator.cpp:1460-2093). */
int athg_stage(athg_ctx* ctx, int stage);
/* main.cpp:478-485: time += dt, ncycle++, Mesh::NewTimeStep (mesh/mesh.cpp:1078). */
int athg_end_cycle(athg_ctx* ctx);
/* n whole cycles (all stages + athg_end_cycle) replayed from one captured CUDA graph;
 * time, dt and ncycle stay on the device. */
int athg_cycles(athg_ctx* ctx, int n);
/* Current time, dt and cycle count (synchronises the context's stream). */
int athg_get_time(athg_ctx* ctx, double* time, double* dt, int64_t* ncycle);
int athg_set_time(athg_ctx* ctx, double time, double dt, int64_t ncycle);
int athg_synchronize(athg_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that time or order work. */
int athg_stream(athg_ctx* ctx, void** stream);
/* One whole cycle run launch group by launch group (not from the captured graph), with
 * CUDA events on the context's stream between groups: device time of each group in ms,
 * in launch order (ms[0..*n-1], at most max), and the groups' names, '\n'-separated, in
 * `names` (names_size bytes, may be NULL). The cycle is a real one: the state advances. */
int athg_cycle_timing(athg_ctx* ctx, int max, double* ms, int* n, char* names,
                      size_t names_size);
/* Kernel launches of one whole cycle (what athg_cycles replays per cycle). */
int athg_launches_per_cycle(athg_ctx* ctx, int* n);

/* ---- individual operators (each over every block) -------------------------------- */
/* Hydro::CalculateFluxes(w, b, bcc, order) (hydro/hydro.hpp:72-73) */
int athg_calculate_fluxes(athg_ctx* ctx, int order);
/* Field::ComputeCornerE(w, bcc) (field/field.hpp:67) */
int athg_compute_corner_e(athg_ctx* ctx);
/* MeshBlock::WeightedAve + Hydro::AddFluxDivergence + Field::CT for stage `stage`
 * (mesh/weighted_ave.cpp:33,238; hydro/hydro.hpp:67; field/field.hpp:65) */
int athg_integrate(athg_ctx* ctx, int stage);
/* BoundaryVariable::Send/ReceiveBoundaryBuffers for U and face B (bvals/bvals_var.cpp:212) */
int athg_exchange_ghosts(athg_ctx* ctx);
/* EquationOfState::ConservedToPrimitive (eos/eos.hpp:37-40) incl. cell-centred B */
int athg_conserved_to_primitive(athg_ctx* ctx);
/* Hydro::NewBlockTimeStep (hydro/hydro.hpp:66) reduced over all blocks: min CFL dt */
int athg_new_block_dt(athg_ctx* ctx, double* dt_out);

/* ---- diagnostics ------------------------------------------------------------------- */
/* max over interior cells of |div B| * dx (the CT invariant) */
int athg_max_div_b(athg_ctx* ctx, double* out);
/* volume integrals of the 5 conserved variables over all interior cells (history) */
int athg_sum_conserved(athg_ctx* ctx, double* out5);

/* ---- multigrid Poisson solver (self-gravity) ----------------------------------------
 * Replaces MGGravityDriver::Solve (gravity/mg_gravity.cpp:166-211) and the Multigrid
 * primitives it drives (multigrid/multigrid.hpp:120-129): red-black Gauss-Seidel smoother
 * (omega = 1.15), defect, restriction, trilinear prolongation, FMG prolongation, V(1,1)
 * and FMG cycles, defect norms, periodic / zero-gradient / zero-fixed / multipole
 * (l <= 4) boundaries. The mesh is cubic with 2^L cells per side; each level is one
 * device grid with one ghost layer (the reference's per-MeshBlock levels plus root grid
 * visit the same uniform levels on such a mesh). Solves  lap(phi) = src. */
enum { ATHG_MG_PERIODIC = 0, ATHG_MG_ZEROGRAD = 1, ATHG_MG_ZEROFIXED = 2, ATHG_MG_MULTIPOLE = 3 };
enum { ATHG_MG_FMG = 0, ATHG_MG_MGI = 1 };

typedef struct athg_mg athg_mg;

typedef struct {
  int nx;                 /* cells per side, a power of two (<mesh> nx1 = nx2 = nx3) */
  double x1min, x1max, x2min, x2max, x3min, x3max;
  int bc[6];              /* <gravity> ix1_bc, ox1_bc, ix2_bc, ox2_bc, ix3_bc, ox3_bc */
  int mporder;            /* <gravity> mporder: 2 or 4 (multipole boundaries only) */
  int auto_mporigin;      /* <gravity> auto_mporigin: expand about the centre of mass */
  int nodipole;           /* <gravity> nodipole */
  double mporigin[3];     /* <gravity> mporigin_x1..x3 when auto_mporigin = 0 */
  int mode;               /* <gravity> mgmode: ATHG_MG_FMG or ATHG_MG_MGI */
  double threshold;       /* <gravity> threshold: >= 0 iterate until the L2 defect <= it
                             (0: until convergence stalls); < 0: niteration cycles */
  int niteration;         /* <gravity> niteration */
  int precision;          /* ATHG_FP64: the reference's FP64 cycle; ATHG_MIXED: FP32 V-cycles
                             on the FP64 defect, corrections accumulated in FP64 */
} athg_mg_config;

int athg_mg_create(const athg_mg_config* cfg, athg_mg** out);
int athg_mg_destroy(athg_mg* mg);
/* Multigrid::LoadSource (multigrid/multigrid.cpp:194): src = fac * rho on the finest
 * level; rho is the nx^3 interior, i fastest. */
int athg_mg_load_source(athg_mg* mg, const double* rho, size_t count, double fac);
/* Multigrid::LoadFinestData: initial guess for ATHG_MG_MGI (nx^3 interior). */
int athg_mg_set_phi(athg_mg* mg, const double* phi, size_t count);
/* MGGravityDriver::Solve after LoadSource: SetupMultigrid, FMG and/or iterations,
 * average subtraction; returns V-cycles done and the final L2 defect norm. */
int athg_mg_solve(athg_mg* mg, int* iterations, double* defect_norm);
/* n V(1,1) cycles on the finest level (MultigridDriver::SolveVCycle). */
int athg_mg_vcycles(athg_mg* mg, int n);
/* MultigridDriver::CalculateDefectNorm(l2) of the current solution. */
int athg_mg_defect_norm(athg_mg* mg, double* out);
/* Multigrid::RetrieveResult: the nx^3 interior of phi. */
int athg_mg_get_phi(athg_mg* mg, double* phi, size_t count);
int athg_mg_stream(athg_mg* mg, void** stream);
/* Multipole coefficients (25) and expansion origin (3), after a solve. */
int athg_mg_multipole(athg_mg* mg, double* out28);

/* Launch shape of the flux sweeps: out3/in3 = {threads per block of the x1 sweep (64 or
 * 128), of the marching x2/x3 sweeps (64 or 128), faces per marching segment (0: whole
 * pencil)}. No counterpart in the reference. The mixed path autotunes one shape per
 * reconstruction order its integrator uses (VL2: donor cell, then xorder) before its first
 * captured cycle, every candidate timed on the context's own state; get returns the
 * xorder shape, set applies to every order and disables the autotuner. Results do not
 * depend on it. */
int athg_get_tuning(athg_ctx* ctx, int* out3);
int athg_set_tuning(athg_ctx* ctx, const int* in3);

/* Stage kernel of the mixed-precision VL2 MHD path (PLM, HLLD or HLLE) on a uniform mesh:
 * single = 1 runs each stage as one launch (reconstruction, Riemann fluxes, corner EMFs,
 * flux divergence, CT and primitive recovery on chip, W/bcc staged by TMA; where it
 * applies: two ghost layers, MeshBlock nx1 a multiple of 32 and nx2 of 8), single = 0 (the
 * default, faster on this GPU) the separate sweep, corner-EMF and update kernels. nseg:
 * k-segments per thread block of the single pass (a divisor of nx3; 0 = autotuned before
 * the first captured cycle). No counterpart in the reference (its stage is one loop nest
 * per MeshBlock). athg_get_stage_kernel reports whether the next cycle runs the single
 * pass. */
int athg_set_stage_kernel(athg_ctx* ctx, int single, int nseg);
int athg_get_stage_kernel(athg_ctx* ctx, int* single, int* nseg);

/* HistoryOutput::WriteOutputFile sums (outputs/history.cpp:45-130), reduced on the
 * device over all blocks' interior cells: out[0] mass, [1..3] momenta, [4..6] kinetic
 * energy per direction, [7] total energy, [8] 1/2 rho phi (0 without self-gravity),
 * [9..11] cell-centred magnetic energy per direction (0 for hydro). *count = 12.
 * The reference's columns are these without the entries its build does not have. */
int athg_history(athg_ctx* ctx, double* out, int* count);

/* Self-gravity (SELF_GRAVITY_ENABLED == 2 with <problem> four_pi_G, Mesh::SetFourPiG).
 * Couples mg to the hydro context: the solve of MGGravityDriver::Solve
 * (gravity/mg_gravity.cpp:166) runs in athg_initialize (mesh/mesh.cpp:1398-1402) and
 * after every stage (main.cpp:461-466), on u(IDN) * four_pi_G of all blocks, and
 * HydroSourceTerms::SelfGravity (hydro/srcterms/self_gravity.cpp:35) adds the
 * momentum and energy sources after each stage's flux divergence. The blocks must be
 * one refinement level tiling mg's nx^3 root grid (the same mesh). The potential of
 * each block, with one ghost layer, downloads as ATHG_VAR_PHI. mg must outlive the
 * coupling; pass mg = NULL to detach. Solves with a threshold or a multipole boundary
 * synchronise with the host, so athg_cycles then runs the stages without a graph. In
 * mixed precision with VL2 the source term runs inside the fused update (the potential
 * read as FP32 pairs), like the rest of the fused stage. */
int athg_attach_gravity(athg_ctx* ctx, athg_mg* mg, double four_pi_G);

/* ---- CFL time step of one caller-owned block, with no device allocation ------------
 * No counterpart in the reference: an addition for callers that cannot allocate device
 * memory (code that must not synchronise the device, which cudaMalloc and cudaFree may
 * do; a host whose device memory belongs to its own pool; a fixed memory budget). Computes the same minimum as
 * athg_new_block_dt (dx / (|v| + c_f) over the interior, times cfg->cfl_number) for ONE
 * block whose device arrays the caller owns, in the AthenaArray layout with ghosts, FP64:
 *   w (5,nc3,nc2,nc1) primitives; for MHD also bcc (3,nc3,nc2,nc1) and the face fields
 *   b1f (nc3,nc2,nc1+1), b2f (nc3,nc2+1,nc1), b3f (nc3+1,nc2,nc1); nc = nx + 2*nghost.
 * The result is written to dt_out, a device pointer, on `stream` (a cudaStream_t, NULL
 * for the default stream); nothing is synchronised.
 * Only cfg->nx1..nx3, nghost, magnetic, gamma and cfl_number are read.
 * Scratch is a fixed file-scope device array of 8192 doubles (64 KiB) that every GPU
 * loading this library keeps until exit; blocks of more than 16,777,216 interior cells
 * are rejected with ATHG_ERR_ARG. Every call looks up the array's device address in the
 * current context (cudaGetSymbolAddress, no allocation), so the entry point stays valid
 * after cudaDeviceReset; the first call on a device also loads this library's device code
 * there, so make that first call before any stream capture.
 * All calls share the array: calls that overlap on the GPU (e.g. on two streams) race. */
int athg_block_cfl_dt_noalloc(const athg_config* cfg, const double* w, const double* bcc,
                              const double* b1f, const double* b2f, const double* b3f,
                              double dx1, double dx2, double dx3, double* dt_out, void* stream);

const char* athg_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* ATHENA_GB300_H_ */
