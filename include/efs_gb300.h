/*
 * efs_gb300.h — C ABI of the GB300 (sm_103a) Eulerian liquid step.
 *
 * One context (efs_ctx) holds one MAC grid resident in HBM, its own CUDA stream and the CUDA graphs
 * that replay whole steps.  Every entry point returns an int status (EFS_OK == 0); the text of the
 * last failure is available from efs_last_error().  Signatures use plain pointers and sizes only.
 *
 * The entry points replace the reference's simulator-backend interface for the liquid step
 * (MarQMark/EulerianFluidSimulation):
 *   - ISimulator::update()              include/simulation/simulator/ISimulator.h:12-38  -> efs_step
 *   - the seven protected stage virtuals include/simulation/simulator/ISimulator.h:43-50 -> efs_stage
 *   - ISolver3D/ISolver2D::solve(IGrid*) include/simulation/solver/ISolver.h:7-47        -> efs_solve
 *   - IGrid3D/IGrid2D field accessors    include/simulation/data/IGrid.h:10-68            -> efs_upload_field /
 *                                                                                         efs_download_field
 *   - CudaGrid3D::upload()/download()    src/simulation/data/CudaGrid3D.cu:247-269        -> efs_upload_fields /
 *                                                                                         efs_download_fields
 *   - the Properties values the step reads include/simulation/Properties.h:136-218       -> efs_params
 *
 * Host field layout is the reference's: x fastest, then y, then z (index z*W*H + y*W + x, W/H/D include the
 * one-cell wall border); velocity and forces are interleaved glm::vec3 (3D) or glm::vec2 (2D) floats;
 * scalar fields are float; `boundary` is 1.0 for solid cells and 0.0 otherwise.
 */
#ifndef EFS_GB300_H
#define EFS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EFS_ABI_VERSION 1

/* ---- status codes ---- */
enum efs_status {
    EFS_OK = 0,
    EFS_ERR_ARG = 1,            /* bad argument (size, pointer, enum, field value)                  */
    EFS_ERR_CUDA = 2,           /* a CUDA runtime call failed                                      */
    EFS_ERR_STATE = 3,          /* call not valid in the context's current state                   */
    EFS_ERR_NO_DEVICE = 4,      /* no CUDA device visible                                          */
    EFS_ERR_DEVICE_FAULT = 5,   /* a kernel reported an error through the device status word       */
    EFS_ERR_NOT_CONVERGED = 6   /* efs_solve only: the pressure solve hit max_steps                */
};

/* ---- the seven stages, in ISimulator::update order (ISimulator.h:15-35) ---- */
enum efs_stage {
    EFS_STAGE_VEL_DECAY = 0,
    EFS_STAGE_VEL_EXTRAPOLATE = 1,
    EFS_STAGE_RHO_SHARPEN = 2,
    EFS_STAGE_RHO_ADVECT = 3,
    EFS_STAGE_VEL_ADVECT = 4,
    EFS_STAGE_ADD_FORCE = 5,
    EFS_STAGE_PROJECT = 6,
    EFS_STAGE_COUNT = 7
};
#define EFS_STAGE_BIT(s) (1u << (s))
#define EFS_STAGES_ALL 0x7Fu

/* ---- pressure solvers (Properties::SolverType, Properties.h:476-482) ---- */
enum efs_solver {
    EFS_SOLVER_JACOBI = 0,      /* JacobiSolverCPU3D: max_steps/2 sweeps from p = 0                */
    EFS_SOLVER_CG = 1,          /* CGSolverCPU3D: p0 = b, true residual every 64 iterations        */
    /* No counterpart in the reference: flexible preconditioned CG (Notay's FCG(1)) on the same matrix and
     * to the same stop rule as EFS_SOLVER_CG, from p0 = 0, with the pressure accumulated as float pairs (about
     * 48 significant bits; efs_download_pressure_fp64 gives their sum) and the true residual recomputed in
     * the same pair arithmetic every 32 iterations and before stopping.  Its preconditioner is a multigrid
     * V-cycle whose coarsest level is solved by the context's learned U-Net (3D; efs_unet_*, fcg_levels and
     * fcg_bottom below).  When the residual stalls (not halved over 10 iterations) or a direction breaks
     * down, the remaining residual system goes to plain CG (EFS_CG_MIXED_RECURRENCE).  The whole solve is
     * device-resident: CUDA graph conditional (while / if) nodes run the iteration, so steps with this solver
     * replay one graph like the others. */
    EFS_SOLVER_FCG_UNET = 2
};

/* CG variants.  Both follow CGSolverCPU3D::solve (CGSolver.cpp:416-465): p0 = b, recurrence residual, the
 * true residual recomputed when (i & 63) == 0, stop when r.r < threshold or after max_steps, FP64-class dot
 * products (summed as float pairs on the GPU, in FP64 by the CPU oracle).  EFS_CG_MIXED keeps the pressure as an extended-precision accumulator (a pair of floats, about
 * 48 significant bits, computed on the FP32 pipe) plus an FP32 increment that is folded in at every
 * recomputation, and computes that true residual in the same pair arithmetic (group-wise reliable updates;
 * the CPU oracle uses FP64 for both); before
 * stopping it recomputes the true residual once more and continues if it is above the threshold.  This
 * reaches relative residuals below what any FP32 pressure field can represent (the rounded exact solution
 * sits near 1e-5 on these grids).  EFS_CG_REFERENCE keeps the pressure in FP32 and recomputes the residual in
 * FP32, like the reference. */
enum efs_cg_variant {
    EFS_CG_MIXED = 0,
    EFS_CG_REFERENCE = 1,
    /* EFS_CG_MIXED_RECURRENCE (default): EFS_CG_MIXED with t = L d stored and beta taken from the
     * residual-norm recurrence r'.r' = alpha^2 t.t - r.r (an exact CG identity), so that alpha and beta both
     * follow from one reduction of d.t and t.t.  The iteration then updates the increment, r and d per cell
     * and sums the exact r'.r' for the stop test (on the GPU that sum travels with the next iteration's
     * reduction).  Every 64th iteration recomputes the residual as EFS_CG_MIXED does, and takes
     * that iteration's beta from it. */
    EFS_CG_MIXED_RECURRENCE = 2,
    /* EFS_CG_FP64: a study solver, not a fast path.  The reference iteration with p, r, d and L d in FP64 and
     * the threshold tol_rel^2 b.b kept in FP64 (set tol_rel to 1e-12 or so): the FP64 pressure solve of the
     * same right-hand side that the FP32 results are measured against.  Its FP64 vectors are allocated when
     * a context first selects it. */
    EFS_CG_FP64 = 3,
    /* EFS_CG_PIPELINED (reserved; contexts reject it with EFS_ERR_ARG): pipelined CG (Ghysels and Vanroose
     * 2014) with the FP64 accumulator and FP64 residual replacement of EFS_CG_MIXED, w = L r, s = L p and
     * z = L s carried by recurrences (one sweep and one reduction per iteration).  Only the CPU oracle
     * implements it, as a studied alternative: with FP32 vectors it needs a replacement every 32 iterations
     * and 9-29 % more iterations than EFS_CG_MIXED_RECURRENCE, which cancels the saved synchronisation. */
    EFS_CG_PIPELINED = 4
};

/* ---- fields (IGrid3D accessors, IGrid.h:44-68) ---- */
enum efs_field {
    EFS_FIELD_VEL = 0,          /* dim floats per cell (MAC faces: vel(x,y,z).x is the face between x-1 and x) */
    EFS_FIELD_RHO = 1,
    EFS_FIELD_GAMMA = 2,
    EFS_FIELD_BETA = 3,
    EFS_FIELD_DIVERGENCE = 4,
    EFS_FIELD_PRESSURE = 5,
    EFS_FIELD_FORCES = 6,       /* dim floats per cell */
    EFS_FIELD_BOUNDARY = 7,     /* 0.0 or 1.0 */
    EFS_FIELD_COUNT = 8
};

/* Density-sharpen scatter semantics.  The reference applies each cell's change and scatters its
 * counter-mass while later cells of the same loop read the updated density
 * (CPUSimulator3D.cpp:446-455, CPUSimulator2D.cpp:388-401).  EFS_SHARPEN_PARALLEL (default, the fast
 * path) applies every cell's change first, then traces all cells on that field, then scatters; the two
 * differ only through the order of those updates.  EFS_SHARPEN_SEQUENTIAL is the reference's order, for
 * parity: one thread walks the changed cells in cell order and applies, traces and scatters each before the
 * next (bit-exact with the reference's loop; about 0.1-2 s a step at 128^3-256^3, so not a fast path).
 * Batches (efs_batch_*) run the parallel mode only. */
enum efs_sharpen_mode {
    EFS_SHARPEN_PARALLEL = 0,
    EFS_SHARPEN_SEQUENTIAL = 1
};

/* Values of the reference Properties the step reads (Properties.h:141-162, 186-192). */
typedef struct efs_params {
    float dt;                 /* DT                                                       */
    float gravity_force;      /* GRAVITY_FORCE in cells/s^2 (= GRAVITY_FORCE_PHYSICAL / CELL_SIZE, Application.cpp:89) */
    int   gravity_enabled;    /* GRAVITY_ENABLED                                          */
    float vel_decay;          /* VEL_DECAY                                                */
    float lambda_minus;       /* LAMBDA_MINUS                                             */
    float lambda_plus;        /* LAMBDA_PLUS                                              */
    float eta;                /* ETA                                                      */
    float liquid_threshold;   /* LIQUID_THRESHOLD                                         */
    float rho_d;              /* RHO_D (sharpen trace length, cells)                      */
    int   solver;             /* enum efs_solver (SOLVER_TYPE)                            */
    int   max_steps;          /* MAX_STEPS (CG iteration cap; Jacobi runs max_steps/2)    */
    float solver_threshold;   /* SOLVER_THRESHOLD: absolute r.r stop, used when tol_rel <= 0 */
    float tol_rel;            /* > 0: stop when r.r < tol_rel^2 * b.b (relative residual) */
    unsigned disable_mask;    /* bit s set = DISABLE_<stage s> (Properties.h:114-120)     */
    int   re_calc_div;        /* RE_CALC_DIV (2D only)                                    */
    int   sharpen_mode;       /* enum efs_sharpen_mode                                    */
    int   cg_variant;         /* enum efs_cg_variant                                      */
    int   fcg_levels;         /* EFS_SOLVER_FCG_UNET: aggregation levels of its preconditioner (below) */
    int   fcg_bottom;         /* EFS_SOLVER_FCG_UNET: enum efs_fcg_bottom                 */
    int   reserved[3];
} efs_params;

/* The preconditioner of EFS_SOLVER_FCG_UNET (no counterpart in the reference) is one V-cycle over a hierarchy
 * of aggregated grids: level 0 is the pressure matrix itself; level l+1 merges 2x2x2 cells of level l, its
 * matrix the Galerkin product P^T A P of the piecewise-constant prolongation P (matrix rows where any merged
 * cell is a row).  At every level above the bottom: 2 damped Jacobi sweeps (weight 6/7), the residual
 * restricted to the next level, the correction prolonged back, 2 more sweeps.  At the bottom level the
 * correction comes from the U-Net (fcg_bottom EFS_FCG_BOTTOM_UNET), scaled by the line search
 * (e.r)/(e.Ae) on that level, or, for comparison without the network, from 20 Jacobi sweeps
 * (EFS_FCG_BOTTOM_JACOBI).  fcg_levels is the number of aggregation levels (0..3); a negative value picks the
 * fewest levels whose bottom grid is at most 32 cells on every side.  The network works on the bottom grid
 * (efs_unet_grid). */
enum efs_fcg_bottom {
    EFS_FCG_BOTTOM_UNET = 0,
    EFS_FCG_BOTTOM_JACOBI = 1
};

/* Per-context statistics (Properties SOLVE_STEPS / SOLVE_ERRORS / PAUSED / SIMULATION_FRAMES). */
typedef struct efs_stats {
    int64_t frames;           /* completed steps (SIMULATION_FRAMES)                      */
    int     solve_steps;      /* iterations of the last pressure solve (SOLVE_STEPS)      */
    int     converged;        /* last solve met its stop rule                             */
    int     paused;           /* set when a solve did not converge (CPUSimulator3D.cpp:541-547) */
    int     device_error;     /* device status word (0 = none)                            */
    double  rr;               /* last solve: final r.r (FP64)                             */
    double  bb;               /* last solve: b.b (FP64)                                   */
    double  threshold;        /* last solve: the r.r threshold it used                    */
    int64_t active_cells;     /* last solve: matrix rows (liquid, non-solid cells)        */
    int64_t total_solve_steps;/* sum of solve_steps over all solves since create / reset  */
    int64_t solves;           /* number of solves since create / reset                    */
    int64_t precond_steps;    /* EFS_SOLVER_FCG_UNET: iterations of the last solve that applied the
                                 preconditioner (the rest of solve_steps were plain CG); 0 otherwise */
} efs_stats;

typedef struct efs_ctx efs_ctx;

/* ---- defaults ---- */
/* Reference Properties defaults (Properties.h:141-162; gravity 10 / cell size 1); the solver fields that
 * Properties does not have: sharpen_mode EFS_SHARPEN_PARALLEL, cg_variant EFS_CG_MIXED_RECURRENCE. */
void efs_params_default(efs_params* p);
/* Dam-break constants of the reference scene assets/scenes/Dam128.json "properties": lambda- 50,
 * lambda+ 10, eta 100, D 32, velocity decay disabled, liquid threshold 0.5, gravity 9.81 / cell_size,
 * with the given dt, solver and relative tolerance. */
void efs_params_dam(efs_params* p, float cell_size, float dt, int solver, float tol_rel);

/* ---- lifetime ---- */
int  efs_abi_version(void);
int  efs_device_count(int* count);
/* dim 2: depth must be 1.  width/height/depth >= 4 and include the one-cell border. */
int  efs_create(int dim, int width, int height, int depth, const efs_params* params, efs_ctx** out);
void efs_destroy(efs_ctx* ctx);
/* Text of the last failure on this context (ctx == NULL: the last efs_create failure). */
const char* efs_last_error(const efs_ctx* ctx);

int  efs_set_params(efs_ctx* ctx, const efs_params* params);
int  efs_get_params(const efs_ctx* ctx, efs_params* params);

/* ---- fields (host buffers in the reference layout) ---- */
int  efs_upload_field(efs_ctx* ctx, int field, const float* host);
int  efs_download_field(efs_ctx* ctx, int field, float* host);
/* CudaGrid3D::upload (CudaGrid3D.cu:247-256): NULL pointers are skipped. */
int  efs_upload_fields(efs_ctx* ctx, const float* vel, const float* rho, const float* gamma,
                       const float* boundary, const float* forces);
/* CudaGrid3D::download (CudaGrid3D.cu:258-269): NULL pointers are skipped. */
int  efs_download_fields(efs_ctx* ctx, float* vel, float* rho, float* gamma, float* beta,
                         float* divergence, float* pressure);
/* One step with host fields in and out: efs_upload_fields, efs_step(ctx, 1) and efs_download_fields in one
 * call (the upload / update / download of a host-mirrored grid, CudaGrid3D::upload and download,
 * src/simulation/data/CudaGrid3D.cu:247-269, around ISimulator::update).  Any pointer may be NULL (skipped).
 * When gamma, forces and the rho / gamma / beta outputs are page-locked host memory, the transfers overlap the
 * step: gamma and forces go up while the stages before rho_advect run, and rho, gamma and beta come down while
 * vel_advect and the pressure solve run; otherwise the three calls run in order.  Returns when the outputs are
 * written. */
int  efs_step_host(efs_ctx* ctx, const float* vel, const float* rho, const float* gamma, const float* boundary,
                   const float* forces, float* vel_out, float* rho_out, float* gamma_out, float* beta_out,
                   float* divergence_out, float* pressure_out);
/* Grid3D/Grid2D constructor state (Grid3D.cpp:10-48): zero fields, gamma = 1, solid border, rho = 0 on it. */
int  efs_reset_fields(efs_ctx* ctx);
/* No counterpart in the reference.  The FP64 pressure of the last CG solve (N doubles, reference layout):
 * the FP64 iterate for EFS_CG_FP64, the FP64 accumulator with its increment folded in for the mixed
 * variants, the float-pair iterate's sum for EFS_SOLVER_FCG_UNET (the FP32 pressure field is this value
 * rounded).  Matrix rows only; other cells hold stale
 * values.  EFS_ERR_STATE for Jacobi and EFS_CG_REFERENCE, which keep no FP64 pressure. */
int  efs_download_pressure_fp64(efs_ctx* ctx, double* host);

/* ---- the step ---- */
/* One reference stage virtual, regardless of disable_mask. */
int  efs_stage(efs_ctx* ctx, int stage);
/* n_steps x ISimulator::update(): the stages not in params.disable_mask, replayed from one CUDA graph
 * per configuration.  Returns after launching; efs_synchronize waits. */
int  efs_step(efs_ctx* ctx, int n_steps);
/* ISolver::solve on the context's current divergence / rho / boundary, into pressure. */
int  efs_solve(efs_ctx* ctx, efs_stats* out);
int  efs_synchronize(efs_ctx* ctx);
int  efs_get_stats(efs_ctx* ctx, efs_stats* out);
/* FP64 sum of rho over all cells (StatsView total, Grid3D.cpp:44-47 in float). */
int  efs_total_mass(efs_ctx* ctx, double* out);

/* Number of kernel launches one efs_step replays for the current parameters (kernel nodes of its graph). */
int  efs_step_kernel_count(efs_ctx* ctx, int* count);

/* ---- timing of the dominant kernel (the pressure solve) over replayed steps ---- */
/* Arms a pool of `capacity` CUDA event pairs recorded around each pressure-solve launch on the
 * context's stream during efs_step.  capacity 0 disarms. */
int  efs_solve_timing_arm(efs_ctx* ctx, int capacity);
/* Number of recorded launches and their summed device time (ms); the work those solves did since arming:
 * the sum of iterations x matrix rows, and the sum of matrix rows (one per solve set-up). */
int  efs_solve_timing_read(efs_ctx* ctx, int* launches, double* total_ms, double* row_iterations,
                           double* row_setups);

/* Device time of one application of FCG's preconditioner (EFS_SOLVER_FCG_UNET; the V-cycle with its bottom
 * solve) on r = the current divergence, after the solve's set-up: mean ms over `reps` applications launched
 * kernel by kernel, and over `reps` replays of one application captured as a graph (the cost inside a solve).
 * A measurement entry point: the pressure field is overwritten with the divergence. */
int  efs_fcg_time_vcycle(efs_ctx* ctx, int reps, float* ms_direct, float* ms_graph);

/* CUDA events on the context's stream: record slot (0..7); elapsed ms between two recorded slots (waits). */
int  efs_timer_mark(efs_ctx* ctx, int slot);
int  efs_timer_elapsed(efs_ctx* ctx, int slot_begin, int slot_end, double* ms);

/* ---- a pressure solve that allocates nothing ---- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc (a host that owns every device
 * allocation of its plug-ins, a real-time loop that may not synchronise the device, work recorded into a CUDA
 * graph): ISolver::solve on caller-owned device buffers rho, boundary, divergence and pressure (N floats each,
 * reference layout), on `stream` (a cudaStream_t; NULL = the legacy default stream).  Working memory is one
 * fixed file-scope device array of EFS_NOALLOC_SCRATCH_BYTES (about 13.2 MB) that every device loading the
 * library keeps until exit, so grids are limited to EFS_NOALLOC_MAX_CELLS cells and larger ones are rejected
 * with EFS_ERR_ARG.  The first call on each device looks up that array's address in the context current then
 * (make it before any stream capture); a cudaDeviceReset or a second driver context on the same device is not
 * supported afterwards.  All calls share the array: calls whose work overlaps on the GPU race.  With
 * stats == NULL the call returns after queueing its work; otherwise it waits for the stream and fills stats
 * (EFS_ERR_NOT_CONVERGED when max_steps ran out).  Errors of this entry point are reported by
 * efs_noalloc_last_error(), per host thread; its text stays valid until that thread's next failing call. */
#define EFS_NOALLOC_MAX_CELLS 262144
#define EFS_NOALLOC_SCRATCH_BYTES 13159168
int  efs_solve_noalloc(int dim, int width, int height, int depth, const efs_params* params,
                       const float* rho, const float* boundary, const float* divergence, float* pressure,
                       void* stream, efs_stats* stats);
const char* efs_noalloc_last_error(void);

/* ---- learned preconditioner: 3D U-Net (3 levels, 16/32/64 channels, BF16 weights, FP32 accumulation) ----
 * No counterpart in the reference.  A context holds at most one network, sized for the bottom grid of the
 * FCG preconditioner's hierarchy (efs_params.fcg_levels at efs_unet_init; with 0 levels, the context's own
 * grid).  The FP32 master parameters are laid out layer by layer as weights [27 taps][cin][cout] then bias
 * [cout] (layers: 16->16, 16->32, 32->64, 64->32, 32->16, 16->16).  The network maps a residual field r on
 * the bottom grid to a correction on that grid's matrix rows; its input channels are r / rms(r), the row
 * mask and, above level 0, the aggregated matrix (diagonal and the six face weights, normalised).  FCG
 * (EFS_SOLVER_FCG_UNET) applies it once per iteration.  Training runs on the device on samples the context
 * stored after its own projections.  The matrix used by efs_unet_apply and efs_unet_loss_grad is the bottom
 * level's, built from the context's current rho and boundary; both entry points overwrite the pressure
 * field with the divergence (the solver's start). */
int  efs_unet_param_count(int64_t* count);
/* Fresh network with He-normal weights from `seed` on the bottom grid of the current fcg_levels; room for
 * `sample_capacity` training samples (0: none). */
int  efs_unet_init(efs_ctx* ctx, uint64_t seed, int sample_capacity);
/* The network's grid (cells per axis) and its aggregation level below the context's grid. */
int  efs_unet_grid(efs_ctx* ctx, int* width, int* height, int* depth, int* level);
int  efs_unet_get_weights(efs_ctx* ctx, float* host, int64_t count);
/* Loading weights also resets the optimiser state of efs_unet_train. */
int  efs_unet_set_weights(efs_ctx* ctx, const float* host, int64_t count);
/* z = net(r) on host fields of the network's grid (its cells' count of floats each). */
int  efs_unet_apply(efs_ctx* ctx, const float* r, float* z);
/* Training losses, for input b and target p (p solves L p = b; host fields):
 *   loss_kind 0: sum over rows of (net(b)_v - p_v / rms(p))^2 / rows (the pressure, normalised);
 *   loss_kind 1: 1 - (z.b)^2 / ((z.Lz)(p.b)) with z = net(b): the share of p's energy norm (-L) that a line
 *                search along z leaves, i.e. how far z is from a perfect preconditioned direction.
 * efs_unet_loss_grad gives the loss and the gradient of every parameter for one sample (grads may be NULL). */
int  efs_unet_loss_grad(efs_ctx* ctx, int loss_kind, const float* b, const float* p, float* loss, float* grads);
/* Device time of the network's forward pass on the current divergence field (CUDA events on the context's
 * stream, `reps` passes after one warm-up): mean ms per pass and per convolution layer (ms_layers[6], may
 * be NULL).  A measurement entry point: the pressure field is overwritten with the divergence. */
int  efs_unet_time_forward(efs_ctx* ctx, int reps, float* ms_forward, float* ms_layers);
/* Stores a training sample (ring buffer).  With 0 aggregation levels: the current (divergence, pressure,
 * matrix rows).  Otherwise: the current divergence carried down the V-cycle's pre-smoothing and restriction
 * chain to the bottom grid (what the network receives in the first FCG iteration), the bottom matrix, and
 * that residual's exact correction on the bottom grid (a CG solve there, relative residual 1e-8). */
int  efs_unet_add_sample(efs_ctx* ctx);
int  efs_unet_sample_count(efs_ctx* ctx, int* count);
/* `iterations` Adam steps (beta 0.9/0.999) of `batch` samples drawn with `seed`; mean loss of the last batch.
 * A fraction `synthetic` of the batch are synthetic pairs on a stored sample's matrix rows: a random
 * multi-scale error field e (hash-valued lattices of spacing 1..16, random spectral slope) and input L e. */
int  efs_unet_train(efs_ctx* ctx, int loss_kind, int iterations, int batch, float lr, float synthetic, uint64_t seed,
                    float* last_loss);

/* ---- many independent 2D scenes of uneven sizes, advanced together ----
 * No counterpart in the reference (each reference simulator owns one grid).  Every scene is a full 2D
 * simulation (CPUSimulator2D stages, CGSolverCPU2D pressure solve with EFS_CG_MIXED_RECURRENCE) on its own
 * grid (W x H, border included); all scenes share `params` except GRAVITY_FORCE, which may be given per
 * scene (cells/s^2 for that scene's cell size).  One step of all scenes is one CUDA graph in which every
 * stage kernel is a single persistent launch over a table of (scene, block) entries, and the pressure solves
 * are a single launch whose blocks each solve whole scenes, largest first.  Fields use the single-context
 * layouts (vel and forces: interleaved vec2).  A new batch holds the Grid2D constructor state: zero fields,
 * gamma = 1, solid border. */
typedef struct efs_batch efs_batch;
typedef struct efs_batch_tuning {
    int   tile_x, tile_y;     /* stage-kernel block: tile_x x tile_y cells (product a multiple of 32)   */
    int   blocks_per_sm;      /* persistent blocks per SM of the stage kernels                          */
    int   solver_threads;     /* threads of a solver block (128, 256, 512 or 1024)                      */
    int   solver_cluster;     /* solver blocks per scene: 1 (one block), or a thread-block cluster of   */
                              /* 2, 4, 8 or 16 blocks exchanging partial sums in distributed shared mem */
    float ms_per_step;        /* efs_batch_autotune: measured step time of the chosen configuration     */
} efs_batch_tuning;
int  efs_batch_create(int n_scenes, const int* widths, const int* heights, const efs_params* params,
                      const float* gravity_force, efs_batch** out);
void efs_batch_destroy(efs_batch* batch);
/* NULL: the error of the last failed efs_batch_create. */
const char* efs_batch_last_error(const efs_batch* batch);
int  efs_batch_scene_count(const efs_batch* batch, int* n);
int  efs_batch_upload_field(efs_batch* batch, int scene, int field, const float* host);
int  efs_batch_download_field(efs_batch* batch, int scene, int field, float* host);
/* One stage of every scene (direct launches). */
int  efs_batch_stage(efs_batch* batch, int stage);
/* n_steps whole steps of every scene (graph replays; asynchronous). */
int  efs_batch_step(efs_batch* batch, int n_steps);
int  efs_batch_synchronize(efs_batch* batch);
/* n_steps steps with CUDA events recorded around them on the batch's stream; *ms = their device time. */
int  efs_batch_time_steps(efs_batch* batch, int n_steps, float* ms);
int  efs_batch_stats(efs_batch* batch, int scene, efs_stats* out);
int  efs_batch_kernel_count(efs_batch* batch, int* count);
int  efs_batch_get_tuning(const efs_batch* batch, efs_batch_tuning* tuning);
int  efs_batch_set_tuning(efs_batch* batch, const efs_batch_tuning* tuning);
/* Times trial steps of candidate tile shapes, blocks per SM, solver block sizes and solver clusters from the current state
 * (restored after every trial) and keeps the fastest; `best` (may be NULL) receives it. */
int  efs_batch_autotune(efs_batch* batch, int trial_steps, efs_batch_tuning* best);

/* ---- scene construction and queries (the editor and scene-node side; between steps) --------------------
 * These write or read a context's device fields directly, on its stream, and return after the work is done.
 * Triangles use the reference Triangle layout (include/assets/Triangle.h:10-19): 12 floats per triangle,
 * v0.xyz, pad, v1.xyz, pad, v2.xyz, pad, in world coordinates; the domain is the simulation domain's
 * world box (SimulationDomainNode / BoundingBoxNode::getWorldBoundingBox: centre and size), which the grid,
 * border included, divides into W x H x D cells.  Mesh operations are 3D only. */

/* The inside/outside label of sdf.comp (assets/shaders/sdf.comp:29-114) for every cell of
 * [0, W-1) x [0, H-1) x [0, D-1): `value_inside` where the cell centre is on a triangle or the mesh's winding
 * number exceeds pi in magnitude, else `value_outside`.  Other cells keep their value.  `field` is a scalar
 * field or EFS_FIELD_BOUNDARY (values 0.0/1.0).  Replaces the sdf.comp dispatches of Editor::initFluid and
 * Editor::initBoundaries (src/core/Editor.cpp:118-137, :199-218). */
int  efs_mesh_label(efs_ctx* ctx, int field, const float* triangles, int n_triangles, const float domain_center[3],
                    const float domain_size[3], float value_inside, float value_outside);
/* The cells that efs_mesh_label labels inside, as ascending linear indices (forcefield_cells.comp:90-111,
 * which appends them in dispatch order).  *count receives their number; at most `capacity` are written. */
int  efs_mesh_cells(efs_ctx* ctx, const float* triangles, int n_triangles, const float domain_center[3],
                    const float domain_size[3], int* cells, long long capacity, long long* count);
/* `value` (1 float, or dim floats for EFS_FIELD_VEL / EFS_FIELD_FORCES) in every cell of the box
 * [lo, hi), clipped to the grid (2D: z ignored).  The box fluid spawn (Editor.cpp:155-161), the initial fill
 * (baseFluidFill.comp:24-35), DeletionNode::update (DeletionNode.cpp:27-33). */
int  efs_fill_box(efs_ctx* ctx, int field, const int lo[3], const int hi[3], const float* value);
/* `value` at the n listed linear cell indices (Scene2D::loadScene, Scene2D.cpp:59-62; the force-field cells,
 * Editor.cpp:325-330).  An index outside the grid is EFS_ERR_ARG (the rest are written). */
int  efs_set_cells(efs_ctx* ctx, int field, const int* cells, long long n, const float* value);
/* The outer layer of cells becomes solid, and rho is 0 in every solid cell (Editor.cpp:220-229). */
int  efs_seal_boundary(efs_ctx* ctx);

/* QueryNode metrics (include/simulation/scene/nodes/QueryNode.h:10-17) over the box of cells
 * [max(0, position), min(dim - 1, position + scale)) per axis (QueryNode.cpp:47-66; 2D: z ignored), only
 * cells with rho >= 0.5 when only_fluid: the largest, smallest and mean cell coordinates, and the mean
 * velocity (the MAC face values stored at each cell) and pressure.  All zero when no cell counts.  Sums are
 * exact (coordinates) or FP64 (velocity, pressure), in a fixed order. */
typedef struct efs_query_metrics {
    float max_position[3];
    float min_position[3];
    float avg_position[3];
    float velocity[3];
    float pressure;
    int   pad;
    long long count;
} efs_query_metrics;
int  efs_query_box(efs_ctx* ctx, const int position[3], const int scale[3], int only_fluid, efs_query_metrics* out);

/* ---- host-only helpers (no device needed) ---- */
/* Seeded synthetic scenes; see efs_scene.h for the generators and their draw order. */
int  efs_scene_dam3d(int w, int h, int d, int n_spheres_min, int n_spheres_max, uint64_t seed,
                     float* boundary, float* rho);
int  efs_scene_dam2d(int w, int h, float* boundary, float* rho);
int  efs_scene_batch2d(uint64_t seed, int* side, float* boundary, float* rho, int capacity);

#ifdef __cplusplus
}
#endif
#endif /* EFS_GB300_H */
