/*
 * efs_oracle.h — CPU oracle for the Eulerian liquid step.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU backend (MarQMark/EulerianFluidSimulation,
 * src/simulation/simulator/CPUSimulator{2D,3D}.cpp, src/simulation/data/{Grid,ScalField,VecField}{2D,3D}.cpp,
 * src/simulation/solver/{CGSolver,JacobiSolver}.cpp).  Every function cites the reference lines it follows.
 * It is the checker for the CUDA path and the timed CPU baseline; nothing in the product links it.
 *
 * Pinning: tests compare this restatement against the unmodified reference sources compiled here with a
 * shim include directory (oracle/Makefile -> oracle/_ref/libefs_ref.so) and against golden fixtures
 * produced by that build (tests/golden/).
 *
 * Deliberate differences from the reference, each selectable or stated:
 *   - The advection matrix A is keyed by the pair (i, j).  The reference packs the key as the 32-bit
 *     product i*size()+j (Grid3D.cpp:168-174, Grid2D.cpp:183-189), which wraps once size()^2 >= 2^32
 *     (3D grids of 41^3 cells and more, 2D grids wider than 256^2) and merges unrelated entries.  At sizes
 *     where the key does not wrap the two agree up to float summation order (the reference sums in
 *     std::unordered_map / std::map order; this oracle sums backward rows in cell order, then forward entries
 *     in insertion order).
 *   - ORC_DOTS_FP64 makes the CG dot products FP64 (the GPU's arithmetic); the default follows the
 *     reference's float accumulation (ScalField3D.h:91-97).
 *   - ORC_SHARPEN_PARALLEL applies all density changes, traces every active cell on that field, then
 *     scatters in cell order (the GPU's semantics); the default is the reference's sequential loop
 *     (CPUSimulator3D.cpp:446-455).
 *   - ORC_REVERSE_SUMS sums the advection matrix in exactly the reverse entry order: a summation-order
 *     perturbation used to ground multi-step drift bounds (oracle against perturbed oracle).
 *   - When params.tol_rel > 0 the solver threshold is (float)(tol_rel^2 * b.b) of the current right-hand
 *     side (FLT_MIN if that is 0), used both by the solver and by project's convergence check.
 */
#ifndef EFS_ORACLE_H
#define EFS_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/efs_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_DOTS_FP64 1
#define ORC_SHARPEN_PARALLEL 2
#define ORC_REVERSE_SUMS 4

typedef struct orc_grid orc_grid;

void      orc_params_default(efs_params* p);
orc_grid* orc_create(int dim, int w, int h, int d, const efs_params* prm);
void      orc_destroy(orc_grid* g);
void      orc_set_params(orc_grid* g, const efs_params* prm);
void      orc_set_mode(orc_grid* g, int mode_flags);
/* Direct pointer to a field (reference layout; EFS_FIELD_* ids).  Valid until orc_destroy. */
float*    orc_field(orc_grid* g, int field);
void      orc_reset(orc_grid* g);
void      orc_stage(orc_grid* g, int stage);
void      orc_step(orc_grid* g, int n_steps);
/* The solver alone on the current divergence/rho/boundary (ISolver::solve); returns its error value. */
float     orc_solve(orc_grid* g);
void      orc_stats(const orc_grid* g, efs_stats* out);

/* FP64 conjugate gradient on the same masked Laplacian (vectors and dots in double), started from 0,
 * stopped at ||r|| <= tol * ||b|| or maxit; result in p_out (N doubles).  Returns iterations. */
int       orc_solve_fp64(orc_grid* g, double tol, int maxit, double* p_out);
/* ||b - L p|| / ||b|| in FP64 for a float pressure field p (N floats). */
double    orc_relres_fp64(orc_grid* g, const float* p);
/* sum of rho over all cells in FP64 */
double    orc_total_mass(orc_grid* g);
/* host threads the solvers' per-cell loops use (1 without OpenMP) */
int       orc_threads(void);

/* seeded scenes of include/efs_scene.h */
int       orc_scene_dam3d(int w, int h, int d, int n_min, int n_max, uint64_t seed, float* boundary, float* rho);
int       orc_scene_dam2d(int w, int h, float* boundary, float* rho);
int       orc_scene_batch2d(uint64_t seed, int* side, float* boundary, float* rho);

#ifdef __cplusplus
}
#endif
#endif
