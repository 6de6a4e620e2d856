// efs_batch.h — internal: many independent 2D scenes of uneven sizes advanced together.
//
// All scenes' fields are packed into one array per field; scene s occupies cells [base_s, base_s + N_s) with
// base_s a multiple of 32 (so 32-cell solver chunks never straddle two scenes).  Arrays with several slots per
// cell (the advection weights) hold scene s at slots * base_s, slot-major inside the scene, exactly as one
// scene's arrays are laid out in a single context.  Work is described by tables of entries (scene, virtual
// block x, virtual block y): every batched kernel is one persistent launch whose blocks walk a table and run
// the same per-block device code the single-scene kernels run, on the scene's geometry and pointers.
#pragma once
#include <cstdint>

#include "efs_internal.h"

namespace efs {

struct BScene {
    Geo g;
    long long base;       // first cell of the scene in the packed arrays (multiple of 32)
    float gforce;         // GRAVITY_FORCE of the scene in cells/s^2 (its own cell size)
    int pad;
};

struct BEntry {
    int scene, bx, by, pad;
};

struct BView {
    const BEntry* e;
    int n;
    const BScene* sc;
};

struct BFields {
    float *u, *v, *rho, *gamma, *beta, *div, *p, *fx, *fy;
    uint8_t* solid;
    float *tu, *tv;                 // vel_advect results / extrapolation ping-pong
    uint8_t *validA, *validB;
    float *wb, *wf;                 // 4 advection weights per cell (2D), slot-major per scene
    int *bb, *fb;
    float *bsum, *gsum, *rho_acc;
    int *sh_idx, *sh_sid;           // density-sharpen list: packed cell index and scene of each entry
    float *sh_val, *sh_end;
    uint16_t* rowinfo;
    uint8_t* chunk_flag;            // one per 32 packed cells
    DevCtl* ctl;                    // shared: sharpen list count, error word
    DevCtl* sctl;                   // one per scene: solve results, paused
    int list_cap;
};

// Launch configuration of the batched stage kernels (picked by the autotuner).
struct BLaunch {
    BView interior;                 // tiles of bx_dim x by_dim interior cells
    BView post;                     // project_post tiles (cells x, y in [1, W-1] x [1, H-1])
    BView linear;                   // 256-cell blocks over every cell of every scene
    BView dx, dy;                   // 128 lines per entry for the diffusion sweeps along x and along y
    int bx_dim, by_dim;
    int grid;                       // persistent blocks per launch
    int list_grid;
    long long total_cells;          // packed cells of all scenes (with their alignment gaps)
    BFields F;
    float dt, vel_decay, rho_d;
    float thrL, lp, lm, eta;
    int gravity;
    cudaStream_t stream;
};

// efs_stages.cu: one stage of every scene (project: walls, divergence, rows; the solve is separate)
// chain_traces: rho_advect and vel_advect run back to back in this step (rho_advect keeps its back-trace ends in
// tu, tv; vel_advect samples at them instead of tracing again)
cudaError_t batch_stage(const BLaunch& L, int stage, bool fuse_add_force, bool chain_traces = false);
cudaError_t batch_project_pre(const BLaunch& L);
cudaError_t batch_project_post(const BLaunch& L);

}  // namespace efs
