// efs_internal.h — the context behind the C ABI and the launch entry points shared by the translation units.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/efs_gb300.h"
#include "efs_device.cuh"

namespace efs {

// Device error bits (efs_stats.device_error).
enum DeviceError : int {
    DEV_ERR_BARRIER_TIMEOUT = 1,   // a grid barrier of the persistent solver gave up waiting
    DEV_ERR_BAD_BOUNDARY = 2,      // an uploaded boundary value was neither 0.0 nor 1.0
    DEV_ERR_LIST_OVERFLOW = 4,     // a compaction list exceeded its capacity
    DEV_ERR_BAD_INDEX = 8          // a listed cell index was outside the grid
};

// Control block in device memory: grid barrier, solve results and counters.  Mirrored into pinned host
// memory by efs_get_stats.
struct DevCtl {
    unsigned bar_count;        // grid barrier arrivals, counting up through the launch (reset before every launch)
    int bar_abort;             // set when a barrier of the current launch gave up (reset before every launch)
    int error;
    int converged;
    int iterations;
    int paused;
    int active_chunks;
    int sh_count;              // density-sharpen active-cell count
    int precond_iterations;    // FCG: iterations of the last solve that applied the preconditioner
    long long active_cells;
    long long total_iterations;
    long long solves;
    double rr, bb, thr;
    double sum_iter_rows;      // sum over solves of iterations x matrix rows (since the timing pool was armed)
    double sum_rows;           // sum over solves of matrix rows
};

// Arguments of the persistent pressure solver (efs_solver.cu).
struct SolverArgs {
    Geo g;
    int dim;
    int solver;                // efs_solver
    int cg_variant;            // efs_cg_variant
    int max_steps;
    float tol_rel;
    float solver_threshold;
    int n_chunks;              // ceil(N / 32)
    const float* b;            // divergence (right-hand side)
    const uint16_t* rowinfo;   // per cell: bit 15 matrix row; bits 0-5 summed neighbours; bits 8-10 count
    const uint8_t* chunk_flag; // per 32-cell chunk: 1 if it holds a matrix row or a non-zero b
    int* chunk_list;           // compacted active chunks (capacity n_chunks)
    int* block_count;          // per block: active chunks in its static range
    float* p;                  // pressure (FP32 field)
    double* p64;               // FP64 pressure accumulator (EFS_CG_MIXED)
    float* e;                  // FP32 increment since the last fold (EFS_CG_MIXED) / Jacobi ping-pong buffer
    float* r;
    float* d0;
    float* d1;
    float* t;                  // L d of the current iteration (EFS_CG_MIXED_RECURRENCE)
    double* r64;               // EFS_CG_FP64 vectors (allocated when that variant is first selected)
    double* d64;
    double* t64;
    double* partials;          // 2 slots x 3 values per block
    DevCtl* ctl;
    const double* thr_dev;     // when set: the absolute r.r threshold, read from device memory (FCG fallback)
};

// A matrix level of the FCG preconditioner's hierarchy (efs_mlfcg.cu): grid dims, per-cell row flag in bit 15
// of info; level 0 (w == nullptr) reads its stencil from the solver's rowinfo bits, coarser levels from a
// float diagonal and six byte face weights (w[k * V + i], k = -x, +x, -y, +y, -z, +z).
struct LvView {
    int W, H, D;
    long long V;
    const uint16_t* info;
    const uint8_t* w;
    const float* diag;
    const float* wd = nullptr;   // coarse levels: the smoother's damping over the diagonal (0 off the rows)
};

struct GraphKey {
    unsigned stages;
    int solver, cg_variant;
    bool operator<(const GraphKey& o) const {
        if (stages != o.stages) return stages < o.stages;
        if (solver != o.solver) return solver < o.solver;
        return cg_variant < o.cg_variant;
    }
};

}  // namespace efs

namespace efs {
struct UNetState;
struct MLState;
}

struct efs_ctx {
    int dim = 3;
    efs::Geo g{};
    efs_params prm{};
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;

    // fields (SoA)
    float *u = nullptr, *v = nullptr, *w = nullptr;
    float *rho = nullptr, *gamma = nullptr, *beta = nullptr, *div = nullptr, *p = nullptr;
    float *fx = nullptr, *fy = nullptr, *fz = nullptr;
    uint8_t* solid = nullptr;
    bool has_forces = false;

    // temporaries
    float* tvel = nullptr;                  // 3N: vel_advect / extrapolation ping-pong and host staging
    uint8_t *validA = nullptr, *validB = nullptr;
    float *wb = nullptr, *wf = nullptr;     // advection weights, slot-major (k * N + i)
    int *bb = nullptr, *fb = nullptr;       // advection base cell (-1: no entries)
    float *bsum = nullptr, *gsum = nullptr, *rho_acc = nullptr;
    int* sh_idx = nullptr;                  // density-sharpen active cells
    float* sh_val = nullptr;
    float* sh_end = nullptr;                // 3 per active cell

    // solver
    uint16_t* rowinfo = nullptr;
    uint8_t* chunk_flag = nullptr;
    int* chunk_list = nullptr;
    int* block_count = nullptr;
    float *r = nullptr, *d0 = nullptr, *d1 = nullptr, *e = nullptr, *t = nullptr;
    double *r64 = nullptr, *d64 = nullptr, *t64 = nullptr;
    double* p64 = nullptr;
    double* partials = nullptr;
    int solver_blocks = 0;
    int solver_threads = 0;
    size_t solver_smem = 0;

    double* mass_partials = nullptr;
    // arrays read at stencil offsets by the solver carry a halo of halo_cells on each side, so neighbour
    // addresses of any cell of any active chunk stay inside the allocation without clamping
    long long halo_cells = 0;
    std::vector<void*> halo_bases;
    efs::DevCtl* ctl = nullptr;
    efs::DevCtl* ctl_host = nullptr;        // pinned

    std::map<efs::GraphKey, cudaGraphExec_t> graphs;
    std::map<efs::GraphKey, cudaGraph_t> graph_defs;    // kept alive: their node handles address the exec nodes
    std::map<efs::GraphKey, cudaGraphNode_t> timing_nodes_begin, timing_nodes_end;
    std::map<efs::GraphKey, int> kernel_nodes;

    // solve timing pool
    std::vector<cudaEvent_t> ev_begin, ev_end;   // only grows: a replayed graph's event nodes may hold any of them
    int ev_used = 0;
    int ev_capacity = 0;                         // pairs armed by efs_solve_timing_arm
    cudaEvent_t ev_solve_begin = nullptr, ev_solve_end = nullptr;   // recorded inside the graph

    cudaEvent_t marks[8] = {};
    int64_t frames = 0;
    std::string err;

    efs::UNetState* unet = nullptr;         // learned preconditioner (efs_unet.cu)
    efs::MLState* ml = nullptr;             // FCG and its multilevel hierarchy (efs_mlfcg.cu)
    void* query_scratch = nullptr;          // efs_query_box block partials and result (efs_scene.cu)
    // efs_step_host: transfers that overlap the step run on `xfer`; the step graph waits for `ev_gamma` before
    // rho_advect and for `ev_forces` before vel_advect, and records `ev_advected` after rho_advect
    cudaStream_t xfer = nullptr;
    cudaEvent_t ev_gamma = nullptr, ev_forces = nullptr, ev_advected = nullptr;
    cudaEvent_t ev_projected = nullptr;   // recorded after project_pre: the divergence is final
    cudaEvent_t ev_early = nullptr;         // the first stages' inputs are on the device
    float* fstage = nullptr;                // efs_step_host: staging of the forces (dim floats a cell)
};

namespace efs {
// efs_stages.cu
// chain_traces: rho_advect and vel_advect run back to back in this step; rho_advect keeps its back-trace ends
// (tvel) and vel_advect samples at them instead of tracing again.
cudaError_t launch_stage(efs_ctx* c, int stage, bool fuse_add_force, bool chain_traces = false);
cudaError_t launch_project_pre(efs_ctx* c);
cudaError_t launch_project_post(efs_ctx* c);
cudaError_t launch_solver_prep(efs_ctx* c);
// efs_solver.cu
cudaError_t solver_configure(efs_ctx* c);
cudaError_t launch_solver(efs_ctx* c);
// persistent CG on right-hand side b (not the context's divergence) with the absolute threshold *thr_dev, on
// stream st; the context's solver vectors, pressure and control block (efs_solver.cu)
cudaError_t launch_solver_on(efs_ctx* c, const float* b, const double* thr_dev, cudaStream_t st);
// efs_mlfcg.cu: FCG with the multilevel preconditioner; inside a stream capture it adds its nodes, otherwise
// it replays a cached solve graph.  ml_alloc (outside any capture) sizes the hierarchy for the current params.
cudaError_t fcg_solve(efs_ctx* c);
cudaError_t ml_alloc(efs_ctx* c);
void ml_free(efs_ctx* c);
void ml_drop_graph(efs_ctx* c);
int ml_resolve_levels(const efs_ctx* c);
int ml_levels(const efs_ctx* c);
void ml_level_dims(const efs_ctx* c, int level, int* W, int* H, int* D);
LvView ml_view(const efs_ctx* c, int level);
cudaError_t ml_build(efs_ctx* c, cudaStream_t st);
cudaError_t ml_matvec(const LvView& L, const float* x, float* y, cudaStream_t st);
cudaError_t ml_descend(efs_ctx* c, const float* r0, cudaStream_t st, const float** out);
cudaError_t ml_time_vcycle(efs_ctx* c, int reps, float* ms_direct, float* ms_graph);
int ml_level_cg(efs_ctx* c, const LvView& L, const float* r0, float* e, float* t1, float* t2, float* t3, double tol,
                int maxit, cudaStream_t st);
// efs_unet.cu: the network's forward pass on bottom-level residual r with its input scale already in
// unet_scale_slot(c) ([0] sum of squares, [1] rows, [2] 1 / rms); output channel 0 in unet_output(c); teardown
cudaError_t unet_forward_prescaled(efs_ctx* c, const LvView& B, const float* r, cudaStream_t st);
double* unet_scale_slot(efs_ctx* c);
cudaError_t unet_scale_rows(efs_ctx* c, const LvView& B, const float* r, cudaStream_t st);   // the slot from r
const float* unet_output(efs_ctx* c);
bool unet_matches(const efs_ctx* c);   // the network was made for the context's current fcg_levels
void unet_free(efs_ctx* c);
void drop_all_graphs(efs_ctx* c);
// efs_fields.cu
cudaError_t launch_upload_vec(efs_ctx* c, const float* staged, float* a, float* b, float* cc, cudaStream_t st = nullptr);
cudaError_t launch_download_vec(efs_ctx* c, float* staged, const float* a, const float* b, const float* cc,
                                cudaStream_t st = nullptr);
cudaError_t launch_boundary_to_solid(efs_ctx* c, const float* staged);
cudaError_t launch_solid_to_boundary(efs_ctx* c, float* staged);
cudaError_t launch_reset_fields(efs_ctx* c);
cudaError_t launch_copy(efs_ctx* c, const float* src, float* dst, long long n);
cudaError_t launch_mass(efs_ctx* c, double* out_dev);
// efs_scene.cu: scene construction and queries
struct FieldPtrsOut {
    float* f[3] = {nullptr, nullptr, nullptr};
    uint8_t* solid = nullptr;
    int ncomp = 0;
};
bool scene_field_ptrs(efs_ctx* c, int field, FieldPtrsOut& out);
cudaError_t launch_mesh_label(efs_ctx* c, const float* d_tris, int ntri, const float center[3], const float size[3],
                              float vin, float vout, int field, uint8_t* mask);
cudaError_t launch_mask_compact(efs_ctx* c, const uint8_t* mask, int* d_out, long long cap, int* d_counts,
                                long long* d_offsets);
long long mask_tiles(const efs_ctx* c);
cudaError_t launch_fill_box(efs_ctx* c, int field, const int lo[3], const int hi[3], const float* value);
cudaError_t launch_set_cells(efs_ctx* c, int field, const int* d_cells, long long n, const float* value);
cudaError_t launch_seal_boundary(efs_ctx* c);
size_t query_scratch_bytes();
cudaError_t launch_query_box(efs_ctx* c, const int lo[3], const int hi[3], int only_fluid, void* scratch,
                             efs_query_metrics* d_out);
}  // namespace efs
