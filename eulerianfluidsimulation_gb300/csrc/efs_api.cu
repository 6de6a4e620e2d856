// efs_api.cu — the C ABI of include/efs_gb300.h.
//
// A context owns its device buffers, one non-blocking stream and one instantiated CUDA graph per step
// configuration (enabled stages, solver, CG variant).  efs_step replays that graph; the pressure solve
// inside it is a single cooperative kernel, so a step never waits on the host.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "efs_internal.h"
#include "../../include/efs_scene.h"

using efs::DevCtl;

namespace {

std::string g_create_error;

int fail(efs_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg; else g_create_error = msg;
    return code;
}

int cuda_fail(efs_ctx* c, cudaError_t e, const char* what) {
    return fail(c, EFS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return cuda_fail(c, e_, what); } while (0)

bool params_valid(const efs_params* p, std::string& why) {
    if (!p) { why = "params is NULL"; return false; }
    if (!std::isfinite(p->dt) || !std::isfinite(p->gravity_force)) { why = "dt and gravity_force must be finite"; return false; }
    if (p->solver != EFS_SOLVER_JACOBI && p->solver != EFS_SOLVER_CG && p->solver != EFS_SOLVER_FCG_UNET) {
        why = "unknown solver";
        return false;
    }
    if (p->cg_variant != EFS_CG_MIXED && p->cg_variant != EFS_CG_REFERENCE && p->cg_variant != EFS_CG_MIXED_RECURRENCE &&
        p->cg_variant != EFS_CG_FP64) {
        why = "unknown cg_variant";
        return false;
    }
    if (p->sharpen_mode != EFS_SHARPEN_PARALLEL && p->sharpen_mode != EFS_SHARPEN_SEQUENTIAL) {
        why = "unknown sharpen_mode";
        return false;
    }
    if (p->max_steps < 0) { why = "max_steps must be >= 0"; return false; }
    if (p->fcg_levels > 3) { why = "fcg_levels must be at most 3"; return false; }
    if (p->fcg_bottom != EFS_FCG_BOTTOM_UNET && p->fcg_bottom != EFS_FCG_BOTTOM_JACOBI) { why = "unknown fcg_bottom"; return false; }
    if (p->disable_mask & ~EFS_STAGES_ALL) { why = "disable_mask has bits beyond the seven stages"; return false; }
    return true;
}

void drop_graphs(efs_ctx* c) {
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    for (auto& kv : c->graph_defs) cudaGraphDestroy(kv.second);
    c->graphs.clear();
    c->graph_defs.clear();
    c->timing_nodes_begin.clear();
    c->timing_nodes_end.clear();
    c->kernel_nodes.clear();
    efs::ml_drop_graph(c);
}

// FCG's buffers are allocated before any capture of a solve (allocation is not allowed while capturing).
int prepare_fcg(efs_ctx* c) {
    if (c->prm.solver != EFS_SOLVER_FCG_UNET) return EFS_OK;
    if (c->dim != 3) return fail(c, EFS_ERR_STATE, "EFS_SOLVER_FCG_UNET is 3D only");
    if (c->prm.fcg_bottom == EFS_FCG_BOTTOM_UNET && !c->unet)
        return fail(c, EFS_ERR_STATE, "FCG needs a U-Net: efs_unet_init or efs_unet_set_weights");
    if (c->prm.fcg_bottom == EFS_FCG_BOTTOM_UNET && c->unet && !efs::unet_matches(c))
        return fail(c, EFS_ERR_STATE, "the U-Net was made for another fcg_levels: efs_unet_init again");
    CK(efs::ml_alloc(c), "FCG buffers");
    return EFS_OK;
}

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    return cudaMalloc(reinterpret_cast<void**>(p), (count ? count : 1) * sizeof(T));
}

// count elements plus c->halo_cells on each side (zeroed); *p points at element 0
template <typename T>
cudaError_t dalloc_halo(efs_ctx* c, T** p, size_t count) {
    T* base = nullptr;
    const size_t h = (size_t)c->halo_cells;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&base), (count + 2 * h) * sizeof(T));
    if (e != cudaSuccess) return e;
    c->halo_bases.push_back(base);
    e = cudaMemset(base, 0, (count + 2 * h) * sizeof(T));
    *p = base + h;
    return e;
}

// The launch sequence of one ISimulator::update() (include/simulation/simulator/ISimulator.h:12-38).
cudaError_t enqueue_step(efs_ctx* c, unsigned stages, bool timing_events) {
    const bool fuse = (stages & EFS_STAGE_BIT(EFS_STAGE_VEL_ADVECT)) && (stages & EFS_STAGE_BIT(EFS_STAGE_ADD_FORCE));
    const bool chain = (stages & EFS_STAGE_BIT(EFS_STAGE_RHO_ADVECT)) && (stages & EFS_STAGE_BIT(EFS_STAGE_VEL_ADVECT));
    for (int s = 0; s < EFS_STAGE_COUNT; s++) {
        // captured steps: efs_step_host uploads gamma and forces on the transfer stream; gamma is first read by
        // rho_advect, the forces by vel_advect's averaging pass (or add_force after it).  rho, gamma and beta
        // are final after rho_advect (the later stages do not write them).
        if (timing_events && s == EFS_STAGE_RHO_ADVECT) {
            cudaError_t e = cudaStreamWaitEvent(c->stream, c->ev_gamma, cudaEventWaitExternal);
            if (e != cudaSuccess) return e;
        }
        if (timing_events && s == EFS_STAGE_VEL_ADVECT) {
            cudaError_t e = cudaEventRecordWithFlags(c->ev_advected, c->stream, cudaEventRecordExternal);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->ev_forces, cudaEventWaitExternal);
            if (e != cudaSuccess) return e;
        }
        if (!(stages & EFS_STAGE_BIT(s))) continue;
        if (s == EFS_STAGE_ADD_FORCE && fuse) continue;   // applied inside vel_advect's averaging pass
        cudaError_t e;
        if (s == EFS_STAGE_PROJECT) {
            if ((e = efs::launch_project_pre(c)) != cudaSuccess) return e;
            if (timing_events && (e = cudaEventRecordWithFlags(c->ev_projected, c->stream, cudaEventRecordExternal)) != cudaSuccess) return e;
            if (timing_events && (e = cudaEventRecordWithFlags(c->ev_solve_begin, c->stream, cudaEventRecordExternal)) != cudaSuccess) return e;
            if ((e = efs::launch_solver(c)) != cudaSuccess) return e;
            if (timing_events && (e = cudaEventRecordWithFlags(c->ev_solve_end, c->stream, cudaEventRecordExternal)) != cudaSuccess) return e;
            if ((e = efs::launch_project_post(c)) != cudaSuccess) return e;
        } else {
            if ((e = efs::launch_stage(c, s, s == EFS_STAGE_VEL_ADVECT && fuse, chain)) != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

int build_graph(efs_ctx* c, const efs::GraphKey& key, cudaGraphExec_t* out) {
    auto it = c->graphs.find(key);
    if (it != c->graphs.end()) { *out = it->second; return EFS_OK; }
    if (key.stages & EFS_STAGE_BIT(EFS_STAGE_PROJECT)) {
        const int s = prepare_fcg(c);
        if (s != EFS_OK) return s;
    }
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    cudaError_t le = enqueue_step(c, key.stages, true);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
    if (le != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return cuda_fail(c, le, "step capture"); }
    if (ce != cudaSuccess) return cuda_fail(c, ce, "cudaStreamEndCapture");
    // locate the two event-record nodes around the solver so their events can be swapped per replay
    size_t n = 0;
    cudaGraphGetNodes(graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) cudaGraphGetNodes(graph, nodes.data(), &n);
    int kernels = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) != cudaSuccess) continue;
        if (t == cudaGraphNodeTypeKernel) kernels++;
        if (t != cudaGraphNodeTypeEventRecord) continue;
        cudaEvent_t ev;
        if (cudaGraphEventRecordNodeGetEvent(nd, &ev) != cudaSuccess) continue;
        if (ev == c->ev_solve_begin) c->timing_nodes_begin[key] = nd;
        if (ev == c->ev_solve_end) c->timing_nodes_end[key] = nd;
    }
    cudaGraphExec_t exec = nullptr;
    cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    if (ie != cudaSuccess) { cudaGraphDestroy(graph); return cuda_fail(c, ie, "cudaGraphInstantiate"); }
    c->graphs[key] = exec;
    c->graph_defs[key] = graph;
    c->kernel_nodes[key] = kernels;
    *out = exec;
    return EFS_OK;
}

int check_device_status(efs_ctx* c) {
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    CK(cudaMemcpy(c->ctl_host, c->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost), "read device status");
    if (c->ctl_host->error) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "device status word %d (1 barrier timeout, 2 boundary not 0/1, 4 list overflow, 8 bad cell index)",
                      c->ctl_host->error);
        const int err = c->ctl_host->error;
        int zero = 0;
        cudaMemcpy(&c->ctl->error, &zero, sizeof(int), cudaMemcpyHostToDevice);
        return fail(c, err == efs::DEV_ERR_BAD_BOUNDARY ? EFS_ERR_ARG : EFS_ERR_DEVICE_FAULT, buf);
    }
    return EFS_OK;
}

// The step graphs bake in whether the forces field is used: recapture them the first time it is.
int note_forces(efs_ctx* c) {
    if (!c->has_forces) {
        CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
        drop_graphs(c);
        c->has_forces = true;
    }
    return EFS_OK;
}

// The FP64 vectors of EFS_CG_FP64, allocated the first time a context selects that variant.
int ensure_fp64_vectors(efs_ctx* c) {
    if (c->r64) return EFS_OK;
    const size_t N = (size_t)c->g.N;
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    CK(dalloc_halo(c, &c->r64, N), "cudaMalloc r64");
    CK(dalloc_halo(c, &c->d64, N), "cudaMalloc d64");
    CK(dalloc_halo(c, &c->t64, N), "cudaMalloc t64");
    return EFS_OK;
}

}  // namespace

namespace efs {
void drop_all_graphs(efs_ctx* c) {
    if (c->stream) cudaStreamSynchronize(c->stream);
    drop_graphs(c);
}
}  // namespace efs

extern "C" {

void efs_params_default(efs_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->dt = 0.0167f;
    p->gravity_force = 10.f;
    p->gravity_enabled = 1;
    p->vel_decay = 0.8f;
    p->lambda_minus = .5f;
    p->lambda_plus = .1f;
    p->eta = 1.f;
    p->liquid_threshold = 0.5f;
    p->rho_d = 3.f;
    p->solver = EFS_SOLVER_CG;
    p->max_steps = 2000;
    p->solver_threshold = 1e-5f;
    p->tol_rel = 0.f;
    p->disable_mask = 0;
    p->re_calc_div = 0;
    p->sharpen_mode = EFS_SHARPEN_PARALLEL;
    p->cg_variant = EFS_CG_MIXED_RECURRENCE;
    p->fcg_levels = -1;
    p->fcg_bottom = EFS_FCG_BOTTOM_UNET;
}

void efs_params_dam(efs_params* p, float cell_size, float dt, int solver, float tol_rel) {
    if (!p) return;
    efs_params_default(p);
    p->dt = dt;
    p->gravity_force = 9.81f / cell_size;
    p->lambda_minus = 50.f;
    p->lambda_plus = 10.f;
    p->eta = 100.f;
    p->rho_d = 32.f;
    p->solver = solver;
    p->tol_rel = tol_rel;
    p->disable_mask = EFS_STAGE_BIT(EFS_STAGE_VEL_DECAY);
}

int efs_abi_version(void) { return EFS_ABI_VERSION; }

int efs_device_count(int* count) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (count) *count = (e == cudaSuccess) ? n : 0;
    return (e == cudaSuccess || e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? EFS_OK : EFS_ERR_CUDA;
}

const char* efs_last_error(const efs_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

void efs_destroy(efs_ctx* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    drop_graphs(c);
    efs::ml_free(c);
    efs::unet_free(c);
    void* bufs[] = {c->u, c->v, c->w, c->rho, c->gamma, c->beta, c->fx, c->fy, c->fz, c->solid,
                    c->tvel, c->validA, c->validB, c->wb, c->wf, c->bb, c->fb, c->bsum, c->gsum, c->rho_acc,
                    c->sh_idx, c->sh_val, c->sh_end, c->rowinfo, c->chunk_flag, c->chunk_list, c->block_count,
                    c->partials, c->ctl, c->mass_partials, c->query_scratch, c->fstage};
    for (void* b : bufs) if (b) cudaFree(b);
    for (void* b : c->halo_bases) cudaFree(b);
    if (c->ctl_host) cudaFreeHost(c->ctl_host);
    for (auto ev : c->ev_begin) cudaEventDestroy(ev);
    for (auto ev : c->ev_end) cudaEventDestroy(ev);
    for (auto ev : c->marks) if (ev) cudaEventDestroy(ev);
    if (c->ev_solve_begin) cudaEventDestroy(c->ev_solve_begin);
    if (c->xfer) { cudaStreamSynchronize(c->xfer); cudaStreamDestroy(c->xfer); }
    if (c->ev_gamma) cudaEventDestroy(c->ev_gamma);
    if (c->ev_forces) cudaEventDestroy(c->ev_forces);
    if (c->ev_advected) cudaEventDestroy(c->ev_advected);
    if (c->ev_projected) cudaEventDestroy(c->ev_projected);
    if (c->ev_early) cudaEventDestroy(c->ev_early);
    if (c->ev_solve_end) cudaEventDestroy(c->ev_solve_end);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int efs_create(int dim, int width, int height, int depth, const efs_params* params, efs_ctx** out) {
    if (!out) return fail(nullptr, EFS_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (dim != 2 && dim != 3) return fail(nullptr, EFS_ERR_ARG, "dim must be 2 or 3");
    if (dim == 2 && depth != 1) return fail(nullptr, EFS_ERR_ARG, "2D grids have depth 1");
    if (width < 4 || height < 4 || (dim == 3 && depth < 4)) return fail(nullptr, EFS_ERR_ARG, "grid sides must be >= 4 (border included)");
    const long long n = (long long)width * height * depth;
    if (n >= (1LL << 31) / 8) return fail(nullptr, EFS_ERR_ARG, "grid too large for 32-bit cell indexing of 8-slot weights");
    std::string why;
    efs_params prm;
    if (params) prm = *params; else efs_params_default(&prm);
    if (!params_valid(&prm, why)) return fail(nullptr, EFS_ERR_ARG, why);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(nullptr, EFS_ERR_NO_DEVICE, "no CUDA device visible");

    efs_ctx* c = new efs_ctx();
    c->dim = dim;
    c->g.W = width; c->g.H = height; c->g.D = depth;
    c->g.WH = width * height;
    c->g.N = (int)n;
    c->prm = prm;
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    const size_t N = (size_t)n;
    const int K = (dim == 3) ? 8 : 4;
    const int nchunks = (int)((N + 31) / 32);
    auto bail = [&](cudaError_t e, const char* what) {
        g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
        efs_destroy(c);
        return EFS_ERR_CUDA;
    };
    cudaError_t e;
#define ALLOC(ptr, cnt) if ((e = dalloc(&(ptr), (cnt))) != cudaSuccess) return bail(e, "cudaMalloc " #ptr)
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "cudaStreamCreate");
    ALLOC(c->u, N); ALLOC(c->v, N); ALLOC(c->w, N);
    c->halo_cells = (dim == 3 ? (long long)width * height : (long long)width) + 64;
#define ALLOC_H(ptr, cnt) if ((e = dalloc_halo(c, &(ptr), (cnt))) != cudaSuccess) return bail(e, "cudaMalloc " #ptr)
    ALLOC(c->rho, N); ALLOC(c->gamma, N); ALLOC(c->beta, N); ALLOC_H(c->div, N); ALLOC_H(c->p, N);
    ALLOC(c->fx, N); ALLOC(c->fy, N); ALLOC(c->fz, N); ALLOC(c->solid, N);
    ALLOC(c->tvel, 3 * N); ALLOC(c->validA, N); ALLOC(c->validB, N);
    ALLOC(c->wb, K * N); ALLOC(c->wf, K * N); ALLOC(c->bb, N); ALLOC(c->fb, N);
    ALLOC(c->bsum, N); ALLOC(c->gsum, N); ALLOC(c->rho_acc, N);
    ALLOC(c->sh_idx, N); ALLOC(c->sh_val, N); ALLOC(c->sh_end, 3 * N);
    ALLOC(c->rowinfo, N); ALLOC(c->chunk_flag, nchunks); ALLOC(c->chunk_list, nchunks);
    ALLOC_H(c->r, N); ALLOC_H(c->d0, N); ALLOC_H(c->d1, N); ALLOC_H(c->e, N); ALLOC_H(c->p64, N); ALLOC_H(c->t, N);
#undef ALLOC_H
    ALLOC(c->ctl, 1);
    ALLOC(c->mass_partials, 256);
#undef ALLOC
    if ((e = efs::solver_configure(c)) != cudaSuccess) return bail(e, "solver occupancy");
    if ((e = dalloc(&c->block_count, c->solver_blocks)) != cudaSuccess) return bail(e, "cudaMalloc block_count");
    if ((e = dalloc(&c->partials, 6 * (size_t)c->solver_blocks)) != cudaSuccess) return bail(e, "cudaMalloc partials");
    if ((e = cudaMallocHost(reinterpret_cast<void**>(&c->ctl_host), sizeof(DevCtl))) != cudaSuccess) return bail(e, "cudaMallocHost");
    if ((e = cudaEventCreate(&c->ev_solve_begin)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreateWithFlags(&c->ev_gamma, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreateWithFlags(&c->ev_forces, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreateWithFlags(&c->ev_advected, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreateWithFlags(&c->ev_projected, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreateWithFlags(&c->ev_early, cudaEventDisableTiming)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaStreamCreateWithFlags(&c->xfer, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "cudaStreamCreate");
    if ((e = cudaEventCreate(&c->ev_solve_end)) != cudaSuccess) return bail(e, "cudaEventCreate");
    if ((e = cudaMemsetAsync(c->ctl, 0, sizeof(DevCtl), c->stream)) != cudaSuccess) return bail(e, "cudaMemset");
    if ((e = cudaMemsetAsync(c->validB, 0, N, c->stream)) != cudaSuccess) return bail(e, "cudaMemset");
    if ((e = cudaMemsetAsync(c->r, 0, N * sizeof(float), c->stream)) != cudaSuccess) return bail(e, "cudaMemset");
    if ((e = cudaMemsetAsync(c->e, 0, N * sizeof(float), c->stream)) != cudaSuccess) return bail(e, "cudaMemset");
    if ((e = efs::launch_reset_fields(c)) != cudaSuccess) return bail(e, "reset");
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return bail(e, "cudaStreamSynchronize");
    if (prm.cg_variant == EFS_CG_FP64) {
        const int s = ensure_fp64_vectors(c);
        if (s != EFS_OK) { efs_destroy(c); return s; }
    }
    *out = c;
    return EFS_OK;
}

int efs_set_params(efs_ctx* c, const efs_params* p) {
    if (!c) return EFS_ERR_ARG;
    std::string why;
    if (!params_valid(p, why)) return fail(c, EFS_ERR_ARG, why);
    if (p->cg_variant == EFS_CG_FP64) {
        const int s = ensure_fp64_vectors(c);
        if (s != EFS_OK) return s;
    }
    if (std::memcmp(&c->prm, p, sizeof(efs_params)) != 0) {
        CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
        drop_graphs(c);
        c->prm = *p;
    }
    return EFS_OK;
}

int efs_download_pressure_fp64(efs_ctx* c, double* host) {
    if (!c) return EFS_ERR_ARG;
    if (!host) return fail(c, EFS_ERR_ARG, "host pointer is NULL");
    const bool fcg = c->prm.solver == EFS_SOLVER_FCG_UNET;
    if (!fcg && (c->prm.solver != EFS_SOLVER_CG || c->prm.cg_variant == EFS_CG_REFERENCE))
        return fail(c, EFS_ERR_STATE, "no FP64 pressure: the solver is not CG with an FP64 accumulator, nor FCG");
    CK(cudaMemcpyAsync(host, c->p64, (size_t)c->g.N * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "download p64");
    return check_device_status(c);
}

int efs_get_params(const efs_ctx* c, efs_params* p) {
    if (!c || !p) return EFS_ERR_ARG;
    *p = c->prm;
    return EFS_OK;
}

}  // extern "C"

namespace {

// The device address of a page-locked host buffer (which the GPU addresses directly: on GB300 over NVLink-C2C),
// or null for pageable memory.  Kernels read such buffers at the link's rate (the velocity and force split
// and the boundary conversion read them in place), but writing the interleaved velocity into one from a
// kernel runs at half of it; downloads therefore go through device staging and the copy engine.
void* mapped(const void* host) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return (at.type == cudaMemoryTypeHost && at.devicePointer) ? at.devicePointer : nullptr;
}

float* scalar_field(efs_ctx* c, int field) {
    switch (field) {
        case EFS_FIELD_RHO: return c->rho;
        case EFS_FIELD_GAMMA: return c->gamma;
        case EFS_FIELD_BETA: return c->beta;
        case EFS_FIELD_DIVERGENCE: return c->div;
        case EFS_FIELD_PRESSURE: return c->p;
        default: return nullptr;
    }
}

// Enqueue one field's upload on the context's stream (no host synchronisation).
int enqueue_upload(efs_ctx* c, int field, const float* host) {
    if (!host) return fail(c, EFS_ERR_ARG, "host pointer is NULL");
    const size_t N = (size_t)c->g.N, bytes = N * sizeof(float);
    switch (field) {
        case EFS_FIELD_VEL:
        case EFS_FIELD_FORCES: {
            const float* src = static_cast<const float*>(mapped(host));
            if (!src) {
                CK(cudaMemcpyAsync(c->tvel, host, bytes * c->dim, cudaMemcpyHostToDevice, c->stream), "upload");
                src = c->tvel;
            }
            if (field == EFS_FIELD_VEL) { CK(efs::launch_upload_vec(c, src, c->u, c->v, c->w), "split"); }
            else {
                CK(efs::launch_upload_vec(c, src, c->fx, c->fy, c->fz), "split");
                const int s = note_forces(c);
                if (s != EFS_OK) return s;
            }
            return EFS_OK;
        }
        case EFS_FIELD_BOUNDARY: {
            const float* src = static_cast<const float*>(mapped(host));
            if (!src) {
                CK(cudaMemcpyAsync(c->tvel, host, bytes, cudaMemcpyHostToDevice, c->stream), "upload");
                src = c->tvel;
            }
            CK(efs::launch_boundary_to_solid(c, src), "boundary");
            return EFS_OK;
        }
        default: {
            float* dst = scalar_field(c, field);
            if (!dst) return fail(c, EFS_ERR_ARG, "unknown field");
            CK(cudaMemcpyAsync(dst, host, bytes, cudaMemcpyHostToDevice, c->stream), "upload");
            return EFS_OK;
        }
    }
}

// Enqueue one field's download on stream `st` (default: the context's; no host synchronisation).
int enqueue_download(efs_ctx* c, int field, float* host, cudaStream_t st = nullptr) {
    if (!host) return fail(c, EFS_ERR_ARG, "host pointer is NULL");
    if (!st) st = c->stream;
    const size_t N = (size_t)c->g.N, bytes = N * sizeof(float);
    switch (field) {
        case EFS_FIELD_VEL:
        case EFS_FIELD_FORCES: {
            if (field == EFS_FIELD_VEL) { CK(efs::launch_download_vec(c, c->tvel, c->u, c->v, c->w, st), "interleave"); }
            else { CK(efs::launch_download_vec(c, c->tvel, c->fx, c->fy, c->fz, st), "interleave"); }
            CK(cudaMemcpyAsync(host, c->tvel, bytes * c->dim, cudaMemcpyDeviceToHost, st), "download");
            return EFS_OK;
        }
        case EFS_FIELD_BOUNDARY: {      // converted on the context's stream
            CK(efs::launch_solid_to_boundary(c, c->tvel), "boundary");
            CK(cudaMemcpyAsync(host, c->tvel, bytes, cudaMemcpyDeviceToHost, c->stream), "download");
            return EFS_OK;
        }
        default: {
            const float* src = scalar_field(c, field);
            if (!src) return fail(c, EFS_ERR_ARG, "unknown field");
            CK(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, st), "download");
            return EFS_OK;
        }
    }
}

}  // namespace

extern "C" {

int efs_upload_field(efs_ctx* c, int field, const float* host) {
    if (!c) return EFS_ERR_ARG;
    const int s = enqueue_upload(c, field, host);
    if (s != EFS_OK) return s;
    if (field == EFS_FIELD_BOUNDARY) return check_device_status(c);
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

int efs_download_field(efs_ctx* c, int field, float* host) {
    if (!c) return EFS_ERR_ARG;
    const int s = enqueue_download(c, field, host);
    if (s != EFS_OK) return s;
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

// All given fields are enqueued on the stream, then one synchronisation (and the boundary check).  The
// staging buffer is reused between fields only in stream order, so no host wait is needed in between.
int efs_upload_fields(efs_ctx* c, const float* vel, const float* rho, const float* gamma, const float* boundary,
                      const float* forces) {
    if (!c) return EFS_ERR_ARG;
    int s;
    if (boundary && (s = enqueue_upload(c, EFS_FIELD_BOUNDARY, boundary)) != EFS_OK) return s;
    if (vel && (s = enqueue_upload(c, EFS_FIELD_VEL, vel)) != EFS_OK) return s;
    if (rho && (s = enqueue_upload(c, EFS_FIELD_RHO, rho)) != EFS_OK) return s;
    if (gamma && (s = enqueue_upload(c, EFS_FIELD_GAMMA, gamma)) != EFS_OK) return s;
    if (forces && (s = enqueue_upload(c, EFS_FIELD_FORCES, forces)) != EFS_OK) return s;
    return check_device_status(c);
}

int efs_download_fields(efs_ctx* c, float* vel, float* rho, float* gamma, float* beta, float* divergence,
                        float* pressure) {
    if (!c) return EFS_ERR_ARG;
    int s;
    if (vel && (s = enqueue_download(c, EFS_FIELD_VEL, vel)) != EFS_OK) return s;
    if (rho && (s = enqueue_download(c, EFS_FIELD_RHO, rho)) != EFS_OK) return s;
    if (gamma && (s = enqueue_download(c, EFS_FIELD_GAMMA, gamma)) != EFS_OK) return s;
    if (beta && (s = enqueue_download(c, EFS_FIELD_BETA, beta)) != EFS_OK) return s;
    if (divergence && (s = enqueue_download(c, EFS_FIELD_DIVERGENCE, divergence)) != EFS_OK) return s;
    if (pressure && (s = enqueue_download(c, EFS_FIELD_PRESSURE, pressure)) != EFS_OK) return s;
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

// One step with host fields in and out (the upload / update / download of a host-mirrored grid,
// CudaGrid3D::upload and download around ISimulator::update).  With page-locked buffers the transfers that do
// not block a stage overlap the step: gamma and forces are uploaded on the transfer stream while
// vel_extrapolate and rho_sharpen run (the step graph waits for them before rho_advect), rho, gamma and
// beta, final after rho_advect, are downloaded on it while vel_advect and the pressure solve run, and the
// divergence, final after project_pre, while the solve runs.
int efs_step_host(efs_ctx* c, const float* vel, const float* rho, const float* gamma, const float* boundary,
                  const float* forces, float* vel_out, float* rho_out, float* gamma_out, float* beta_out, float* div_out,
                  float* p_out) {
    if (!c) return EFS_ERR_ARG;
    auto locked = [](const void* p) { return !p || mapped(p) != nullptr; };
    // the copy engine overlaps only page-locked transfers with kernels
    const bool overlap = c->prm.solver != EFS_SOLVER_FCG_UNET && locked(gamma) && locked(forces) && locked(rho_out) &&
                         locked(gamma_out) && locked(beta_out) && locked(div_out);
    int s;
    if (!overlap) {
        if ((s = efs_upload_fields(c, vel, rho, gamma, boundary, forces)) != EFS_OK) return s;
        if ((s = efs_step(c, 1)) != EFS_OK) return s;
        return efs_download_fields(c, vel_out, rho_out, gamma_out, beta_out, div_out, p_out);
    }
    const size_t bytes = (size_t)c->g.N * sizeof(float);
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");     // nothing of an earlier call still reads
    if (forces && (s = note_forces(c)) != EFS_OK) return s;
    // inputs of the first stages, on the compute stream
    if (boundary && (s = enqueue_upload(c, EFS_FIELD_BOUNDARY, boundary)) != EFS_OK) return s;
    if (vel && (s = enqueue_upload(c, EFS_FIELD_VEL, vel)) != EFS_OK) return s;
    if (rho && (s = enqueue_upload(c, EFS_FIELD_RHO, rho)) != EFS_OK) return s;
    // inputs first read by rho_advect (gamma) and vel_advect (forces), on the transfer stream once the first
    // stages' inputs are up (the host link is the bottleneck: sharing it would delay the first stage); the
    // step waits for each where it first reads it, so the forces move while rho_advect runs
    CK(cudaEventRecord(c->ev_early, c->stream), "cudaEventRecord");
    CK(cudaStreamWaitEvent(c->xfer, c->ev_early, 0), "cudaStreamWaitEvent");
    if (gamma) CK(cudaMemcpyAsync(c->gamma, gamma, bytes, cudaMemcpyHostToDevice, c->xfer), "upload gamma");
    CK(cudaEventRecord(c->ev_gamma, c->xfer), "cudaEventRecord");
    if (forces) {
        // the copy engine brings the interleaved forces up; a short split kernel follows (a kernel reading the
        // host buffer itself would wait for SMs behind the first stages)
        if (!c->fstage) CK(cudaMalloc(&c->fstage, bytes * c->dim), "cudaMalloc force staging");
        CK(cudaMemcpyAsync(c->fstage, forces, bytes * c->dim, cudaMemcpyHostToDevice, c->xfer), "upload forces");
        CK(efs::launch_upload_vec(c, c->fstage, c->fx, c->fy, c->fz, c->xfer), "split forces");
    }
    CK(cudaEventRecord(c->ev_forces, c->xfer), "cudaEventRecord");
    if ((s = efs_step(c, 1)) != EFS_OK) return s;
    // rho, gamma, beta: on the transfer stream once rho_advect is done
    CK(cudaStreamWaitEvent(c->xfer, c->ev_advected, 0), "cudaStreamWaitEvent");
    if (rho_out && (s = enqueue_download(c, EFS_FIELD_RHO, rho_out, c->xfer)) != EFS_OK) return s;
    if (gamma_out && (s = enqueue_download(c, EFS_FIELD_GAMMA, gamma_out, c->xfer)) != EFS_OK) return s;
    if (beta_out && (s = enqueue_download(c, EFS_FIELD_BETA, beta_out, c->xfer)) != EFS_OK) return s;
    // the divergence, final after project_pre, while the pressure solve runs
    CK(cudaStreamWaitEvent(c->xfer, c->ev_projected, 0), "cudaStreamWaitEvent");
    if (div_out && (s = enqueue_download(c, EFS_FIELD_DIVERGENCE, div_out, c->xfer)) != EFS_OK) return s;
    // the fields of the last stages, after the step on the compute stream
    if (vel_out && (s = enqueue_download(c, EFS_FIELD_VEL, vel_out)) != EFS_OK) return s;
    if (p_out && (s = enqueue_download(c, EFS_FIELD_PRESSURE, p_out)) != EFS_OK) return s;
    CK(cudaStreamSynchronize(c->xfer), "cudaStreamSynchronize");
    return check_device_status(c);
}

int efs_reset_fields(efs_ctx* c) {
    if (!c) return EFS_ERR_ARG;
    CK(efs::launch_reset_fields(c), "reset");
    c->has_forces = false;
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

int efs_stage(efs_ctx* c, int stage) {
    if (!c) return EFS_ERR_ARG;
    if (stage < 0 || stage >= EFS_STAGE_COUNT) return fail(c, EFS_ERR_ARG, "unknown stage");
    if (stage == EFS_STAGE_PROJECT) {
        const int s = prepare_fcg(c);
        if (s != EFS_OK) return s;
    }
    CK(efs::launch_stage(c, stage, false), "stage launch");
    return EFS_OK;
}

int efs_step(efs_ctx* c, int n_steps) {
    if (!c) return EFS_ERR_ARG;
    if (n_steps < 0) return fail(c, EFS_ERR_ARG, "n_steps < 0");
    if (n_steps == 0) return EFS_OK;
    efs::GraphKey key{EFS_STAGES_ALL & ~c->prm.disable_mask, c->prm.solver, c->prm.cg_variant};
    cudaGraphExec_t exec = nullptr;
    int s = build_graph(c, key, &exec);
    if (s != EFS_OK) return s;
    auto nb = c->timing_nodes_begin.find(key), ne = c->timing_nodes_end.find(key);
    const bool can_time = nb != c->timing_nodes_begin.end() && ne != c->timing_nodes_end.end();
    for (int k = 0; k < n_steps; k++) {
        if (can_time && c->ev_used < c->ev_capacity) {
            CK(cudaGraphExecEventRecordNodeSetEvent(exec, nb->second, c->ev_begin[c->ev_used]), "timing event");
            CK(cudaGraphExecEventRecordNodeSetEvent(exec, ne->second, c->ev_end[c->ev_used]), "timing event");
            c->ev_used++;
        } else if (can_time && c->ev_capacity > 0) {
            CK(cudaGraphExecEventRecordNodeSetEvent(exec, nb->second, c->ev_solve_begin), "timing event");
            CK(cudaGraphExecEventRecordNodeSetEvent(exec, ne->second, c->ev_solve_end), "timing event");
        }
        CK(cudaGraphLaunch(exec, c->stream), "cudaGraphLaunch");
    }
    c->frames += n_steps;
    return EFS_OK;
}

int efs_step_kernel_count(efs_ctx* c, int* count) {
    if (!c || !count) return EFS_ERR_ARG;
    efs::GraphKey key{EFS_STAGES_ALL & ~c->prm.disable_mask, c->prm.solver, c->prm.cg_variant};
    cudaGraphExec_t exec = nullptr;
    int s = build_graph(c, key, &exec);
    if (s != EFS_OK) return s;
    *count = c->kernel_nodes[key];
    return EFS_OK;
}

int efs_solve(efs_ctx* c, efs_stats* out) {
    if (!c) return EFS_ERR_ARG;
    const int ps = prepare_fcg(c);
    if (ps != EFS_OK) return ps;
    CK(efs::launch_solver_prep(c), "solver prep");
    CK(efs::launch_solver(c), "solver launch");
    int s = efs_get_stats(c, out);
    if (s != EFS_OK) return s;
    if (!c->ctl_host->converged) return fail(c, EFS_ERR_NOT_CONVERGED, "pressure solve reached max_steps");
    return EFS_OK;
}

int efs_fcg_time_vcycle(efs_ctx* c, int reps, float* ms_direct, float* ms_graph) {
    if (!c || reps < 1 || !ms_direct || !ms_graph) return EFS_ERR_ARG;
    if (c->prm.solver != EFS_SOLVER_FCG_UNET) return fail(c, EFS_ERR_STATE, "solver is not EFS_SOLVER_FCG_UNET");
    const int ps = prepare_fcg(c);
    if (ps != EFS_OK) return ps;
    CK(efs::launch_solver_prep(c), "solver prep");
    CK(efs::ml_time_vcycle(c, reps, ms_direct, ms_graph), "V-cycle timing");
    return check_device_status(c);
}

int efs_synchronize(efs_ctx* c) {
    if (!c) return EFS_ERR_ARG;
    return check_device_status(c);
}

int efs_get_stats(efs_ctx* c, efs_stats* out) {
    if (!c) return EFS_ERR_ARG;
    int s = check_device_status(c);
    if (s != EFS_OK) return s;
    if (out) {
        const DevCtl& h = *c->ctl_host;
        std::memset(out, 0, sizeof(*out));
        out->frames = c->frames;
        out->solve_steps = h.iterations;
        out->converged = h.converged;
        out->paused = h.paused;
        out->device_error = h.error;
        out->rr = h.rr;
        out->bb = h.bb;
        out->threshold = h.thr;
        out->active_cells = h.active_cells;
        out->total_solve_steps = h.total_iterations;
        out->solves = h.solves;
        out->precond_steps = h.precond_iterations;
    }
    return EFS_OK;
}

int efs_total_mass(efs_ctx* c, double* out) {
    if (!c || !out) return EFS_ERR_ARG;
    CK(efs::launch_mass(c, c->mass_partials), "mass");
    double part[256];
    CK(cudaMemcpyAsync(part, c->mass_partials, sizeof part, cudaMemcpyDeviceToHost, c->stream), "mass readback");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    double s = 0;
    for (double v : part) s += v;
    *out = s;
    return EFS_OK;
}

int efs_solve_timing_arm(efs_ctx* c, int capacity) {
    if (!c || capacity < 0) return EFS_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    // the pool only grows (events stay alive while a graph's event-record nodes may refer to them)
    while ((int)c->ev_begin.size() < capacity) {
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a), "cudaEventCreate");
        CK(cudaEventCreate(&b), "cudaEventCreate");
        c->ev_begin.push_back(a);
        c->ev_end.push_back(b);
    }
    c->ev_capacity = capacity;
    c->ev_used = 0;
    // work counters restart with the pool
    CK(cudaMemset(&c->ctl->sum_iter_rows, 0, 2 * sizeof(double)), "cudaMemset");
    return EFS_OK;
}

int efs_solve_timing_read(efs_ctx* c, int* launches, double* total_ms, double* row_iterations,
                          double* row_setups) {
    if (!c) return EFS_ERR_ARG;
    int s = check_device_status(c);
    if (s != EFS_OK) return s;
    double ms = 0;
    for (int k = 0; k < c->ev_used; k++) {
        float t = 0;
        CK(cudaEventElapsedTime(&t, c->ev_begin[k], c->ev_end[k]), "cudaEventElapsedTime");
        ms += t;
    }
    if (launches) *launches = c->ev_used;
    if (total_ms) *total_ms = ms;
    if (row_iterations) *row_iterations = c->ctl_host->sum_iter_rows;
    if (row_setups) *row_setups = c->ctl_host->sum_rows;
    return EFS_OK;
}

int efs_timer_mark(efs_ctx* c, int slot) {
    if (!c || slot < 0 || slot >= 8) return EFS_ERR_ARG;
    if (!c->marks[slot]) CK(cudaEventCreate(&c->marks[slot]), "cudaEventCreate");
    CK(cudaEventRecord(c->marks[slot], c->stream), "cudaEventRecord");
    return EFS_OK;
}

int efs_timer_elapsed(efs_ctx* c, int a, int b, double* ms) {
    if (!c || !ms || a < 0 || a >= 8 || b < 0 || b >= 8 || !c->marks[a] || !c->marks[b]) return EFS_ERR_ARG;
    CK(cudaEventSynchronize(c->marks[b]), "cudaEventSynchronize");
    float t = 0;
    CK(cudaEventElapsedTime(&t, c->marks[a], c->marks[b]), "cudaEventElapsedTime");
    *ms = t;
    return EFS_OK;
}

// ---- scene construction and queries (efs_scene.cu) --------------------------------------------------------

int efs_mesh_label(efs_ctx* c, int field, const float* tris, int ntri, const float center[3], const float size[3],
                   float vin, float vout) {
    if (!c) return EFS_ERR_ARG;
    if (c->dim != 3) return fail(c, EFS_ERR_ARG, "mesh labels are 3D only");
    if ((ntri > 0 && !tris) || ntri < 0 || !center || !size) return fail(c, EFS_ERR_ARG, "bad triangles or domain");
    efs::FieldPtrsOut o;
    if (!efs::scene_field_ptrs(c, field, o) || o.ncomp != 1) return fail(c, EFS_ERR_ARG, "field must be scalar or the boundary");
    if (field == EFS_FIELD_BOUNDARY && !((vin == 0.0f || vin == 1.0f) && (vout == 0.0f || vout == 1.0f)))
        return fail(c, EFS_ERR_ARG, "boundary values are 0.0 or 1.0");
    float* d_tris = nullptr;
    const size_t bytes = (size_t)std::max(ntri, 1) * 12 * sizeof(float);
    CK(cudaMalloc(&d_tris, bytes), "cudaMalloc triangles");
    cudaError_t e = ntri > 0 ? cudaMemcpyAsync(d_tris, tris, (size_t)ntri * 12 * sizeof(float), cudaMemcpyHostToDevice, c->stream)
                             : cudaSuccess;
    if (e == cudaSuccess) e = efs::launch_mesh_label(c, d_tris, ntri, center, size, vin, vout, field, nullptr);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_tris);
    if (e != cudaSuccess) return cuda_fail(c, e, "mesh label");
    return EFS_OK;
}

int efs_mesh_cells(efs_ctx* c, const float* tris, int ntri, const float center[3], const float size[3], int* cells,
                   long long capacity, long long* count) {
    if (!c) return EFS_ERR_ARG;
    if (c->dim != 3) return fail(c, EFS_ERR_ARG, "mesh labels are 3D only");
    if ((ntri > 0 && !tris) || ntri < 0 || !center || !size || !count || capacity < 0 || (capacity > 0 && !cells))
        return fail(c, EFS_ERR_ARG, "bad arguments");
    const long long N = c->g.N, tiles = efs::mask_tiles(c), cap = std::min(capacity, N);
    float* d_tris = nullptr;
    uint8_t* mask = nullptr;
    int *counts = nullptr, *out = nullptr;
    long long* offsets = nullptr;
    cudaError_t e = cudaMalloc(&d_tris, (size_t)std::max(ntri, 1) * 12 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&mask, (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc(&counts, (size_t)tiles * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&offsets, (size_t)(tiles + 1) * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&out, (size_t)std::max(cap, 1LL) * sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(mask, 0, (size_t)N, c->stream);
    if (e == cudaSuccess && ntri > 0)
        e = cudaMemcpyAsync(d_tris, tris, (size_t)ntri * 12 * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = efs::launch_mesh_label(c, d_tris, ntri, center, size, 1.0f, 0.0f, EFS_FIELD_RHO, mask);
    if (e == cudaSuccess) e = efs::launch_mask_compact(c, mask, out, cap, counts, offsets);
    long long total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, offsets + tiles, sizeof(long long), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && cap > 0 && total > 0)
        e = cudaMemcpy(cells, out, (size_t)std::min(total, cap) * sizeof(int), cudaMemcpyDeviceToHost);
    for (void* b : {(void*)d_tris, (void*)mask, (void*)counts, (void*)offsets, (void*)out}) if (b) cudaFree(b);
    if (e != cudaSuccess) return cuda_fail(c, e, "mesh cells");
    *count = total;
    return EFS_OK;
}

int efs_fill_box(efs_ctx* c, int field, const int lo[3], const int hi[3], const float* value) {
    if (!c) return EFS_ERR_ARG;
    if (!lo || !hi || !value) return fail(c, EFS_ERR_ARG, "lo, hi and value must not be NULL");
    efs::FieldPtrsOut o;
    if (!efs::scene_field_ptrs(c, field, o)) return fail(c, EFS_ERR_ARG, "unknown field");
    if (field == EFS_FIELD_BOUNDARY && !(value[0] == 0.0f || value[0] == 1.0f))
        return fail(c, EFS_ERR_ARG, "boundary values are 0.0 or 1.0");
    const int dims[3] = {c->g.W, c->g.H, c->dim == 3 ? c->g.D : 1};
    int l[3], h[3];
    for (int d = 0; d < 3; d++) { l[d] = std::max(0, lo[d]); h[d] = std::min(dims[d], hi[d]); }
    if (c->dim == 2) { l[2] = 0; h[2] = 1; }
    CK(efs::launch_fill_box(c, field, l, h, value), "fill box");
    if (field == EFS_FIELD_FORCES) { const int s = note_forces(c); if (s != EFS_OK) return s; }
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

int efs_set_cells(efs_ctx* c, int field, const int* cells, long long n, const float* value) {
    if (!c) return EFS_ERR_ARG;
    if (n < 0 || (n > 0 && !cells) || !value) return fail(c, EFS_ERR_ARG, "bad cell list or value");
    efs::FieldPtrsOut o;
    if (!efs::scene_field_ptrs(c, field, o)) return fail(c, EFS_ERR_ARG, "unknown field");
    if (field == EFS_FIELD_BOUNDARY && !(value[0] == 0.0f || value[0] == 1.0f))
        return fail(c, EFS_ERR_ARG, "boundary values are 0.0 or 1.0");
    if (n == 0) return EFS_OK;
    int* d_cells = nullptr;
    CK(cudaMalloc(&d_cells, (size_t)n * sizeof(int)), "cudaMalloc cells");
    cudaError_t e = cudaMemcpyAsync(d_cells, cells, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = efs::launch_set_cells(c, field, d_cells, n, value);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_cells);
    if (e != cudaSuccess) return cuda_fail(c, e, "set cells");
    if (field == EFS_FIELD_FORCES) { const int s = note_forces(c); if (s != EFS_OK) return s; }
    CK(cudaMemcpy(c->ctl_host, c->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost), "read device status");
    if (c->ctl_host->error & efs::DEV_ERR_BAD_INDEX) {
        const int cleared = c->ctl_host->error & ~efs::DEV_ERR_BAD_INDEX;
        cudaMemcpy(&c->ctl->error, &cleared, sizeof(int), cudaMemcpyHostToDevice);
        return fail(c, EFS_ERR_ARG, "a cell index is outside the grid");
    }
    return EFS_OK;
}

int efs_seal_boundary(efs_ctx* c) {
    if (!c) return EFS_ERR_ARG;
    CK(efs::launch_seal_boundary(c), "seal boundary");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

int efs_query_box(efs_ctx* c, const int position[3], const int scale[3], int only_fluid, efs_query_metrics* out) {
    if (!c) return EFS_ERR_ARG;
    if (!position || !scale || !out) return fail(c, EFS_ERR_ARG, "position, scale and out must not be NULL");
    const int dims[3] = {c->g.W, c->g.H, c->dim == 3 ? c->g.D : 2};
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = std::max(0, position[d]);
        hi[d] = std::min(dims[d] - 1, position[d] + scale[d]);
    }
    if (c->dim == 2) { lo[2] = 0; hi[2] = 1; }
    if (!c->query_scratch) CK(cudaMalloc(&c->query_scratch, efs::query_scratch_bytes()), "cudaMalloc query scratch");
    const size_t res_off = efs::query_scratch_bytes() - sizeof(efs_query_metrics) - 64;
    efs_query_metrics* d_out = reinterpret_cast<efs_query_metrics*>(static_cast<char*>(c->query_scratch) + res_off);
    CK(efs::launch_query_box(c, lo, hi, only_fluid, c->query_scratch, d_out), "query box");
    CK(cudaMemcpyAsync(out, d_out, sizeof(efs_query_metrics), cudaMemcpyDeviceToHost, c->stream), "download metrics");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

int efs_scene_dam3d(int w, int h, int d, int n_min, int n_max, uint64_t seed, float* boundary, float* rho) {
    if (!boundary || !rho) return EFS_ERR_ARG;
    return efs_scene_dam3d_fill(w, h, d, n_min, n_max, seed, boundary, rho) < 0 ? EFS_ERR_ARG : EFS_OK;
}

int efs_scene_dam2d(int w, int h, float* boundary, float* rho) {
    if (!boundary || !rho) return EFS_ERR_ARG;
    return efs_scene_dam2d_fill(w, h, boundary, rho) < 0 ? EFS_ERR_ARG : EFS_OK;
}

int efs_scene_batch2d(uint64_t seed, int* side, float* boundary, float* rho, int capacity) {
    int s = 0;
    efs_scene_batch2d_fill(seed, &s, nullptr, nullptr);
    if (side) *side = s;
    if (!boundary || !rho) return EFS_OK;
    if (capacity < s * s) return EFS_ERR_ARG;
    return efs_scene_batch2d_fill(seed, &s, boundary, rho) < 0 ? EFS_ERR_ARG : EFS_OK;
}

}  // extern "C"
