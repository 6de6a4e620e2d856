// efs_noalloc.cu — the pressure solve without any device allocation (efs_solve_noalloc).
//
// Some callers cannot call cudaMalloc: a host application that hands its simulation plug-ins a fixed device
// budget and owns every allocation, a real-time loop where the implicit device synchronisation of cudaMalloc /
// cudaFree is not allowed, or code that records its work into a CUDA graph.  For them this entry point solves
// on the caller's device buffers and keeps its working vectors in one file-scope __device__ array of fixed
// size (EFS_NOALLOC_SCRATCH_BYTES, about 13.2 MB), which every device that loads the library holds until the
// process exits.  It covers grids up to EFS_NOALLOC_MAX_CELLS cells (larger grids are rejected with
// EFS_ERR_ARG) and has no counterpart in the reference, whose solvers own heap-allocated fields.
//
// All calls share the array and find it as the previous call left it: everything the solve reads is written
// first in the same call (the control block is cleared, the matrix rows and the working vectors are
// rebuilt), and calls whose work overlaps on the GPU race on it.
#include <cstring>
#include <mutex>
#include <string>

#include "efs_internal.h"

namespace efs {
cudaError_t solver_launch_shape(int n_chunks, int sm_count, int* blocks_out, size_t* smem_out);
cudaError_t launch_solver_args(const SolverArgs& a, int blocks, size_t smem, cudaStream_t stream);
}  // namespace efs

namespace {

using efs::DevCtl;
using efs::Geo;

constexpr long long kMaxCells = EFS_NOALLOC_MAX_CELLS;
constexpr long long kMaxHalo = (1LL << 16) + 64;          // one z plane (3D) or one row (2D) plus a chunk
constexpr long long kMaxChunks = kMaxCells / 32;
constexpr int kMaxBlocks = (int)((kMaxChunks + 63) / 64);  // the launch rule gives at most one block per 64 chunks
constexpr long long kVec = kMaxCells + 2 * kMaxHalo;       // one working vector with its halo on both sides

constexpr size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }
constexpr size_t kOffCtl = 0;
constexpr size_t kOffRowinfo = align256(kOffCtl + sizeof(DevCtl));
constexpr size_t kOffChunkFlag = align256(kOffRowinfo + kMaxCells * sizeof(uint16_t));
constexpr size_t kOffChunkList = align256(kOffChunkFlag + kMaxChunks);
constexpr size_t kOffBlockCount = align256(kOffChunkList + kMaxChunks * sizeof(int));
constexpr size_t kOffPartials = align256(kOffBlockCount + kMaxBlocks * sizeof(int));
constexpr size_t kOffR = align256(kOffPartials + 6 * (size_t)kMaxBlocks * sizeof(double));
constexpr size_t kOffD0 = align256(kOffR + kVec * sizeof(float));
constexpr size_t kOffD1 = align256(kOffD0 + kVec * sizeof(float));
constexpr size_t kOffE = align256(kOffD1 + kVec * sizeof(float));
constexpr size_t kOffP = align256(kOffE + kVec * sizeof(float));
constexpr size_t kOffP64 = align256(kOffP + kVec * sizeof(float));
constexpr size_t kOffT = align256(kOffP64 + kVec * sizeof(double));
constexpr size_t kScratchBytes = align256(kOffT + kVec * sizeof(float));
static_assert(kScratchBytes == EFS_NOALLOC_SCRATCH_BYTES, "the header states the fixed scratch size");

// The solver's working memory (EFS_NOALLOC_SCRATCH_BYTES), zero at load, shared by every call on a device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Host code cannot use g_noalloc_scratch as an address: its device address is looked up once per device, in
// the context current at that first call (the device's primary context for runtime-API callers).  After a
// cudaDeviceReset, or from another driver context on the same device, the cached address is not valid; neither
// is supported.
std::mutex g_addr_mutex;
unsigned char* g_addr[64] = {};

// Per host thread, so that failing calls on different threads do not race on it; the text returned by
// efs_noalloc_last_error() stays valid until the next failing call on the same thread.
thread_local std::string g_noalloc_error;

int nfail(int code, const std::string& msg) {
    g_noalloc_error = msg;
    return code;
}

// Matrix rows and active-chunk flags from the caller's rho and float boundary (CGSolver.cpp:467-497), the
// solver's start pressure in the scratch copy (CG: p = b; Jacobi: the caller's current pressure).
template <int DIM>
__global__ void k_noalloc_prep(Geo g, const float* __restrict__ rho, const float* __restrict__ boundary,
                               const float* __restrict__ div, const float* __restrict__ p_in, float* __restrict__ p,
                               uint16_t* __restrict__ rowinfo, uint8_t* __restrict__ chunk_flag, int jacobi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool active = false;
    if (i < g.N) {
        const int x = i % g.W, y = (i / g.W) % g.H, z = (DIM == 3) ? i / g.WH : 0;
        const float d = div[i];
        p[i] = jacobi ? p_in[i] : d;
        uint16_t info = 0;
        if (!(rho[i] <= 0.5f || boundary[i] == 1.f)) {
            const int nx[6] = {x - 1, x + 1, x, x, x, x}, ny[6] = {y, y, y - 1, y + 1, y, y};
            const int nz[6] = {z, z, z, z, z - 1, z + 1};
            const int off[6] = {-1, 1, -g.W, g.W, -g.WH, g.WH};
            int cnt = 0;
#pragma unroll
            for (int k = 0; k < 2 * DIM; k++) {
                if (nx[k] <= 0 || nx[k] >= g.W - 1 || ny[k] <= 0 || ny[k] >= g.H - 1) continue;
                if (DIM == 3 && (nz[k] <= 0 || nz[k] >= g.D - 1)) continue;
                const int j = i + off[k];
                if (boundary[j] > 0.5f) continue;
                cnt++;
                if (rho[j] > 0.5f) info |= (uint16_t)(1u << k);
            }
            info |= (uint16_t)(cnt << 8) | (uint16_t)0x8000u;
        }
        rowinfo[i] = info;
        active = (info & 0x8000u) || d != 0.f || (jacobi && p[i] != 0.f);
    }
    const unsigned any = __ballot_sync(0xffffffffu, active);
    if ((threadIdx.x & 31) == 0 && (i >> 5) < ((g.N + 31) >> 5)) chunk_flag[i >> 5] = any ? 1 : 0;
}

}  // namespace

extern "C" int efs_solve_noalloc(int dim, int width, int height, int depth, const efs_params* params,
                                 const float* rho, const float* boundary, const float* divergence, float* pressure,
                                 void* stream, efs_stats* stats) {
    if (dim != 2 && dim != 3) return nfail(EFS_ERR_ARG, "dim must be 2 or 3");
    if (dim == 2) depth = 1;
    if (width < 4 || height < 4 || (dim == 3 && depth < 4)) return nfail(EFS_ERR_ARG, "grid sides must be >= 4 (border included)");
    const long long n = (long long)width * height * depth;
    const long long halo = (dim == 3 ? (long long)width * height : (long long)width) + 64;
    if (n > kMaxCells)
        return nfail(EFS_ERR_ARG, "grid has " + std::to_string(n) + " cells; efs_solve_noalloc handles at most " +
                                      std::to_string(kMaxCells));
    if (halo > kMaxHalo) return nfail(EFS_ERR_ARG, "grid planes too large for the fixed solver scratch");
    if (!params || !rho || !boundary || !divergence || !pressure) return nfail(EFS_ERR_ARG, "NULL argument");
    if (params->solver != EFS_SOLVER_JACOBI && params->solver != EFS_SOLVER_CG) return nfail(EFS_ERR_ARG, "unknown solver");
    if (params->cg_variant != EFS_CG_MIXED && params->cg_variant != EFS_CG_REFERENCE &&
        params->cg_variant != EFS_CG_MIXED_RECURRENCE)
        return nfail(EFS_ERR_ARG, "unknown cg_variant");
    if (params->max_steps < 0) return nfail(EFS_ERR_ARG, "max_steps must be >= 0");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return nfail(EFS_ERR_NO_DEVICE, cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return nfail(EFS_ERR_ARG, "device ordinal beyond 63");
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lock(g_addr_mutex);
        if (!g_addr[dev]) {
            // first call on this device (make it before any stream capture): find the array's device address
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess) return nfail(EFS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_addr[dev] = static_cast<unsigned char*>(ptr);
        }
        base = g_addr[dev];
    }
    int sm = 0;
    if ((e = cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return nfail(EFS_ERR_CUDA, cudaGetErrorString(e));
    const cudaStream_t st = static_cast<cudaStream_t>(stream);

    Geo g;
    g.W = width; g.H = height; g.D = depth; g.WH = width * height; g.N = (int)n;
    const int n_chunks = (int)((n + 31) / 32);
    int blocks = 0;
    size_t smem = 0;
    if ((e = efs::solver_launch_shape(n_chunks, sm, &blocks, &smem)) != cudaSuccess) return nfail(EFS_ERR_CUDA, cudaGetErrorString(e));
    if (blocks > kMaxBlocks) return nfail(EFS_ERR_STATE, "solver launch shape exceeds the fixed scratch");

    DevCtl* ctl = reinterpret_cast<DevCtl*>(base + kOffCtl);
    float* p_s = reinterpret_cast<float*>(base + kOffP) + kMaxHalo;
    efs::SolverArgs a{};      // the FP64-variant vectors stay null: that variant is rejected above
    a.g = g;
    a.dim = dim;
    a.solver = params->solver;
    a.cg_variant = params->cg_variant;
    a.max_steps = params->max_steps;
    a.tol_rel = params->tol_rel;
    a.solver_threshold = params->solver_threshold;
    a.n_chunks = n_chunks;
    a.b = divergence;
    uint16_t* rowinfo = reinterpret_cast<uint16_t*>(base + kOffRowinfo);
    a.rowinfo = rowinfo;
    a.chunk_flag = base + kOffChunkFlag;
    a.chunk_list = reinterpret_cast<int*>(base + kOffChunkList);
    a.block_count = reinterpret_cast<int*>(base + kOffBlockCount);
    a.partials = reinterpret_cast<double*>(base + kOffPartials);
    a.r = reinterpret_cast<float*>(base + kOffR) + kMaxHalo;
    a.d0 = reinterpret_cast<float*>(base + kOffD0) + kMaxHalo;
    a.d1 = reinterpret_cast<float*>(base + kOffD1) + kMaxHalo;
    a.e = reinterpret_cast<float*>(base + kOffE) + kMaxHalo;
    a.p = p_s;
    a.p64 = reinterpret_cast<double*>(base + kOffP64) + kMaxHalo;
    a.t = reinterpret_cast<float*>(base + kOffT) + kMaxHalo;
    a.ctl = ctl;

    if ((e = cudaMemsetAsync(ctl, 0, sizeof(DevCtl), st)) != cudaSuccess) return nfail(EFS_ERR_CUDA, cudaGetErrorString(e));
    const int threads = 256;
    const int nblk = (n_chunks * 32 + threads - 1) / threads;
    const int jacobi = params->solver == EFS_SOLVER_JACOBI;
    if (dim == 3)
        k_noalloc_prep<3><<<nblk, threads, 0, st>>>(g, rho, boundary, divergence, pressure, p_s, rowinfo, base + kOffChunkFlag, jacobi);
    else
        k_noalloc_prep<2><<<nblk, threads, 0, st>>>(g, rho, boundary, divergence, pressure, p_s, rowinfo, base + kOffChunkFlag, jacobi);
    if ((e = cudaGetLastError()) != cudaSuccess) return nfail(EFS_ERR_CUDA, cudaGetErrorString(e));
    if ((e = efs::launch_solver_args(a, blocks, smem, st)) != cudaSuccess) return nfail(EFS_ERR_CUDA, cudaGetErrorString(e));
    if ((e = cudaMemcpyAsync(pressure, p_s, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
        return nfail(EFS_ERR_CUDA, cudaGetErrorString(e));
    if (!stats) return EFS_OK;
    DevCtl h;
    if ((e = cudaMemcpyAsync(&h, ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return nfail(EFS_ERR_CUDA, cudaGetErrorString(e));
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return nfail(EFS_ERR_CUDA, cudaGetErrorString(e));
    std::memset(stats, 0, sizeof(*stats));
    stats->solve_steps = h.iterations;
    stats->converged = h.converged;
    stats->device_error = h.error;
    stats->rr = h.rr;
    stats->bb = h.bb;
    stats->threshold = h.thr;
    stats->active_cells = h.active_cells;
    stats->total_solve_steps = h.total_iterations;
    stats->solves = h.solves;
    if (h.error) return nfail(EFS_ERR_DEVICE_FAULT, "device status word " + std::to_string(h.error));
    if (!h.converged) return nfail(EFS_ERR_NOT_CONVERGED, "pressure solve reached max_steps");
    return EFS_OK;
}

extern "C" const char* efs_noalloc_last_error(void) { return g_noalloc_error.c_str(); }
