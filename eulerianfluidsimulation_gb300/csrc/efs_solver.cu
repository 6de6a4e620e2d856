// efs_solver.cu — the pressure solve of project() as one persistent, cooperative sm_103a kernel.
//
// Restates CGSolverCPU3D::solve / CGSolverCPU2D::solve (src/simulation/solver/CGSolver.cpp:32-83, :416-465)
// with impl_mat_mul (:85-111, :467-497), and JacobiSolverCPU3D/2D::solve (src/simulation/solver/
// JacobiSolver.cpp:18-71, :154-212).  Differences from the reference, all in what is computed where:
//   - the whole iteration runs inside one kernel: phases are separated by a grid barrier (bounded spin; a
//     barrier that gives up sets DEV_ERR_BARRIER_TIMEOUT and every block returns), the stop test is made on
//     the device, and no scalar goes to the host;
//   - dot products are accumulated in FP64: per-block partial sums, then every block adds the partials in
//     the same fixed order, so all blocks take the same branch and results do not depend on timing;
//   - only 32-cell chunks that hold a matrix row or a non-zero right-hand side are visited.  Rows outside
//     the matrix are the identity in the reference (result = x), start at p = b and keep r = d = 0, so
//     skipping them changes nothing;
//   - d <- beta d + r is fused into the next matrix-vector product (d is double-buffered), and the
//     product L d is recomputed in the update phase instead of being stored.
// EFS_CG_MIXED additionally keeps p as an FP64 accumulator plus an FP32 increment (see efs_gb300.h).
#include <cooperative_groups.h>
#include <cfloat>

#include "efs_internal.h"

namespace efs {

namespace {

constexpr int SOLVER_THREADS = 512;
constexpr int SOLVER_WARPS = SOLVER_THREADS / 32;
constexpr long long BARRIER_SPIN_LIMIT = 1LL << 25;   // ~ several seconds with the back-off below

// Grid-wide barrier for a cooperative launch.  Returns false when it (or another block) gave up.
__device__ bool grid_barrier(DevCtl* ctl) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &ctl->bar_gen;
        volatile int* vabort = &ctl->bar_abort;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&ctl->bar_count, 1u);
        int ok = 1;
        if (arrived == gridDim.x - 1) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            atomicAdd(&ctl->bar_gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == gen) {
                if (*vabort) { ok = 0; break; }
                __nanosleep(40);
                if (++spins > BARRIER_SPIN_LIMIT) {
                    atomicOr(&ctl->error, DEV_ERR_BARRIER_TIMEOUT);
                    atomicExch(&ctl->bar_abort, 1);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Block sums of three doubles; thread 0 stores them as this block's partials in `slot`.
__device__ void block_partials(double a, double b, double c, double* partials, int slot) {
    __shared__ double s_v[3][SOLVER_WARPS];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { s_v[0][warp] = a; s_v[1][warp] = b; s_v[2][warp] = c; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0, tb = 0, tc = 0;
        for (int k = 0; k < SOLVER_WARPS; k++) { ta += s_v[0][k]; tb += s_v[1][k]; tc += s_v[2][k]; }
        double* dst = partials + (size_t)slot * 3 * gridDim.x + 3 * blockIdx.x;
        dst[0] = ta; dst[1] = tb; dst[2] = tc;
    }
}

// Every block adds all blocks' partials of `slot` in the same order; totals returned to every thread.
__device__ void grid_totals(const double* partials, int slot, double& a, double& b, double& c) {
    __shared__ double s_tot[3];
    const volatile double* src = partials + (size_t)slot * 3 * gridDim.x;
    if (threadIdx.x < 32) {
        double ta = 0, tb = 0, tc = 0;
        for (int k = threadIdx.x; k < (int)gridDim.x; k += 32) { ta += src[3 * k]; tb += src[3 * k + 1]; tc += src[3 * k + 2]; }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ta += __shfl_down_sync(0xffffffffu, ta, o);
            tb += __shfl_down_sync(0xffffffffu, tb, o);
            tc += __shfl_down_sync(0xffffffffu, tc, o);
        }
        if (threadIdx.x == 0) { s_tot[0] = ta; s_tot[1] = tb; s_tot[2] = tc; }
    }
    __syncthreads();
    a = s_tot[0]; b = s_tot[1]; c = s_tot[2];
    __syncthreads();
}

// Grid reduction with two alternating partial slots: put (block partials), grid barrier, get (totals).
// A slot is rewritten two reductions later, after every block has passed the barrier of the reduction in
// between, so no second barrier is needed.
struct Reduction {
    double* partials;
    int slot;
    __device__ bool run(DevCtl* ctl, double a, double b, double c, double& ta, double& tb, double& tc);
};

__device__ bool Reduction::run(DevCtl* ctl, double a, double b, double c, double& ta, double& tb, double& tc) {
    block_partials(a, b, c, partials, slot);
    if (!grid_barrier(ctl)) return false;
    grid_totals(partials, slot, ta, tb, tc);
    slot ^= 1;
    return true;
}

// Neighbour order of the reference matrix-vector product: x-1, x+1, y-1, y+1, z+1, z-1 (CGSolver.cpp:489-494)
// and of the Jacobi sweep: x-1, x+1, y-1, y+1, z-1, z+1 (JacobiSolver.cpp:189-194).  rowinfo bits are
// x-1, x+1, y-1, y+1, z-1, z+1.
struct Nb {
    int o[6];
};
__device__ __forceinline__ Nb cg_order(const Geo& g) { return Nb{{-1, 1, -g.W, g.W, g.WH, -g.WH}}; }
__device__ __forceinline__ int cg_bit(int k) { return (k == 4) ? 5 : (k == 5 ? 4 : k); }

// L x (float, reference rounding) on row i
__device__ __forceinline__ float lap_f(const float* x, uint16_t info, int i, const Nb& nb) {
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; k++)
        if (info & (1u << cg_bit(k))) sum += x[i + nb.o[k]];
    return sum - (float)((info >> 8) & 7) * x[i];
}
// L d for d = beta * dp + r evaluated on the fly (the same float operations as forming d first)
__device__ __forceinline__ float lap_dir(const float* dp, const float* r, float beta, uint16_t info, int i,
                                         const Nb& nb, float& d_own) {
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; k++)
        if (info & (1u << cg_bit(k))) {
            const int j = i + nb.o[k];
            sum += dp[j] * beta + r[j];
        }
    d_own = dp[i] * beta + r[i];
    return sum - (float)((info >> 8) & 7) * d_own;
}
// L x in FP64 on row i
__device__ __forceinline__ double lap_d(const double* x, uint16_t info, int i, const Nb& nb) {
    double sum = 0.0;
#pragma unroll
    for (int k = 0; k < 6; k++)
        if (info & (1u << cg_bit(k))) sum += x[i + nb.o[k]];
    return sum - (double)((info >> 8) & 7) * x[i];
}
// L b in FP64 (p64 == b at the start)
__device__ __forceinline__ double lap_df(const float* x, uint16_t info, int i, const Nb& nb) {
    double sum = 0.0;
#pragma unroll
    for (int k = 0; k < 6; k++)
        if (info & (1u << cg_bit(k))) sum += (double)x[i + nb.o[k]];
    return sum - (double)((info >> 8) & 7) * (double)x[i];
}

// Iterate over this block's share of the active chunks: f(cell index) for every matrix row (rows only) or
// every in-range cell (all).
template <typename F>
__device__ __forceinline__ void for_rows(const SolverArgs& a, int m, F f) {
    const int per = (m + gridDim.x - 1) / gridDim.x;
    const int c0 = blockIdx.x * per, c1 = min(m, c0 + per);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = c0 + warp; c < c1; c += SOLVER_WARPS) {
        const int i = a.chunk_list[c] * 32 + lane;
        if (i < a.g.N) f(i);
    }
}

__global__ void __launch_bounds__(SOLVER_THREADS) k_solver(SolverArgs a) {
    DevCtl* ctl = a.ctl;
    __shared__ int s_scan[SOLVER_THREADS];
    // ---- phase 0: ordered compaction of the active chunks -------------------------------------------
    const int per_blk = (a.n_chunks + gridDim.x - 1) / gridDim.x;
    const int r0 = blockIdx.x * per_blk, r1 = min(a.n_chunks, r0 + per_blk);
    int cnt = 0;
    for (int c = r0 + threadIdx.x; c < r1; c += SOLVER_THREADS) cnt += a.chunk_flag[c] ? 1 : 0;
    s_scan[threadIdx.x] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < SOLVER_THREADS; k++) t += s_scan[k];
        a.block_count[blockIdx.x] = t;
    }
    if (!grid_barrier(ctl)) return;
    __shared__ int s_off, s_total;
    if (threadIdx.x == 0) {
        int off = 0, tot = 0;
        for (int b = 0; b < (int)gridDim.x; b++) {
            const int v = ((volatile int*)a.block_count)[b];
            if (b < (int)blockIdx.x) off += v;
            tot += v;
        }
        s_off = off;
        s_total = tot;
    }
    __syncthreads();
    {
        int base = s_off;
        for (int c0 = r0; c0 < r1; c0 += SOLVER_THREADS) {
            const int c = c0 + threadIdx.x;
            const int f = (c < r1 && a.chunk_flag[c]) ? 1 : 0;
            s_scan[threadIdx.x] = f;
            __syncthreads();
            // inclusive scan (Hillis-Steele) over the tile
            for (int o = 1; o < SOLVER_THREADS; o <<= 1) {
                const int v = (threadIdx.x >= o) ? s_scan[threadIdx.x - o] : 0;
                __syncthreads();
                s_scan[threadIdx.x] += v;
                __syncthreads();
            }
            if (f) a.chunk_list[base + s_scan[threadIdx.x] - 1] = c;
            const int tile = s_scan[SOLVER_THREADS - 1];
            __syncthreads();
            base += tile;
        }
    }
    const int M = s_total;
    if (!grid_barrier(ctl)) return;

    const Nb nb = cg_order(a.g);
    const float* __restrict__ b = a.b;
    const uint16_t* __restrict__ info = a.rowinfo;

    Reduction red{a.partials, 0};
    double u1, u2;

    // ---- Jacobi ---------------------------------------------------------------------------------------
    if (a.solver == EFS_SOLVER_JACOBI) {
        const int iters = a.max_steps / 2;
        const int jo[6] = {-1, 1, -a.g.W, a.g.W, -a.g.WH, a.g.WH};
        double rows = 0;
        for_rows(a, M, [&](int i) { if (info[i] & 0x8000u) rows += 1.0; });
        double nrows;
        if (!red.run(ctl, rows, 0.0, 0.0, nrows, u1, u2)) return;
        for (int it = 0; it < iters; it++) {
            const float* src = (it & 1) ? a.e : a.p;
            float* dst = (it & 1) ? a.p : a.e;
            for_rows(a, M, [&](int i) {
                const uint16_t f = info[i];
                if (!(f & 0x8000u)) return;
                float sum = 0.0f;
#pragma unroll
                for (int k = 0; k < 6; k++)
                    if (f & (1u << k)) sum += src[i + jo[k]];
                const int n = (f >> 8) & 7;
                dst[i] = n > 0 ? (sum - b[i]) / (float)n : 0.0f;
            });
            if (!grid_barrier(ctl)) return;
        }
        if (iters & 1) {
            for_rows(a, M, [&](int i) { if (info[i] & 0x8000u) a.p[i] = a.e[i]; });
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctl->converged = 1; ctl->iterations = iters; ctl->rr = 0; ctl->bb = 0; ctl->thr = 0;
            ctl->active_chunks = M; ctl->active_cells = (long long)nrows;
            ctl->total_iterations += iters; ctl->solves += 1;
            ctl->sum_iter_rows += (double)iters * nrows; ctl->sum_rows += nrows;
        }
        return;
    }

    // ---- CG ---------------------------------------------------------------------------------------------
    const bool mixed = a.cg_variant == EFS_CG_MIXED;
    float* __restrict__ r = a.r;
    float* __restrict__ e = a.e;
    double* __restrict__ p64 = a.p64;
    float* __restrict__ p = a.p;

    // initial residual r = b - L p0 with p0 = b (CGSolver.cpp:425-434); d = r
    double rr, bb, nrows;
    {
        double rr_p = 0, bb_p = 0, rows = 0;
        for_rows(a, M, [&](int i) {
            const float bi = b[i];
            bb_p += (double)bi * (double)bi;
            const uint16_t f = info[i];
            if (!(f & 0x8000u)) return;
            rows += 1.0;
            float ri;
            if (mixed) {
                p64[i] = (double)bi;
                e[i] = 0.f;
                ri = (float)((double)bi - lap_df(b, f, i, nb));
            } else {
                ri = bi - lap_f(b, f, i, nb);
            }
            r[i] = ri;
            a.d0[i] = ri;
            rr_p += (double)ri * (double)ri;
        });
        if (!red.run(ctl, rr_p, bb_p, rows, rr, bb, nrows)) return;
    }
    float thr_f;
    if (a.tol_rel > 0) {
        thr_f = (float)((double)a.tol_rel * (double)a.tol_rel * bb);
        if (!(thr_f > 0)) thr_f = FLT_MIN;
    } else {
        thr_f = a.solver_threshold;
    }
    const double thr = (double)thr_f;

    // residual recomputation (CGSolver.cpp:447-451): fold e into p64 and r = b - L p64 in FP64 (mixed), or
    // r = b - L p in FP32 (reference)
    auto replace = [&](double& rr_out) -> bool {
        if (mixed) {
            for_rows(a, M, [&](int i) {
                if (!(info[i] & 0x8000u)) return;
                p64[i] += (double)e[i];
                e[i] = 0.f;
            });
        }
        if (!grid_barrier(ctl)) return false;
        double rp = 0;
        for_rows(a, M, [&](int i) {
            const uint16_t f = info[i];
            if (!(f & 0x8000u)) return;
            const float ri = mixed ? (float)((double)b[i] - lap_d(p64, f, i, nb)) : b[i] - lap_f(p, f, i, nb);
            r[i] = ri;
            rp += (double)ri * (double)ri;
        });
        return red.run(ctl, rp, 0.0, 0.0, rr_out, u1, u2);
    };

    int conv = rr < thr;
    int iters = 0;
    float beta = 0.f;
    if (!conv) {
        int it;
        for (it = 0; it < a.max_steps; it++) {
            float* dcur = (it & 1) ? a.d1 : a.d0;
            const float* dprev = (it & 1) ? a.d0 : a.d1;
            // A: d = beta d + r (it > 0; CGSolver.cpp:458-460), t = L d, d.t
            double dt_p = 0;
            for_rows(a, M, [&](int i) {
                const uint16_t f = info[i];
                if (!(f & 0x8000u)) return;
                float di, t;
                if (it == 0) { di = dcur[i]; t = lap_f(dcur, f, i, nb); }
                else { t = lap_dir(dprev, r, beta, f, i, nb, di); dcur[i] = di; }
                dt_p += (double)di * (double)t;
            });
            double dt;
            if (!red.run(ctl, dt_p, 0.0, 0.0, dt, u1, u2)) return;
            const float alpha = (float)(rr / dt);
            // B: p (or e) += alpha d; r -= alpha L d, or the true residual every 64 iterations (:442-451)
            const double old = rr;
            bool replaced = false;
            if (it & 0x3F) {
                double rp = 0;
                for_rows(a, M, [&](int i) {
                    const uint16_t f = info[i];
                    if (!(f & 0x8000u)) return;
                    const float di = dcur[i];
                    if (mixed) e[i] += alpha * di; else p[i] += alpha * di;
                    const float t = lap_f(dcur, f, i, nb);
                    const float ri = r[i] + (-alpha) * t;
                    r[i] = ri;
                    rp += (double)ri * (double)ri;
                });
                if (!red.run(ctl, rp, 0.0, 0.0, rr, u1, u2)) return;
            } else {
                for_rows(a, M, [&](int i) {
                    if (!(info[i] & 0x8000u)) return;
                    if (mixed) e[i] += alpha * dcur[i]; else p[i] += alpha * dcur[i];
                });
                if (!replace(rr)) return;
                replaced = true;
            }
            // C: stop test (:453-456); the mixed variant confirms it on a recomputed residual
            if (rr < thr) {
                if (mixed && !replaced) {
                    if (!replace(rr)) return;
                }
                if (rr < thr) { conv = 1; break; }
            }
            beta = (float)(rr / old);
        }
        iters = it + 1;
    }
    if (mixed) {
        for_rows(a, M, [&](int i) {
            if (!(info[i] & 0x8000u)) return;
            p[i] = (float)(p64[i] + (double)e[i]);
        });
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->converged = conv;
        ctl->iterations = iters;
        ctl->rr = rr;
        ctl->bb = bb;
        ctl->thr = thr;
        ctl->active_chunks = M;
        ctl->active_cells = (long long)nrows;
        ctl->total_iterations += iters;
        ctl->solves += 1;
        ctl->sum_iter_rows += (double)iters * nrows;
        ctl->sum_rows += nrows;
    }
}

}  // namespace

cudaError_t solver_configure(efs_ctx* c) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_solver, SOLVER_THREADS, 0);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorLaunchOutOfResources;
    const int n_chunks = (c->g.N + 31) / 32;
    int blocks = std::min(occ, 2) * c->sm_count;
    // small grids: about four chunks per warp so barrier cost stays proportionate
    const int want = (n_chunks + SOLVER_WARPS * 4 - 1) / (SOLVER_WARPS * 4);
    blocks = std::max(1, std::min(blocks, want));
    c->solver_blocks = blocks;
    c->solver_threads = SOLVER_THREADS;
    return cudaSuccess;
}

cudaError_t launch_solver(efs_ctx* c) {
    SolverArgs a;
    a.g = c->g;
    a.dim = c->dim;
    a.solver = c->prm.solver;
    a.cg_variant = c->prm.cg_variant;
    a.max_steps = c->prm.max_steps;
    a.tol_rel = c->prm.tol_rel;
    a.solver_threshold = c->prm.solver_threshold;
    a.n_chunks = (c->g.N + 31) / 32;
    a.b = c->div;
    a.rowinfo = c->rowinfo;
    a.chunk_flag = c->chunk_flag;
    a.chunk_list = c->chunk_list;
    a.block_count = c->block_count;
    a.p = c->p;
    a.p64 = c->p64;
    a.e = c->e;
    a.r = c->r;
    a.d0 = c->d0;
    a.d1 = c->d1;
    a.partials = c->partials;
    a.ctl = c->ctl;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c->solver_blocks);
    cfg.blockDim = dim3(SOLVER_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = c->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // a fresh barrier for this launch (a previous launch may have aborted mid-barrier)
    cudaError_t e = cudaMemsetAsync(c->ctl, 0, 2 * sizeof(int), c->stream);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, k_solver, a);
}

}  // namespace efs
