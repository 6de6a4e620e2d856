// efs_mlfcg.cu — flexible preconditioned CG (EFS_SOLVER_FCG_UNET) with a multilevel preconditioner whose
// coarsest level is solved by the learned U-Net (efs_unet.cu), run entirely on the device.
//
// No counterpart in the reference: its solvers are CGSolverCPU3D / JacobiSolverCPU3D
// (src/simulation/solver/CGSolver.cpp:416-497, JacobiSolver.cpp:154-212).  FCG solves the same matrix L p = b
// (rows: liquid, non-solid cells, as built by k_solver_prep) to the same stop rule.
//
// Hierarchy.  Level 0 is L itself, read from rowinfo (bit 15 row, bits 0-5 the liquid neighbours in the
// order -x, +x, -y, +y, -z, +z, bits 8-10 the neighbour count: row i of L is sum of its liquid neighbours
// minus count x_i).  Level l+1 merges 2x2x2 cells of level l (the last cell of an odd side alone); its matrix
// is P^T A P for the piecewise-constant prolongation P, again a 7-point stencil: per coarse cell a diagonal
// (the children's diagonals plus the couplings between children) and six face weights (the couplings that
// cross that face, at most 4^l), stored as one float and six bytes.
//
// V-cycle M(r) (one preconditioner application), at each level above the bottom: two damped Jacobi sweeps
// (weight 0.8) from zero, the residual restricted (summed over the merged cells), the next level's
// correction, prolongation (added to the merged cells), two more sweeps.  At the bottom level: the U-Net's
// output e scaled by the line search (e.r)/(e.Ae) on that level, or (for comparison without the network)
// 20 Jacobi sweeps.
//
// FCG(1) (Notay 2000, truncation 1): beta = -(z.q_old)/(d_old.q_old), d = z + beta d, q = A d,
// alpha = (r.z)/(d.q), x += alpha d, r -= alpha q.  x is FP64 and starts at 0; the true residual b - A x is
// recomputed in FP64 every 32 iterations and before stopping.  Every scalar lives in device memory: the
// iteration is the body of a CUDA graph WHILE node whose condition the convergence test sets, with the
// residual recomputation in an IF node inside it; after the loop an IF node hands a stalled solve (residual
// not halved over 10 iterations, or d.Ad >= 0) to the persistent CG kernel on the residual system.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "efs_internal.h"
#include "efs_pair.cuh"

namespace efs {

namespace {

constexpr float kOmega = 6.0f / 7.0f;  // Jacobi damping (the smoothing optimum of the 3D 7-point stencil)
constexpr int kBottomJacobi = 20;     // sweeps of the bottom solve without the network
constexpr int kThreads = 256;
// Most blocks of a level kernel (threads loop over the rest; the partials buffer holds one per block): 8 per SM
// of GB300's 152.  A 4096-block launch of these short kernels spends microseconds distributing blocks (a trivial
// 4096-block kernel takes 4.9 µs); at 1216 the preconditioner took 280 instead of 297 µs and the 256^3 solve
// 12.8 instead of 13.7 ms (608, 912 and 1520 blocks were slower or equal).
constexpr int kGrid = 1216;

// Arrival counters of the last-block reductions: a block counts itself in group blockIdx.x % kArriveGroups, and
// the last block of each group in the top counter.  One 128-byte line per counter: same-address atomics from
// thousands of blocks queue at one L2 slice (4096 arrivals cost tens of microseconds), 32 lines do not.
constexpr int kArriveGroups = 32;
constexpr int kArriveStride = 32;     // unsigned per counter line

// device scalars of one FCG solve
struct FcgDev {
    double rr, rz, dq, zq, bb, thr, alpha, beta, rr_window, rows;
    double ls_alpha;                  // bottom-level line search factor of the current V-cycle (1 without the network)
    float alpha_hi, alpha_lo, beta_f; // alpha as a float pair and beta in float, for the level-0 kernels
    float alpha_prev_hi, alpha_prev_lo;   // the previous iteration's alpha (x may still lack its step)
    // The two direction buffers (d0, d1) alternate: the direction of iteration k is written to buffer par ^ 1 and
    // becomes buffer par when the iteration's last finisher toggles par.  x takes its steps two iterations at a
    // time: xlag = 1 while it lacks alpha d of the direction in buffer par.
    int par, xlag;
    int it, conv, stall, verify, fallback, nchunks;
    int ncchunks;                     // level 1's 32-cell chunks that hold a row (the restriction's list)
    // arrival counters (groups, then the top), back to 0 after each reduction
    alignas(128) unsigned count[(kArriveGroups + 1) * kArriveStride];
};

inline unsigned blocks_for(long long n) { return (unsigned)std::max(1LL, (n + kThreads - 1) / kThreads); }
// reduction kernels: at most kGrid blocks, looping over the rest
inline unsigned grid_for(long long n) { return (unsigned)std::min<long long>(kGrid, blocks_for(n)); }

// ---- matrix rows at a level -----------------------------------------------------------------------------------
template <bool FINE>
__device__ __forceinline__ bool lrow(const LvView& L, long long i, float& dg, float (&w)[6]) {
    const uint16_t f = L.info[i];
    if (!(f & 0x8000u)) return false;
    if (FINE) {
        dg = -(float)((f >> 8) & 7);
#pragma unroll
        for (int k = 0; k < 6; k++) w[k] = ((f >> k) & 1u) ? 1.f : 0.f;
    } else {
        dg = L.diag[i];
#pragma unroll
        for (int k = 0; k < 6; k++) w[k] = (float)L.w[k * L.V + i];
    }
    return true;
}
__device__ __forceinline__ long long noff(const LvView& L, int k) {
    const long long W = L.W, WH = (long long)L.W * L.H;
    return k == 0 ? -1 : k == 1 ? 1 : k == 2 ? -W : k == 3 ? W : k == 4 ? -WH : WH;
}
// (A x)_i for a row (neighbours are read only where the weight is non-zero, i.e. inside the grid)
template <typename T>
__device__ __forceinline__ T lapply(const LvView& L, long long i, const T* x, float dg, const float (&w)[6]) {
    T s = (T)dg * x[i];
#pragma unroll
    for (int k = 0; k < 6; k++)
        if (w[k] != 0.f) s += (T)w[k] * x[i + noff(L, k)];
    return s;
}

// FCG's x as a pair of floats (efs_pair.cuh), updated on the FP32 pipe: GB300's FP64 rate made the FP64 update
// of every row a sixth of the vector update's time.
// b_i - (A x)_i for x held as float pairs, on a level-0 row with flags f (lapply's neighbour order), in pair
// arithmetic, rounded to float
__device__ __forceinline__ float resid_pair(const LvView& L, long long i, const float2* x, float b, unsigned f) {
    float2 sum = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 6; k++)
        if ((f >> k) & 1u) sum = df_add(sum, x[i + noff(L, k)]);
    const float2 lap = df_add(sum, df_neg(df_mul_k(x[i], (float)((f >> 8) & 7))));
    const float2 t = df_add_f(df_neg(lap), b);
    return __fadd_rn(t.x, t.y);
}
// resid_pair of x + (ah + al) d, the pending step formed at each of the seven points as the vector update forms it
__device__ __forceinline__ float resid_pair_step(const LvView& L, long long i, const float2* x, const float* d, float ah,
                                                 float al, float b, unsigned f) {
    float2 sum = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 6; k++)
        if ((f >> k) & 1u) {
            const long long j = i + noff(L, k);
            sum = df_add(sum, df_axpy(x[j], ah, al, d[j]));
        }
    const float2 lap = df_add(sum, df_neg(df_mul_k(df_axpy(x[i], ah, al, d[i]), (float)((f >> 8) & 7))));
    const float2 t = df_add_f(df_neg(lap), b);
    return __fadd_rn(t.x, t.y);
}
// the start of an iteration's vector step: the old alpha becomes the previous one
__device__ __forceinline__ void shift_alpha(FcgDev* s) {
    s->alpha_prev_hi = s->alpha_hi;
    s->alpha_prev_lo = s->alpha_lo;
}
// alpha / beta for the float kernels
__device__ __forceinline__ void set_alpha(FcgDev* s, double a) {
    s->alpha = a;
    s->alpha_hi = (float)a;
    s->alpha_lo = (float)(a - (double)s->alpha_hi);
}
__device__ __forceinline__ void set_beta(FcgDev* s, double b) {
    s->beta = b;
    s->beta_f = (float)b;
}

// The cells a level kernel visits: at level 0 (and at level 1 when its list is built) the 32-cell chunks that hold a
// matrix row (the list built at the start of the solve, warp-aligned, *count of them), at coarser levels every
// cell.  item -> cell, or -1 past the end.  Only rows are read at a level, so unvisited cells are never needed.
struct Walk {
    const int* chunks;
    const int* count;
    long long V;
    __device__ __forceinline__ long long items() const { return chunks ? (long long)*count * 32 : V; }
    __device__ __forceinline__ long long cell(long long t) const {
        if (!chunks) return t;
        const long long i = (long long)chunks[t >> 5] * 32 + (t & 31);
        return i < V ? i : -1;
    }
};
#define WALK(wk, t, i)                                                                                        \
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x, n_items_ = (wk).items(); t < n_items_; \
         t += (long long)gridDim.x * blockDim.x)                                                              \
        if (const long long i = (wk).cell(t); i >= 0)

// ---- reductions ------------------------------------------------------------------------------------------------
// Block partials of the NV values v into part[3 * blockIdx.x + j]: the warp sums and the block's eight warp sums
// (thread 0, warp order) in the threads' accumulator type T (FP32 for the level-0 kernels, whose threads sum a
// few cells each).  GB300's FP64 pipe runs at a small fraction of its FP32 rate: a shuffle tree in FP64 over every
// warp of a 4096-block launch cost more than the sweep it finished.
template <int NV, typename T>
__device__ __forceinline__ void block_partials(T (&v)[NV], double* part) {
    __shared__ double sh[NV][kThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int j = 0; j < NV; j++) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < NV; j++) sh[j][warp] = (double)v[j];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < NV; j++) {
            T t = 0;
            for (int k = 0; k < kThreads / 32; k++) t += (T)sh[j][k];
            part[3 * blockIdx.x + j] = (double)t;
        }
}
// Every block stores its partials; the block that arrives last sums them all in a fixed order (lane-strided over
// the blocks, then a fixed shuffle tree) and returns true on its thread 0, with the NV totals in tot (the rest 0).
template <int NV, typename T>
__device__ bool reduce_last(T (&v)[NV], double* part, unsigned* counter, double (&tot)[3]) {
    block_partials<NV>(v, part);
    __shared__ unsigned s_last;
    const unsigned ngroups = min(gridDim.x, (unsigned)kArriveGroups);
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned g = blockIdx.x % kArriveGroups;
        const unsigned gsize = (gridDim.x - g + kArriveGroups - 1) / kArriveGroups;
        unsigned last = 0u;
        if (atomicAdd(counter + g * kArriveStride, 1u) == gsize - 1) {
            __threadfence();
            last = (atomicAdd(counter + kArriveGroups * kArriveStride, 1u) == ngroups - 1) ? 1u : 0u;
        }
        s_last = last;
    }
    __syncthreads();
    if (!s_last || threadIdx.x >= 32) return false;
    __threadfence();
    // four independent chains per lane (FP64 adds have a long latency), combined in a fixed order
    double acc[NV][4];
#pragma unroll
    for (int j = 0; j < NV; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0;
    for (unsigned k = threadIdx.x; k < gridDim.x; k += 128) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const unsigned kk = k + 32u * u;
            if (kk < gridDim.x)
#pragma unroll
                for (int j = 0; j < NV; j++) acc[j][u] += __ldcg(part + 3 * kk + j);
        }
    }
    double t[NV];
#pragma unroll
    for (int j = 0; j < NV; j++) t[j] = (acc[j][0] + acc[j][1]) + (acc[j][2] + acc[j][3]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int j = 0; j < NV; j++) t[j] += __shfl_down_sync(0xffffffffu, t[j], o);
    // every block has arrived: the counters go back to 0 for the next reduction
    if (threadIdx.x < ngroups) counter[threadIdx.x * kArriveStride] = 0u;
    if (threadIdx.x == 0) counter[kArriveGroups * kArriveStride] = 0u;
    if (threadIdx.x != 0) return false;
    tot[0] = tot[1] = tot[2] = 0.0;
#pragma unroll
    for (int j = 0; j < NV; j++) tot[j] = t[j];
    return true;
}

// The level-0 reduction kernels (thousands of blocks) only store their FP32 block partials; one block then sums
// them: thread t adds blocks t, t + 256, ... with a compensated FP32 sum (Kahan), the 256 results go through a
// fixed FP64 tree.  Blocks that waited for their own fence and arrival atomic before exiting had cost about
// 20 us per 4096-block launch.
constexpr int kFinishPer = (kGrid + kThreads - 1) / kThreads;   // partials per thread of a finisher block
template <int NV>
__device__ bool finish_partials(const double* __restrict__ part, int n, double (&tot)[NV]) {
    __shared__ double sh[NV][kThreads / 32];
    double a[NV];
#pragma unroll
    for (int j = 0; j < NV; j++) {
        float v[kFinishPer];
#pragma unroll
        for (int u = 0; u < kFinishPer; u++) {      // all loads first: one round trip
            const int k = (int)threadIdx.x + u * kThreads;
            v[u] = k < n ? (float)__ldcg(part + 3 * k + j) : 0.f;
        }
        float sum = 0.f, comp = 0.f;
#pragma unroll
        for (int u = 0; u < kFinishPer; u++) {
            const float y = v[u] - comp;
            const float t = sum + y;
            comp = (t - sum) - y;
            sum = t;
        }
        a[j] = (double)sum;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int j = 0; j < NV; j++) a[j] += __shfl_down_sync(0xffffffffu, a[j], o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < NV; j++) sh[j][warp] = a[j];
    __syncthreads();
    if (threadIdx.x != 0) return false;
#pragma unroll
    for (int j = 0; j < NV; j++) {
        double t = 0;
        for (int k = 0; k < kThreads / 32; k++) t += sh[j][k];
        tot[j] = t;
    }
    return true;
}

// ---- the level-0 chunk list (ordered compaction of the chunks that hold a row) ---------------------------------
__device__ __forceinline__ bool chunk_has_row(const uint16_t* info, long long N, long long ch) {
    const long long i0 = ch * 32;
    if (i0 + 32 <= N) {
        const uint4* q = reinterpret_cast<const uint4*>(info + i0);
        unsigned any = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint4 v = q[k];
            any |= (v.x | v.y | v.z | v.w);
        }
        return (any & 0x80008000u) != 0;
    }
    for (long long i = i0; i < N; i++)
        if (info[i] & 0x8000u) return true;
    return false;
}
__global__ void k_chunks_count(const uint16_t* __restrict__ info, long long N, long long nch, int* __restrict__ bcount) {
    const long long ch = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int f = (ch < nch) && chunk_has_row(info, N, ch);
    const int n = __syncthreads_count(f);
    if (threadIdx.x == 0) bcount[blockIdx.x] = n;
}
// exclusive scan of the block counts (one block of 1024 threads), total into *total
__global__ void k_chunks_scan(int* __restrict__ bcount, int nb, int* __restrict__ total) {
    __shared__ int warp_tot[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < nb; base += 1024) {
        const int k = base + threadIdx.x;
        const int v = k < nb ? bcount[k] : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_tot[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const int wv = warp_tot[lane];
            int wi = wv;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += y;
            }
            warp_tot[lane] = wi - wv;
        }
        __syncthreads();
        const int excl = carry + warp_tot[warp] + incl - v;
        if (k < nb) bcount[k] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}
__global__ void k_chunks_write(const uint16_t* __restrict__ info, long long N, long long nch, const int* __restrict__ boff,
                               int* __restrict__ chunks) {
    __shared__ int wcount[kThreads / 32];
    const long long ch = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool f = (ch < nch) && chunk_has_row(info, N, ch);
    const unsigned m = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wcount[warp] = __popc(m);
    __syncthreads();
    int off = boff[blockIdx.x];
    for (int k = 0; k < warp; k++) off += wcount[k];
    if (f) chunks[off + __popc(m & ((1u << lane) - 1u))] = (int)ch;
}

// ---- hierarchy -------------------------------------------------------------------------------------------------
struct LvOut {
    int W, H, D;
    long long V;
    uint16_t* info;
    uint8_t* w;
    float* diag;
    float* wd;
};
template <bool FINE>
__global__ void k_ml_build(LvView src, LvOut dst) {
    const long long C = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (C >= dst.V) return;
    const int c32 = (int)C;           // grids stay below 2^31 cells
    const int X = c32 % dst.W, Y = (c32 / dst.W) % dst.H, Z = c32 / (dst.W * dst.H);
    bool row = false;
    float dg = 0.f, w[6] = {0, 0, 0, 0, 0, 0};
    for (int c8 = 0; c8 < 8; c8++) {
        const int dx = c8 & 1, dy = (c8 >> 1) & 1, dz = c8 >> 2;
        const int x = 2 * X + dx, y = 2 * Y + dy, z = 2 * Z + dz;
        if (x >= src.W || y >= src.H || z >= src.D) continue;
        const long long i = ((long long)z * src.H + y) * src.W + x;
        float cd, cw[6];
        if (!lrow<FINE>(src, i, cd, cw)) continue;
        row = true;
        dg += cd;
        // 1 where the neighbour in direction k lies in the same merged cell
        const int same[6] = {dx, 1 - dx, dy, 1 - dy, dz, 1 - dz};
#pragma unroll
        for (int k = 0; k < 6; k++) {
            if (cw[k] == 0.f) continue;
            if (same[k]) dg += cw[k]; else w[k] += cw[k];
        }
    }
    dst.info[C] = row ? (uint16_t)0x8000u : (uint16_t)0;
    dst.diag[C] = row ? dg : 0.f;
    dst.wd[C] = (row && dg != 0.f) ? kOmega / dg : 0.f;
#pragma unroll
    for (int k = 0; k < 6; k++) dst.w[k * dst.V + C] = row ? (uint8_t)w[k] : (uint8_t)0;
}

// ---- level operators ------------------------------------------------------------------------------------------
// zout = zin + w (r - A zin) / diag on rows (zin null: zout = w r / diag), 0 on the other visited cells.
// DOTS (level 0, the last sweep of the V-cycle): also the partials of z.q and r.z, and in the last block
// beta = -(z.q) / (d.q) of FCG(1) (0 in the first iteration) and r.z.
template <bool FINE, bool DOTS>
__global__ void k_ml_smooth(LvView L, Walk wk, const float* __restrict__ r, const float* __restrict__ zin,
                            float* __restrict__ zout, float omega, const float* __restrict__ q, FcgDev* s,
                            double* __restrict__ part) {
    float zq = 0.f, rz = 0.f;
    WALK(wk, t, i) {
        float dg, w[6];
        float zi = 0.f;
        if (lrow<FINE>(L, i, dg, w) && dg != 0.f) {
            if (FINE) zi = zin ? zin[i] + omega * (r[i] - lapply<float>(L, i, zin, dg, w)) / dg : omega * r[i] / dg;
            else zi = zin ? zin[i] + (r[i] - lapply<float>(L, i, zin, dg, w)) * L.wd[i] : r[i] * L.wd[i];
        }
        zout[i] = zi;
        if (DOTS) {
            zq += zi * q[i];
            rz += zi * r[i];
        }
    }
    if (DOTS) {
        double tot[3];
        float v[2] = {zq, rz};
        if (reduce_last(v, part, s->count, tot)) {
            s->zq = tot[0];
            s->rz = tot[1];
            double beta = 0.0;
            if (s->it > 0 && s->dq != 0.0) beta = -tot[0] / s->dq;
            set_beta(s, isfinite(beta) ? beta : 0.0);
        }
    }
}
// The first damped Jacobi sweep from zero is pointwise (z1 = w r / diag on the rows), so the two pre-smoothing
// sweeps are one pass: zout = z1 + w (r - A z1) / diag, with z1 formed at the row and at its neighbours exactly as
// the first sweep would store it (a neighbour with a non-zero weight is a row).
template <bool FINE>
__device__ __forceinline__ float z1_at(const LvView& L, long long j, const float* __restrict__ r, float omega) {
    if (!FINE) return r[j] * L.wd[j];
    const float dj = -(float)((L.info[j] >> 8) & 7);
    return dj != 0.f ? omega * r[j] / dj : 0.f;
}
template <bool FINE>
__global__ void k_ml_smooth2(LvView L, Walk wk, const float* __restrict__ r, float* __restrict__ zout, float omega) {
    WALK(wk, t, i) {
        float dg, w[6];
        float zi = 0.f;
        if (lrow<FINE>(L, i, dg, w) && dg != 0.f) {
            const float z1 = z1_at<FINE>(L, i, r, omega);
            float s = dg * z1;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if (w[k] != 0.f) s += w[k] * z1_at<FINE>(L, i + noff(L, k), r, omega);
            zi = FINE ? z1 + omega * (r[i] - s) / dg : z1 + (r[i] - s) * L.wd[i];
        }
        zout[i] = zi;
    }
}
// Restriction rc[C] = sum over the merged rows i of C of (r - A z)_i, in two passes whose threads each make one
// load round trip (a thread gathering its eight children's stencils in sequence made the coarse levels'
// restriction a chain of dependent loads): res = r - A z on the level's rows (visited cells), then per coarse
// row the sum of its row children's res, children in the order x fastest, then y, then z.  scal (non-null: the
// level below is the network's): the sum of rc^2 over the coarse rows, their count and 1 / rms into scal[0..2].
template <bool FINE>
__global__ void k_ml_resid(LvView L, Walk wk, const float* __restrict__ r, const float* __restrict__ z,
                           float* __restrict__ res) {
    WALK(wk, t, i) {
        float dg, w[6];
        res[i] = lrow<FINE>(L, i, dg, w) ? r[i] - lapply<float>(L, i, z, dg, w) : 0.f;
    }
}
template <bool FINE>
__global__ void k_ml_sum8(LvView F, const float* __restrict__ res, LvView Cv, float* __restrict__ rc,
                          double* __restrict__ scal, FcgDev* s, double* __restrict__ part) {
    double ss = 0, cnt = 0;
    for (long long C = blockIdx.x * (long long)blockDim.x + threadIdx.x; C < Cv.V; C += (long long)gridDim.x * blockDim.x) {
        if (!(Cv.info[C] & 0x8000u)) { rc[C] = 0.f; continue; }
        const int c32 = (int)C;
        const int X = c32 % Cv.W, Y = (c32 / Cv.W) % Cv.H, Z = c32 / (Cv.W * Cv.H);
        long long ch[8];
        bool ok[8];
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++) {
            const int x = 2 * X + (c8 & 1), y = 2 * Y + ((c8 >> 1) & 1), zz = 2 * Z + (c8 >> 2);
            ok[c8] = x < F.W && y < F.H && zz < F.D;
            ch[c8] = ok[c8] ? ((long long)zz * F.H + y) * F.W + x : 0;
        }
        uint16_t f[8];
        float v[8];
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++) { f[c8] = F.info[ch[c8]]; v[c8] = res[ch[c8]]; }
        float acc = 0.f;
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++)
            if (ok[c8] && (f[c8] & 0x8000u)) acc += v[c8];
        rc[C] = acc;
        if (scal) {
            ss += (double)acc * acc;
            cnt += 1.0;
        }
    }
    if (scal) {
        double tot[3], v2[2] = {ss, cnt};
        if (reduce_last(v2, part, s->count, tot)) {
            scal[0] = tot[0];
            scal[1] = tot[1];
            scal[2] = (tot[0] > 0 && tot[1] > 0) ? 1.0 / sqrt(tot[0] / tot[1]) : 1.0;
        }
    }
}
// The first sweep after the coarse correction, with the prolongation folded in: with zp = z + a ec(parent) on
// the rows (a = *alpha, or 1), tout = zp + w (r - A zp) / diag.
template <bool FINE>
__global__ void k_ml_prolong_smooth(LvView L, Walk wk, const float* __restrict__ r, const float* __restrict__ z,
                                    const float* __restrict__ ec, LvView Cv, const double* __restrict__ alpha,
                                    float* __restrict__ tout, float omega) {
    const float a = alpha ? (float)*alpha : 1.f;
    const int W = L.W, H = L.H;
    WALK(wk, t, i) {
        float dg, w[6];
        if (!lrow<FINE>(L, i, dg, w) || dg == 0.f) { tout[i] = 0.f; continue; }
        const int i32 = (int)i;
        const int x = i32 % W, y = (i32 / W) % H, zz = i32 / (W * H);
        auto parent = [&](int px, int py, int pz) {
            return ec[((long long)(pz >> 1) * Cv.H + (py >> 1)) * Cv.W + (px >> 1)];
        };
        const float zi = z[i] + a * parent(x, y, zz);
        float s = dg * zi;
        if (w[0] != 0.f) s += w[0] * (z[i - 1] + a * parent(x - 1, y, zz));
        if (w[1] != 0.f) s += w[1] * (z[i + 1] + a * parent(x + 1, y, zz));
        if (w[2] != 0.f) s += w[2] * (z[i - W] + a * parent(x, y - 1, zz));
        if (w[3] != 0.f) s += w[3] * (z[i + W] + a * parent(x, y + 1, zz));
        const long long WH = (long long)W * H;
        if (w[4] != 0.f) s += w[4] * (z[i - WH] + a * parent(x, y, zz - 1));
        if (w[5] != 0.f) s += w[5] * (z[i + WH] + a * parent(x, y, zz + 1));
        tout[i] = FINE ? zi + omega * (r[i] - s) / dg : zi + (r[i] - s) * L.wd[i];
    }
}
template <bool FINE>
__global__ void k_ml_matvec(LvView L, const float* __restrict__ x, float* __restrict__ y) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= L.V) return;
    float dg, w[6];
    y[i] = lrow<FINE>(L, i, dg, w) ? lapply<float>(L, i, x, dg, w) : 0.f;
}
// bottom line search for the network's output e (read on the rows): a = (e.r) / (e.Ae) into s->ls_alpha
template <bool FINE>
__global__ void k_ml_line_search(LvView L, Walk wk, const float* __restrict__ e, const float* __restrict__ r, FcgDev* s,
                                 double* __restrict__ part) {
    float er = 0.f, eae = 0.f;
    WALK(wk, t, i) {
        float dg, w[6];
        if (!lrow<FINE>(L, i, dg, w)) continue;
        const float ei = e[i];
        er += ei * r[i];
        eae += ei * lapply<float>(L, i, e, dg, w);
    }
    double tot[3];
    float v[2] = {er, eae};
    if (reduce_last(v, part, s->count, tot)) {
        const double a = (tot[1] != 0.0) ? tot[0] / tot[1] : 0.0;
        s->ls_alpha = isfinite(a) ? a : 0.0;
    }
}
// level 0 is the bottom: z = a e on the rows, with FCG's dots and beta as in the last sweep (k_ml_smooth DOTS)
__global__ void k_take_dots(LvView F, Walk wk, const float* __restrict__ e, const float* __restrict__ q,
                            const float* __restrict__ r, float* __restrict__ z, FcgDev* s, double* __restrict__ part) {
    const double a = s->ls_alpha;
    float zq = 0.f, rz = 0.f;
    WALK(wk, t, i) {
        const float zi = (F.info[i] & 0x8000u) ? (float)(a * (double)e[i]) : 0.f;
        z[i] = zi;
        zq += zi * q[i];
        rz += zi * r[i];
    }
    double tot[3];
    float v[2] = {zq, rz};
    if (reduce_last(v, part, s->count, tot)) {
        s->zq = tot[0];
        s->rz = tot[1];
        double beta = 0.0;
        if (s->it > 0 && s->dq != 0.0) beta = -tot[0] / s->dq;
        set_beta(s, isfinite(beta) ? beta : 0.0);
    }
}

// ---- level 0 with 128-bit accesses ----------------------------------------------------------------------------
// When the grid's width is a multiple of 32, every 32-cell chunk is one piece of one grid row, and the chunks in
// the list lie inside the border (rows are interior cells), so for every 4-cell group of a listed chunk the
// loads at +-1, +-W and +-W*H stay inside the grid.  Thread t of a level-0 kernel takes the 4-cell group
// t & 7 of listed chunk t >> 3: a warp covers four chunks, each vector load is 16 bytes a lane.
struct QWalk {
    const int* chunks;
    const FcgDev* s;
};
#define QWALK(qw, i)                                                                                            \
    for (long long t_ = blockIdx.x * (long long)blockDim.x + threadIdx.x, n_ = (long long)(qw).s->nchunks * 8; \
         t_ < n_; t_ += (long long)gridDim.x * blockDim.x)                                                      \
        if (const int i = (qw).chunks[t_ >> 3] * 32 + ((int)t_ & 7) * 4; true)

__device__ __forceinline__ void ld4(const float* __restrict__ p, int i, float (&v)[4]) {
    const float4 a = *reinterpret_cast<const float4*>(p + i);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void st4(float* __restrict__ p, int i, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p + i) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void info4(const uint16_t* __restrict__ info, int i, unsigned (&f)[4]) {
    const uint2 u = *reinterpret_cast<const uint2*>(info + i);
    f[0] = u.x & 0xFFFFu; f[1] = u.x >> 16; f[2] = u.y & 0xFFFFu; f[3] = u.y >> 16;
}
// x at the group's 4 cells (c) and at their six neighbours (nb[k][n], n = -x, +x, -y, +y, -z, +z)
__device__ __forceinline__ void stencil4(const float* __restrict__ x, int i, int W, int WH, float (&c)[4],
                                         float (&nb)[4][6]) {
    float ym[4], yp[4], zm[4], zp[4];
    ld4(x, i, c);
    ld4(x, i - W, ym);
    ld4(x, i + W, yp);
    ld4(x, i - WH, zm);
    ld4(x, i + WH, zp);
    const float left = x[i - 1], right = x[i + 4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        nb[k][0] = k == 0 ? left : c[k - 1 < 0 ? 0 : k - 1];
        nb[k][1] = k == 3 ? right : c[k + 1 > 3 ? 3 : k + 1];
        nb[k][2] = ym[k]; nb[k][3] = yp[k]; nb[k][4] = zm[k]; nb[k][5] = zp[k];
    }
}
__device__ __forceinline__ float lap4(unsigned f, float c, const float (&nb)[6]) {
    float s = -(float)((f >> 8) & 7) * c;
#pragma unroll
    for (int n = 0; n < 6; n++)
        if (f & (1u << n)) s += nb[n];
    return s;
}

// The level-0 diagonal is -(count of non-solid neighbours), count 0..6: the sweeps multiply by omega / diagonal,
// taken per block from a table of the eight counts (0 for count 0 and for the unused 7), instead of dividing.
__device__ __forceinline__ void init_wod(float* wod) {
    if (threadIdx.x < 8) {
        const unsigned k = threadIdx.x;
        wod[k] = (k == 0 || k == 7) ? 0.f : kOmega / -(float)k;
    }
    __syncthreads();
}
__device__ __forceinline__ unsigned q_count(unsigned f) { return (f >> 8) & 7u; }
__device__ __forceinline__ bool q_live(unsigned f) { return (f & 0x8000u) && q_count(f) != 0; }

// k_ml_smooth at level 0 (damping omega = kOmega)
// (the level-0 kernels sum their few cells per thread in FP32, and the block and grid sums in FP64: GB300's FP64
// pipe is a small fraction of its FP32 one)
template <bool DOTS>
__global__ void k_q_smooth(QWalk qw, const uint16_t* __restrict__ info, int W, int WH, const float* __restrict__ r,
                           const float* __restrict__ zin, float* __restrict__ zout, const float* __restrict__ q,
                           double* __restrict__ part) {
    __shared__ float wod[8];
    init_wod(wod);
    float zq = 0.f, rz = 0.f;
    QWALK(qw, i) {
        unsigned f[4];
        float rv[4], out[4];
        info4(info, i, f);
        ld4(r, i, rv);
        if (zin) {
            float c[4], nb[4][6];
            stencil4(zin, i, W, WH, c, nb);
#pragma unroll
            for (int k = 0; k < 4; k++)
                out[k] = q_live(f[k]) ? c[k] + (rv[k] - lap4(f[k], c[k], nb[k])) * wod[q_count(f[k])] : 0.f;
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) out[k] = q_live(f[k]) ? rv[k] * wod[q_count(f[k])] : 0.f;
        }
        st4(zout, i, out);
        if (DOTS) {
            float qv[4];
            ld4(q, i, qv);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                zq += out[k] * qv[k];
                rz += out[k] * rv[k];
            }
        }
    }
    if (DOTS) {
        float v[2] = {zq, rz};
        block_partials<2>(v, part);
    }
}
// the dots of k_q_smooth<true> (its n block partials): FCG's z.q, r.z and beta, as k_ml_smooth DOTS
__global__ void k_q_finish_dots(const double* __restrict__ part, int n, FcgDev* s) {
    double tot[2];
    if (!finish_partials<2>(part, n, tot)) return;
    s->zq = tot[0];
    s->rz = tot[1];
    double beta = 0.0;
    if (s->it > 0 && s->dq != 0.0) beta = -tot[0] / s->dq;
    set_beta(s, isfinite(beta) ? beta : 0.0);
}
// k_ml_smooth2 at level 0: the first sweep's values at the group and at its six neighbours from r and the
// neighbours' counts (a neighbour with its stencil bit set is a row)
__global__ void k_q_smooth2(QWalk qw, const uint16_t* __restrict__ info, int W, int WH, const float* __restrict__ r,
                            float* __restrict__ zout) {
    __shared__ float wod[8];
    init_wod(wod);
    QWALK(qw, i) {
        unsigned f[4], fym[4], fyp[4], fzm[4], fzp[4];
        float rv[4], rym[4], ryp[4], rzm[4], rzp[4], c[4], out[4];
        info4(info, i, f);
        info4(info, i - W, fym);
        info4(info, i + W, fyp);
        info4(info, i - WH, fzm);
        info4(info, i + WH, fzp);
        ld4(r, i, rv);
        ld4(r, i - W, rym);
        ld4(r, i + W, ryp);
        ld4(r, i - WH, rzm);
        ld4(r, i + WH, rzp);
        const float left = r[i - 1] * wod[q_count(info[i - 1])], right = r[i + 4] * wod[q_count(info[i + 4])];
#pragma unroll
        for (int k = 0; k < 4; k++) c[k] = q_live(f[k]) ? rv[k] * wod[q_count(f[k])] : 0.f;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (!q_live(f[k])) { out[k] = 0.f; continue; }
            float nb[6];
            nb[0] = k == 0 ? left : c[k - 1 < 0 ? 0 : k - 1];
            nb[1] = k == 3 ? right : c[k + 1 > 3 ? 3 : k + 1];
            nb[2] = rym[k] * wod[q_count(fym[k])];
            nb[3] = ryp[k] * wod[q_count(fyp[k])];
            nb[4] = rzm[k] * wod[q_count(fzm[k])];
            nb[5] = rzp[k] * wod[q_count(fzp[k])];
            out[k] = c[k] + (rv[k] - lap4(f[k], c[k], nb)) * wod[q_count(f[k])];
        }
        st4(zout, i, out);
    }
}
// The restriction at level 0 (width a multiple of 64): one warp per listed level-1 chunk, i.e. 32 coarse cells of a
// coarse row that hold a row, and the 64 x 4 fine cells below them.  Lane 8 j + g takes the 4-cell groups g and
// g + 8 of fine row j ((dy, dz) = (j & 1, j >> 1)) and sums each group's residuals into the two coarse cells the
// group covers; a fixed butterfly over the four rows finishes the coarse sums, which lanes 0-7 store.  A group's
// stencil is read where the group holds a row, and so lies in the grid's interior rows (the loads stay inside the
// grid); a group without rows reads the interior group at WH + W + 4 (the grid has at least 4 cells on each side)
// and adds nothing.  Coarse cells outside the listed chunks hold no row and stay 0 from the solve's set-up.
// scal: as k_ml_sum8.
__global__ void k_q_restrict(const int* __restrict__ cchunks, const FcgDev* s, const uint16_t* __restrict__ info, int W,
                             int H, int D, const float* __restrict__ r, const float* __restrict__ z, LvView Cv,
                             float* __restrict__ rc, double* __restrict__ scal, FcgDev* sw, double* __restrict__ part) {
    const int lane = threadIdx.x & 31, j = lane >> 3, g = lane & 7;
    const long long items = s->ncchunks;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const int WH = W * H, cpr = Cv.W / 32;
    double ss = 0, cnt = 0;
    for (long long it = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; it < items; it += nwarps) {
        const int ch = cchunks[it];
        const int crow = ch / cpr, cx0 = (ch - crow * cpr) * 32, Y = crow % Cv.H, Z = crow / Cv.H;
        const long long C0 = (long long)ch * 32;
        const int y = 2 * Y + (j & 1), zz = 2 * Z + (j >> 1);
        const bool inside = y < H && zz < D;
        const int i0 = inside ? (zz * H + y) * W + 2 * cx0 + 4 * g : 0, i1 = inside ? i0 + 32 : 0;
        unsigned f0[4], f1[4];
        info4(info, i0, f0);
        info4(info, i1, f1);
        const bool h0 = inside && ((f0[0] | f0[1] | f0[2] | f0[3]) & 0x8000u);
        const bool h1 = inside && ((f1[0] | f1[1] | f1[2] | f1[3]) & 0x8000u);
        const int safe = WH + W + 4;
        float rv0[4], rv1[4], c0[4], c1[4], nb0[4][6], nb1[4][6];
        ld4(r, h0 ? i0 : safe, rv0);
        ld4(r, h1 ? i1 : safe, rv1);
        stencil4(z, h0 ? i0 : safe, W, WH, c0, nb0);
        stencil4(z, h1 ? i1 : safe, W, WH, c1, nb1);
        float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;   // coarse cells 2g, 2g + 1 and 16 + 2g, 17 + 2g
        if (h0) {
            if (f0[0] & 0x8000u) a0 += rv0[0] - lap4(f0[0], c0[0], nb0[0]);
            if (f0[1] & 0x8000u) a0 += rv0[1] - lap4(f0[1], c0[1], nb0[1]);
            if (f0[2] & 0x8000u) a1 += rv0[2] - lap4(f0[2], c0[2], nb0[2]);
            if (f0[3] & 0x8000u) a1 += rv0[3] - lap4(f0[3], c0[3], nb0[3]);
        }
        if (h1) {
            if (f1[0] & 0x8000u) b0 += rv1[0] - lap4(f1[0], c1[0], nb1[0]);
            if (f1[1] & 0x8000u) b0 += rv1[1] - lap4(f1[1], c1[1], nb1[1]);
            if (f1[2] & 0x8000u) b1 += rv1[2] - lap4(f1[2], c1[2], nb1[2]);
            if (f1[3] & 0x8000u) b1 += rv1[3] - lap4(f1[3], c1[3], nb1[3]);
        }
#pragma unroll
        for (int o = 8; o <= 16; o <<= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, o);
            a1 += __shfl_xor_sync(0xffffffffu, a1, o);
            b0 += __shfl_xor_sync(0xffffffffu, b0, o);
            b1 += __shfl_xor_sync(0xffffffffu, b1, o);
        }
        if (j == 0) {
            *reinterpret_cast<float2*>(rc + C0 + 2 * g) = make_float2(a0, a1);
            *reinterpret_cast<float2*>(rc + C0 + 16 + 2 * g) = make_float2(b0, b1);
            if (scal) {
                const unsigned ca = *reinterpret_cast<const unsigned*>(Cv.info + C0 + 2 * g);
                const unsigned cb = *reinterpret_cast<const unsigned*>(Cv.info + C0 + 16 + 2 * g);
                if (ca & 0x8000u) { ss += (double)a0 * a0; cnt += 1.0; }
                if (ca & 0x80000000u) { ss += (double)a1 * a1; cnt += 1.0; }
                if (cb & 0x8000u) { ss += (double)b0 * b0; cnt += 1.0; }
                if (cb & 0x80000000u) { ss += (double)b1 * b1; cnt += 1.0; }
            }
        }
    }
    if (scal) {
        double tot[3], v[2] = {ss, cnt};
        if (reduce_last(v, part, sw->count, tot)) {
            scal[0] = tot[0];
            scal[1] = tot[1];
            scal[2] = (tot[0] > 0 && tot[1] > 0) ? 1.0 / sqrt(tot[0] / tot[1]) : 1.0;
        }
    }
}
// k_ml_prolong_smooth at level 0 (its coarse level is level 1 or the network's grid, CW x CH x CD).  The group's
// cells x0 .. x0 + 3 have the parents px = x0 / 2 (cells 0, 1) and px + 1 (cells 2, 3); their x neighbours add
// px - 1 and px + 2, their y and z neighbours the same two parents in the neighbouring parent rows (clamped to the
// grid: a neighbour outside it has no stencil bit).
__global__ void k_q_prolong_smooth(QWalk qw, const uint16_t* __restrict__ info, int W, int H, int D,
                                   const float* __restrict__ r, const float* __restrict__ z, const float* __restrict__ ec,
                                   int CW, int CH, const double* __restrict__ alpha, float* __restrict__ tout) {
    __shared__ float wod[8];
    init_wod(wod);
    const float a = alpha ? (float)*alpha : 1.f;
    const int WH = W * H;
    QWALK(qw, i) {
        unsigned f[4];
        float rv[4], c[4], nb[4][6], out[4];
        info4(info, i, f);
        ld4(r, i, rv);
        stencil4(z, i, W, WH, c, nb);
        const int row = i / W, x0 = i - row * W, y = row % H, zz = row / H;
        const int px = x0 >> 1;
        auto prow = [&](int py, int pz) { return ec + ((long long)(pz >> 1) * CH + (py >> 1)) * CW; };
        const float* pc = prow(y, zz);
        const float2 pcc = *reinterpret_cast<const float2*>(pc + px);
        const float pl = pc[px > 0 ? px - 1 : 0], pr = pc[px + 2 < CW ? px + 2 : CW - 1];
        const float2 pym = *reinterpret_cast<const float2*>(prow(y > 0 ? y - 1 : 0, zz) + px);
        const float2 pyp = *reinterpret_cast<const float2*>(prow(y + 1 < H ? y + 1 : H - 1, zz) + px);
        const float2 pzm = *reinterpret_cast<const float2*>(prow(y, zz > 0 ? zz - 1 : 0) + px);
        const float2 pzp = *reinterpret_cast<const float2*>(prow(y, zz + 1 < D ? zz + 1 : D - 1) + px);
        const float P[4] = {pcc.x, pcc.x, pcc.y, pcc.y};
        const float PL[4] = {pl, pcc.x, pcc.x, pcc.y};
        const float PR[4] = {pcc.x, pcc.y, pcc.y, pr};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const unsigned fk = f[k];
            if (!q_live(fk)) { out[k] = 0.f; continue; }
            const float zc = c[k] + a * P[k];
            float sum = -(float)q_count(fk) * zc;
            if (fk & 1u) sum += nb[k][0] + a * PL[k];
            if (fk & 2u) sum += nb[k][1] + a * PR[k];
            if (fk & 4u) sum += nb[k][2] + a * (k < 2 ? pym.x : pym.y);
            if (fk & 8u) sum += nb[k][3] + a * (k < 2 ? pyp.x : pyp.y);
            if (fk & 16u) sum += nb[k][4] + a * (k < 2 ? pzm.x : pzm.y);
            if (fk & 32u) sum += nb[k][5] + a * (k < 2 ? pzp.x : pzp.y);
            out[k] = zc + (rv[k] - sum) * wod[q_count(fk)];
        }
        st4(tout, i, out);
    }
}
// k_fcg_dir_matvec at level 0
__global__ void k_q_dir_matvec(QWalk qw, const uint16_t* __restrict__ info, int W, int WH, const float* __restrict__ z,
                               float* __restrict__ d0, float* __restrict__ d1, float* __restrict__ q, FcgDev* s,
                               double* __restrict__ part) {
    const float beta = s->beta_f;
    const float* d = s->par ? d1 : d0;
    float* dn = s->par ? d0 : d1;
    float dq = 0.f;
    QWALK(qw, i) {
        unsigned f[4];
        float zc[4], zn[4][6], dc[4], dnb[4][6], dv[4], qv[4];
        info4(info, i, f);
        stencil4(z, i, W, WH, zc, zn);
        stencil4(d, i, W, WH, dc, dnb);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            dv[k] = zc[k] + beta * dc[k];
            float nbv[6];
#pragma unroll
            for (int n = 0; n < 6; n++) nbv[n] = zn[k][n] + beta * dnb[k][n];
            qv[k] = (f[k] & 0x8000u) ? lap4(f[k], dv[k], nbv) : 0.f;
            dq += dv[k] * qv[k];
        }
        st4(dn, i, dv);
        st4(q, i, qv);
    }
    float v[1] = {dq};
    block_partials<1>(v, part);
}
// d.q of k_q_dir_matvec and alpha, as k_fcg_dir_matvec
__global__ void k_q_finish_dq(const double* __restrict__ part, int n, FcgDev* s) {
    double tot[1];
    if (!finish_partials<1>(part, n, tot)) return;
    s->dq = tot[0];
    shift_alpha(s);
    const double al = s->rz / tot[0];
    if (!(tot[0] < 0.0) || !isfinite(al)) {
        s->stall = 1;
        set_alpha(s, 0.0);
    } else {
        set_alpha(s, al);
    }
}
// k_fcg_update at level 0
__global__ void k_q_update(QWalk qw, float2* __restrict__ x, float* __restrict__ r, const float* __restrict__ d0,
                           const float* __restrict__ d1, const float* __restrict__ q, const FcgDev* s,
                           double* __restrict__ part) {
    const float af = s->alpha_hi, al = s->alpha_lo, pf = s->alpha_prev_hi, pl = s->alpha_prev_lo;
    const bool lag = s->xlag;
    const float* dprev = s->par ? d1 : d0;   // the previous direction, whose step x lacks when lag
    const float* dcur = s->par ? d0 : d1;    // this iteration's
    float rr = 0.f;
    QWALK(qw, i) {
        float rv[4], qv[4];
        ld4(r, i, rv);
        ld4(q, i, qv);
        if (lag) {
            // both steps, in the order the iterations take them
            float dp[4], dv[4];
            ld4(dprev, i, dp);
            ld4(dcur, i, dv);
            float4* x4 = reinterpret_cast<float4*>(x + i);
            float4 x01 = x4[0], x23 = x4[1];
            float2 p0 = df_axpy(df_axpy(make_float2(x01.x, x01.y), pf, pl, dp[0]), af, al, dv[0]);
            float2 p1 = df_axpy(df_axpy(make_float2(x01.z, x01.w), pf, pl, dp[1]), af, al, dv[1]);
            float2 p2 = df_axpy(df_axpy(make_float2(x23.x, x23.y), pf, pl, dp[2]), af, al, dv[2]);
            float2 p3 = df_axpy(df_axpy(make_float2(x23.z, x23.w), pf, pl, dp[3]), af, al, dv[3]);
            x4[0] = make_float4(p0.x, p0.y, p1.x, p1.y);
            x4[1] = make_float4(p2.x, p2.y, p3.x, p3.y);
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            rv[k] = rv[k] - af * qv[k];
            rr += rv[k] * rv[k];
        }
        st4(r, i, rv);
    }
    float v[1] = {rr};
    block_partials<1>(v, part);
}
// r.r of k_q_update, the iteration count, the stall window and the verification decision, as k_fcg_update
__global__ void k_q_finish_rr(const double* __restrict__ part, int n, FcgDev* s, cudaGraphConditionalHandle verify) {
    double tot[1];
    if (!finish_partials<1>(part, n, tot)) return;
    s->rr = tot[0];
    s->it += 1;
    const bool below = s->rr < s->thr;
    if (!below && !s->stall && (s->it % 10) == 0) {
        if (!(s->rr <= 0.5 * s->rr_window)) s->stall = 1;
        s->rr_window = s->rr;
    }
    s->verify = !s->stall && (below || (s->it % 32) == 0);
    s->par ^= 1;
    s->xlag ^= 1;
    cudaGraphSetConditional(verify, s->verify ? 1u : 0u);
}

// ---- FCG ------------------------------------------------------------------------------------------------------
// x = 0, r = b on rows (0 on the other visited cells), d = q = 0; b.b and the row count; the stop threshold as
// the CG solvers form it (k_solver): tol_rel^2 b.b rounded to float, or the absolute one
__global__ void k_fcg_init(LvView F, Walk wk, const float* __restrict__ b, float2* __restrict__ x, float* __restrict__ r,
                           float* __restrict__ d, float* __restrict__ q, FcgDev* s, double* __restrict__ part,
                           float tol_rel, float abs_thr, int max_it, cudaGraphConditionalHandle loop) {
    double bb = 0, rows = 0;
    WALK(wk, t, i) {
        const bool row = F.info[i] & 0x8000u;
        const float bi = row ? b[i] : 0.f;
        x[i] = make_float2(0.f, 0.f);
        r[i] = bi;
        d[i] = 0.f;
        q[i] = 0.f;
        bb += (double)bi * bi;
        rows += row ? 1.0 : 0.0;
    }
    double tot[3];
    double v[2] = {bb, rows};
    if (reduce_last(v, part, s->count, tot)) {
        s->bb = tot[0];
        s->rows = tot[1];
        s->rr = tot[0];
        double thr;
        if (tol_rel > 0) {
            float tf = (float)((double)tol_rel * (double)tol_rel * tot[0]);
            if (!(tf > 0)) tf = FLT_MIN;
            thr = (double)tf;
        } else {
            thr = (double)abs_thr;
        }
        s->thr = thr;
        s->conv = s->rr < thr;
        s->it = 0;
        s->stall = 0;
        s->verify = 0;
        s->fallback = 0;
        s->rr_window = s->rr;
        s->rz = s->dq = s->zq = 0;
        set_alpha(s, 0.0);
        shift_alpha(s);
        set_beta(s, 0.0);
        s->par = 0;          // d (zeroed above) is buffer 0
        s->xlag = 0;
        s->ls_alpha = 1.0;
        cudaGraphSetConditional(loop, (!s->conv && max_it > 0) ? 1u : 0u);
    }
}
// dn = z + beta d (on the fly for the stencil's neighbours), q = A dn; d.q and alpha = (r.z) / (dn.q).  L is
// negative definite on the rows, so dn.q >= 0 (or a non-finite alpha) is a breakdown: the solve stalls.
// d is direction buffer par, dn the other.
__global__ void k_fcg_dir_matvec(LvView F, Walk wk, const float* __restrict__ z, float* __restrict__ d0,
                                 float* __restrict__ d1, float* __restrict__ q, FcgDev* s, double* __restrict__ part) {
    const float beta = s->beta_f;
    const float* d = s->par ? d1 : d0;
    float* dn = s->par ? d0 : d1;
    float dq = 0.f;
    WALK(wk, t, i) {
        float dg, w[6];
        const float di = z[i] + beta * d[i];
        float qi = 0.f;
        if (lrow<true>(F, i, dg, w)) {
            qi = dg * di;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if (w[k] != 0.f) {
                    const long long j = i + noff(F, k);
                    qi += z[j] + beta * d[j];
                }
        }
        dn[i] = di;
        q[i] = qi;
        dq += di * qi;
    }
    double tot[3];
    float v[1] = {dq};
    if (reduce_last(v, part, s->count, tot)) {
        s->dq = tot[0];
        shift_alpha(s);
        const double a = s->rz / tot[0];
        if (!(tot[0] < 0.0) || !isfinite(a)) {
            s->stall = 1;
            set_alpha(s, 0.0);
        } else {
            set_alpha(s, a);
        }
    }
}
// r -= alpha q and, every other iteration, x += alpha' d' + alpha dn (the previous step and this one, in that
// order); r.r, the iteration count, the stall window and whether the true residual is recomputed now (every 32
// iterations and when the recurrence residual meets the threshold); the direction buffers swap
__global__ void k_fcg_update(Walk wk, float2* __restrict__ x, float* __restrict__ r, const float* __restrict__ d0,
                             const float* __restrict__ d1, const float* __restrict__ q, FcgDev* s,
                             double* __restrict__ part, cudaGraphConditionalHandle verify) {
    const float af = s->alpha_hi, al = s->alpha_lo, pf = s->alpha_prev_hi, pl = s->alpha_prev_lo;
    const bool lag = s->xlag;
    const float* dprev = s->par ? d1 : d0;
    const float* dcur = s->par ? d0 : d1;
    float rr = 0.f;
    WALK(wk, t, i) {
        if (lag) x[i] = df_axpy(df_axpy(x[i], pf, pl, dprev[i]), af, al, dcur[i]);
        const float ri = r[i] - af * q[i];
        r[i] = ri;
        rr += ri * ri;
    }
    double tot[3];
    float v[1] = {rr};
    if (reduce_last(v, part, s->count, tot)) {
        s->rr = tot[0];
        s->it += 1;
        const bool below = s->rr < s->thr;
        if (!below && !s->stall && (s->it % 10) == 0) {
            if (!(s->rr <= 0.5 * s->rr_window)) s->stall = 1;
            s->rr_window = s->rr;
        }
        s->verify = !s->stall && (below || (s->it % 32) == 0);
        s->par ^= 1;
        s->xlag ^= 1;
        cudaGraphSetConditional(verify, s->verify ? 1u : 0u);
    }
}
// r = b - A x in float pairs (rows), with x's pending step alpha d (d: direction buffer par) formed on the fly;
// r.r and the convergence decision
__global__ void k_fcg_true_resid(LvView F, Walk wk, const float* __restrict__ b, const float2* __restrict__ x,
                                 const float* __restrict__ d0, const float* __restrict__ d1, float* __restrict__ r,
                                 FcgDev* s, double* __restrict__ part) {
    const bool lag = s->xlag;
    const float* d = s->par ? d1 : d0;
    const float ah = s->alpha_hi, al = s->alpha_lo;
    double rr = 0;
    WALK(wk, t, i) {
        float dg, w[6];
        float ri = 0.f;
        if (lrow<true>(F, i, dg, w))
            ri = lag ? resid_pair_step(F, i, x, d, ah, al, b[i], F.info[i]) : resid_pair(F, i, x, b[i], F.info[i]);
        r[i] = ri;
        rr += (double)ri * ri;
    }
    double tot[3];
    double v[1] = {rr};
    if (reduce_last(v, part, s->count, tot)) {
        s->rr = tot[0];
        s->conv = s->rr < s->thr;
    }
}
// after the loop: x's pending step, if any (x += alpha d, d: direction buffer par)
__global__ void k_fcg_flush(Walk wk, float2* __restrict__ x, const float* __restrict__ d0, const float* __restrict__ d1,
                            const FcgDev* __restrict__ s) {
    if (!s->xlag) return;
    const float* d = s->par ? d1 : d0;
    const float ah = s->alpha_hi, al = s->alpha_lo;
    WALK(wk, t, i) { x[i] = df_axpy(x[i], ah, al, d[i]); }
}
// the loop condition for the next iteration
__global__ void k_fcg_loop(const FcgDev* __restrict__ s, int max_it, cudaGraphConditionalHandle loop) {
    if (threadIdx.x != 0) return;
    cudaGraphSetConditional(loop, (!s->conv && !s->stall && s->it < max_it) ? 1u : 0u);
}
// after the loop: hand a stalled, unconverged solve to plain CG
__global__ void k_fcg_post(FcgDev* s, cudaGraphConditionalHandle fallback) {
    if (threadIdx.x != 0) return;
    cudaGraphSetConditional(fallback, (s->stall && !s->conv) ? 1u : 0u);
}
// fb = b - A x in FP64 on rows, 0 elsewhere (the right-hand side of the fallback CG; every cell written)
__global__ void k_fcg_fb_rhs(LvView F, const float* __restrict__ b, const float2* __restrict__ x, float* __restrict__ fb) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= F.V) return;
    float dg, w[6];
    fb[i] = lrow<true>(F, i, dg, w) ? resid_pair(F, i, x, b[i], F.info[i]) : 0.f;
}
__global__ void k_fcg_fb_add(LvView F, Walk wk, float2* __restrict__ x, const float* __restrict__ p) {
    WALK(wk, t, i) {
        if (F.info[i] & 0x8000u) x[i] = df_axpy(x[i], 1.f, 0.f, p[i]);
    }
}
__global__ void k_fcg_fb_done(FcgDev* s, const DevCtl* ctl) {
    if (threadIdx.x != 0) return;
    s->fallback = 1;
    s->conv = ctl->converged;
}
__global__ void k_fcg_out(LvView F, Walk wk, const float2* __restrict__ x, float* __restrict__ p, double* __restrict__ p64) {
    WALK(wk, t, i) {
        if (F.info[i] & 0x8000u) {
            const double v = df_val(x[i]);
            p[i] = (float)v;
            p64[i] = v;
        }
    }
}
// solve statistics into the control block; after a fallback the CG launch has counted the solve and its own
// iterations and convergence, to which the FCG iterations are added
__global__ void k_fcg_stats(const FcgDev* __restrict__ s, DevCtl* ctl) {
    if (threadIdx.x != 0) return;
    const int it = s->it;
    ctl->precond_iterations = it;
    if (s->fallback) {
        ctl->iterations += it;
        ctl->bb = s->bb;
    } else {
        ctl->converged = s->conv;
        ctl->iterations = it;
        ctl->rr = s->rr;
        ctl->bb = s->bb;
        ctl->thr = s->thr;
        ctl->active_cells = (long long)s->rows;
        ctl->solves += 1;
        ctl->sum_rows += s->rows;
    }
    ctl->total_iterations += it;
    ctl->sum_iter_rows += (double)it * s->rows;
}

// host-driven CG on one level (training samples): dots through these partials
__global__ void k_lv_dot3(long long n, const float* a0, const float* b0, const float* a1, const float* b1,
                          double* __restrict__ part) {
    double s0 = 0, s1 = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        s0 += (double)a0[i] * b0[i];
        if (a1) s1 += (double)a1[i] * b1[i];
    }
    double v[2] = {s0, s1};
    block_partials<2>(v, part);
}
__global__ void k_lv_axpy2(long long n, float* __restrict__ x, float* __restrict__ r, const float* __restrict__ d,
                           const float* __restrict__ q, double alpha) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = (float)((double)x[i] + alpha * d[i]);
    r[i] = (float)((double)r[i] - alpha * q[i]);
}
__global__ void k_lv_xpby(long long n, float* __restrict__ d, const float* __restrict__ r, double beta) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) d[i] = (float)((double)r[i] + beta * d[i]);
}

#define MCK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return e_; } while (0)

}  // namespace

// ---- state -----------------------------------------------------------------------------------------------------
struct MLLevel {
    int W = 0, H = 0, D = 0;
    long long V = 0;
    uint16_t* info = nullptr;
    uint8_t* w = nullptr;
    float* diag = nullptr;
    float* wd = nullptr;          // kOmega / diag on the rows, 0 elsewhere
    float *r = nullptr, *z = nullptr, *t = nullptr;
};

struct MLState {
    int nlev = 0;                 // aggregation levels of the allocated hierarchy
    MLLevel lv[4];                // lv[1..nlev]
    float2* xp = nullptr;         // FCG's x as float pairs (df_axpy), and its other vectors (fine grid)
    float *r = nullptr, *z = nullptr, *zt = nullptr, *d = nullptr, *dn = nullptr, *q = nullptr, *fb = nullptr;
    int* chunks = nullptr;        // level 0: the 32-cell chunks that hold a matrix row, in order
    int* bcount = nullptr;        // their per-block counts / offsets
    int* cchunks = nullptr;       // level 1: the 32-cell chunks that hold a row, in order (k_q_restrict)
    int* cbcount = nullptr;
    long long cnch = 0;           // chunks of level 1
    long long nch = 0;            // chunks of the fine grid
    double* part = nullptr;       // 3 * kGrid block partials
    FcgDev* s = nullptr;
    double* hpart = nullptr;      // pinned: partials of the host-driven level CG
    cudaStream_t cap1 = nullptr, cap2 = nullptr;   // streams for capturing conditional bodies
    cudaGraph_t solve_graph = nullptr;
    cudaGraphExec_t solve_exec = nullptr;          // efs_solve / efs_stage outside a step graph
    std::vector<void*> allocs;
};

namespace {

template <typename T>
cudaError_t malloc_ml(MLState* m, T** p, long long count) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), (size_t)std::max(1LL, count) * sizeof(T));
    if (e == cudaSuccess) m->allocs.push_back(*p);
    return e;
}

// Level 1's chunk list is built (and walked by level 1's kernels and the level-0 restriction) when level 1's rows
// are whole 32-cell chunks of its grid rows.
bool restrict_list(const efs_ctx* c) { return c->g.W % 64 == 0 && c->g.H >= 4 && c->g.D >= 4; }

LvView fine_view(const efs_ctx* c) {
    return LvView{c->g.W, c->g.H, c->g.D, (long long)c->g.N, c->rowinfo, nullptr, nullptr};
}
LvView level_view(const efs_ctx* c, const MLState* m, int l) {
    if (l == 0) return fine_view(c);
    const MLLevel& L = m->lv[l];
    return LvView{L.W, L.H, L.D, L.V, L.info, L.w, L.diag, L.wd};
}
// level 0 visits the chunk list, coarser levels every cell
Walk walk_of(const efs_ctx* c, const MLState* m, int l) {
    if (l == 0) return Walk{m->chunks, &m->s->nchunks, (long long)c->g.N};
    if (l == 1 && m->cchunks && restrict_list(c)) return Walk{m->cchunks, &m->s->ncchunks, m->lv[1].V};
    return Walk{nullptr, nullptr, m->lv[l].V};
}

}  // namespace

int ml_resolve_levels(const efs_ctx* c) {
    if (c->dim != 3) return 0;
    int l = c->prm.fcg_levels;
    if (l >= 0) return std::min(l, 3);
    int W = c->g.W, H = c->g.H, D = c->g.D;
    l = 0;
    while (l < 3 && std::max(W, std::max(H, D)) > 32) {
        W = (W + 1) / 2; H = (H + 1) / 2; D = (D + 1) / 2;
        l++;
    }
    return l;
}

void ml_level_dims(const efs_ctx* c, int level, int* W, int* H, int* D) {
    int w = c->g.W, h = c->g.H, d = c->g.D;
    for (int k = 0; k < level; k++) { w = (w + 1) / 2; h = (h + 1) / 2; d = (d + 1) / 2; }
    *W = w; *H = h; *D = d;
}

void ml_free(efs_ctx* c) {
    MLState* m = c->ml;
    if (!m) return;
    if (m->solve_exec) cudaGraphExecDestroy(m->solve_exec);
    if (m->solve_graph) cudaGraphDestroy(m->solve_graph);
    for (void* p : m->allocs) cudaFree(p);
    if (m->hpart) cudaFreeHost(m->hpart);
    if (m->cap1) cudaStreamDestroy(m->cap1);
    if (m->cap2) cudaStreamDestroy(m->cap2);
    delete m;
    c->ml = nullptr;
}

void ml_drop_graph(efs_ctx* c) {
    MLState* m = c->ml;
    if (!m) return;
    if (m->solve_exec) cudaGraphExecDestroy(m->solve_exec);
    if (m->solve_graph) cudaGraphDestroy(m->solve_graph);
    m->solve_exec = nullptr;
    m->solve_graph = nullptr;
}

// Buffers for the context's current level count (outside any stream capture; kept while the count holds).
cudaError_t ml_alloc(efs_ctx* c) {
    const int nlev = ml_resolve_levels(c);
    if (c->ml && c->ml->nlev == nlev) return cudaSuccess;
    ml_free(c);
    MLState* m = new MLState();
    c->ml = m;
    m->nlev = nlev;
    const long long N = c->g.N;
    m->nch = (N + 31) / 32;
    MCK(malloc_ml(m, &m->xp, N));
    MCK(malloc_ml(m, &m->r, N));
    MCK(malloc_ml(m, &m->z, N));
    MCK(malloc_ml(m, &m->zt, N));
    MCK(malloc_ml(m, &m->d, N));
    MCK(malloc_ml(m, &m->dn, N));
    MCK(malloc_ml(m, &m->q, N));
    MCK(malloc_ml(m, &m->fb, N));
    MCK(malloc_ml(m, &m->chunks, m->nch));
    MCK(malloc_ml(m, &m->bcount, (long long)blocks_for(m->nch)));
    if (nlev >= 1) {
        long long W1 = 0;
        { int w, h, d; ml_level_dims(c, 1, &w, &h, &d); W1 = (long long)w * h * d; }
        m->cnch = (W1 + 31) / 32;
        MCK(malloc_ml(m, &m->cchunks, m->cnch));
        MCK(malloc_ml(m, &m->cbcount, (long long)blocks_for(m->cnch)));
    }
    MCK(malloc_ml(m, &m->part, 3LL * kGrid));
    MCK(malloc_ml(m, &m->s, 1));
    MCK(cudaMemset(m->s, 0, sizeof(FcgDev)));
    for (int l = 1; l <= nlev; l++) {
        MLLevel& L = m->lv[l];
        ml_level_dims(c, l, &L.W, &L.H, &L.D);
        L.V = (long long)L.W * L.H * L.D;
        MCK(malloc_ml(m, &L.info, L.V));
        MCK(malloc_ml(m, &L.w, 6 * L.V));
        MCK(malloc_ml(m, &L.diag, L.V));
        MCK(malloc_ml(m, &L.wd, L.V));
        MCK(malloc_ml(m, &L.r, L.V));
        MCK(malloc_ml(m, &L.z, L.V));
        MCK(malloc_ml(m, &L.t, L.V));
    }
    MCK(cudaMallocHost(reinterpret_cast<void**>(&m->hpart), 3 * kGrid * sizeof(double)));
    MCK(cudaStreamCreateWithFlags(&m->cap1, cudaStreamNonBlocking));
    MCK(cudaStreamCreateWithFlags(&m->cap2, cudaStreamNonBlocking));
    return cudaSuccess;
}

int ml_levels(const efs_ctx* c) { return c->ml ? c->ml->nlev : ml_resolve_levels(c); }

LvView ml_view(const efs_ctx* c, int level) { return level_view(c, c->ml, level); }

// The hierarchy's matrices and the level-0 chunk list from the current rowinfo; with restrict_list, level 1's
// chunk list, and level 1's right-hand side zeroed (k_q_restrict writes only the listed chunks).
cudaError_t ml_build(efs_ctx* c, cudaStream_t st) {
    MLState* m = c->ml;
    const long long N = c->g.N;
    const unsigned nb = blocks_for(m->nch);
    k_chunks_count<<<nb, kThreads, 0, st>>>(c->rowinfo, N, m->nch, m->bcount);
    k_chunks_scan<<<1, 1024, 0, st>>>(m->bcount, (int)nb, &m->s->nchunks);
    k_chunks_write<<<nb, kThreads, 0, st>>>(c->rowinfo, N, m->nch, m->bcount, m->chunks);
    MCK(cudaGetLastError());
    for (int l = 1; l <= m->nlev; l++) {
        const MLLevel& L = m->lv[l];
        const LvOut out{L.W, L.H, L.D, L.V, L.info, L.w, L.diag, L.wd};
        if (l == 1) k_ml_build<true><<<blocks_for(L.V), kThreads, 0, st>>>(level_view(c, m, 0), out);
        else k_ml_build<false><<<blocks_for(L.V), kThreads, 0, st>>>(level_view(c, m, l - 1), out);
        MCK(cudaGetLastError());
    }
    if (m->nlev >= 1 && restrict_list(c)) {
        const MLLevel& L1 = m->lv[1];
        const unsigned nb1 = blocks_for(m->cnch);
        k_chunks_count<<<nb1, kThreads, 0, st>>>(L1.info, L1.V, m->cnch, m->cbcount);
        k_chunks_scan<<<1, 1024, 0, st>>>(m->cbcount, (int)nb1, &m->s->ncchunks);
        k_chunks_write<<<nb1, kThreads, 0, st>>>(L1.info, L1.V, m->cnch, m->cbcount, m->cchunks);
        MCK(cudaGetLastError());
        MCK(cudaMemsetAsync(L1.r, 0, (size_t)L1.V * sizeof(float), st));
    }
    return cudaSuccess;
}

cudaError_t ml_matvec(const LvView& L, const float* x, float* y, cudaStream_t st) {
    if (!L.w) k_ml_matvec<true><<<blocks_for(L.V), kThreads, 0, st>>>(L, x, y);
    else k_ml_matvec<false><<<blocks_for(L.V), kThreads, 0, st>>>(L, x, y);
    return cudaGetLastError();
}

namespace {

// level 0 takes the 128-bit kernels when its rows are whole 32-cell chunks of grid rows
bool quad_level0(const efs_ctx* c) { return (c->g.W % 32) == 0 && c->g.H >= 4 && c->g.D >= 4; }
QWalk qwalk_of(const MLState* m) { return QWalk{m->chunks, m->s}; }
// k_q_restrict: one warp per listed level-1 chunk (at most all of them)
unsigned q_restrict_grid(const MLState* m) { return grid_for(m->cnch * 32); }

// one damped Jacobi sweep at level l (zin null: from zero); dots: FCG's z.q and r.z with beta (level 0 only)
cudaError_t sweep(efs_ctx* c, int l, const float* r, const float* zin, float* zout, cudaStream_t st, bool dots = false) {
    MLState* m = c->ml;
    const LvView L = level_view(c, m, l);
    const Walk wk = walk_of(c, m, l);
    const unsigned g = grid_for(l == 0 ? c->g.N : L.V);
    if (l == 0 && quad_level0(c)) {
        const unsigned gq = grid_for(c->g.N / 4);
        if (dots) {
            k_q_smooth<true><<<gq, kThreads, 0, st>>>(qwalk_of(m), c->rowinfo, c->g.W, c->g.WH, r, zin, zout, m->q, m->part);
            k_q_finish_dots<<<1, kThreads, 0, st>>>(m->part, (int)gq, m->s);
        } else {
            k_q_smooth<false><<<gq, kThreads, 0, st>>>(qwalk_of(m), c->rowinfo, c->g.W, c->g.WH, r, zin, zout, nullptr, m->part);
        }
        return cudaGetLastError();
    }
    if (l == 0) {
        if (dots) k_ml_smooth<true, true><<<g, kThreads, 0, st>>>(L, wk, r, zin, zout, kOmega, m->q, m->s, m->part);
        else k_ml_smooth<true, false><<<g, kThreads, 0, st>>>(L, wk, r, zin, zout, kOmega, nullptr, m->s, m->part);
    } else {
        k_ml_smooth<false, false><<<grid_for(L.V), kThreads, 0, st>>>(L, wk, r, zin, zout, kOmega, nullptr, m->s, m->part);
    }
    return cudaGetLastError();
}

// the two pre-smoothing sweeps from zero at level l, in one pass
cudaError_t sweep2(efs_ctx* c, int l, const float* r, float* zout, cudaStream_t st) {
    MLState* m = c->ml;
    const LvView L = level_view(c, m, l);
    const Walk wk = walk_of(c, m, l);
    if (l == 0 && quad_level0(c))
        k_q_smooth2<<<grid_for(c->g.N / 4), kThreads, 0, st>>>(qwalk_of(m), c->rowinfo, c->g.W, c->g.WH, r, zout);
    else if (l == 0) k_ml_smooth2<true><<<grid_for(c->g.N), kThreads, 0, st>>>(L, wk, r, zout, kOmega);
    else k_ml_smooth2<false><<<grid_for(L.V), kThreads, 0, st>>>(L, wk, r, zout, kOmega);
    return cudaGetLastError();
}

// restriction from level l to l + 1 (the non-128-bit paths): residual into the level's scratch t, then the sums
cudaError_t restrict2(efs_ctx* c, int l, const float* r, const float* z, float* t, float* rc, double* scal,
                      cudaStream_t st) {
    MLState* m = c->ml;
    const LvView L = level_view(c, m, l), Cv = level_view(c, m, l + 1);
    const Walk wk = walk_of(c, m, l);
    if (l == 0) k_ml_resid<true><<<grid_for(c->g.N), kThreads, 0, st>>>(L, wk, r, z, t);
    else k_ml_resid<false><<<grid_for(L.V), kThreads, 0, st>>>(L, wk, r, z, t);
    MCK(cudaGetLastError());
    if (l == 0) k_ml_sum8<true><<<grid_for(Cv.V), kThreads, 0, st>>>(L, t, Cv, rc, scal, m->s, m->part);
    else k_ml_sum8<false><<<grid_for(Cv.V), kThreads, 0, st>>>(L, t, Cv, rc, scal, m->s, m->part);
    return cudaGetLastError();
}

bool net_bottom(const efs_ctx* c) { return c->prm.fcg_bottom == EFS_FCG_BOTTOM_UNET && c->unet; }

// z = M(r) at level l (r, z, t: that level's vectors).  Level 0 ends with FCG's z.q, r.z and beta.  At the
// bottom level with the network the correction stays in the network's output buffer, scaled by s->ls_alpha when
// the level above prolongs it.
cudaError_t vcycle(efs_ctx* c, int l, const float* r, float* z, float* t, cudaStream_t st) {
    MLState* m = c->ml;
    const LvView L = level_view(c, m, l);
    const Walk wk = walk_of(c, m, l);
    const int nb = m->nlev;
    if (l == nb) {
        // bottom solve
        if (net_bottom(c)) {
            if (l == 0) MCK(unet_scale_rows(c, L, r, st));
            MCK(unet_forward_prescaled(c, L, r, st));
            const float* e = unet_output(c);
            const unsigned g = grid_for(l == 0 ? c->g.N : L.V);
            if (l == 0) k_ml_line_search<true><<<g, kThreads, 0, st>>>(L, wk, e, r, m->s, m->part);
            else k_ml_line_search<false><<<g, kThreads, 0, st>>>(L, wk, e, r, m->s, m->part);
            MCK(cudaGetLastError());
            if (l == 0) {
                k_take_dots<<<g, kThreads, 0, st>>>(L, wk, e, m->q, r, z, m->s, m->part);
                MCK(cudaGetLastError());
            }
            return cudaSuccess;
        }
        float* a = z;
        float* o = t;
        MCK(sweep(c, l, r, nullptr, a, st, l == 0 && kBottomJacobi == 1));
        for (int k = 1; k < kBottomJacobi; k++) {
            MCK(sweep(c, l, r, a, o, st, l == 0 && k == kBottomJacobi - 1));
            std::swap(a, o);
        }
        if (a != z) MCK(cudaMemcpyAsync(z, a, L.V * sizeof(float), cudaMemcpyDeviceToDevice, st));
        return cudaSuccess;
    }
    const LvView Cv = level_view(c, m, l + 1);
    MLLevel& N = m->lv[l + 1];
    const bool to_net = (l + 1 == nb) && net_bottom(c);
    // pre-smoothing, restriction
    MCK(sweep2(c, l, r, z, st));
    if (l == 0 && restrict_list(c))
        k_q_restrict<<<q_restrict_grid(m), kThreads, 0, st>>>(m->cchunks, m->s, c->rowinfo, c->g.W, c->g.H, c->g.D, r, z,
                                                              Cv, N.r, to_net ? unet_scale_slot(c) : nullptr, m->s, m->part);
    else MCK(restrict2(c, l, r, z, t, N.r, to_net ? unet_scale_slot(c) : nullptr, st));
    MCK(cudaGetLastError());
    MCK(vcycle(c, l + 1, N.r, N.z, N.t, st));
    // prolongation folded into the first post-smoothing sweep, then the second sweep
    const float* ec = to_net ? unet_output(c) : N.z;
    const double* a = to_net ? &m->s->ls_alpha : nullptr;
    const unsigned g = grid_for(l == 0 ? c->g.N : L.V);
    if (l == 0 && quad_level0(c))
        k_q_prolong_smooth<<<grid_for(c->g.N / 4), kThreads, 0, st>>>(qwalk_of(m), c->rowinfo, c->g.W, c->g.H, c->g.D, r, z,
                                                                     ec, Cv.W, Cv.H, a, t);
    else if (l == 0) k_ml_prolong_smooth<true><<<g, kThreads, 0, st>>>(L, wk, r, z, ec, Cv, a, t, kOmega);
    else k_ml_prolong_smooth<false><<<grid_for(L.V), kThreads, 0, st>>>(L, wk, r, z, ec, Cv, a, t, kOmega);
    MCK(cudaGetLastError());
    return sweep(c, l, r, t, z, st, l == 0);
}

// a conditional handle on the graph `st` is capturing into
cudaError_t make_handle(cudaStream_t st, cudaGraphConditionalHandle* h) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    MCK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
    if (cs != cudaStreamCaptureStatusActive || !g) return cudaErrorStreamCaptureUnmatched;
    return cudaGraphConditionalHandleCreate(h, g, 0, 0);
}
// a conditional node after `st`'s current capture dependencies; `st` continues after it; *body to be filled
cudaError_t add_conditional(cudaStream_t st, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                            cudaGraph_t* body) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    MCK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = type;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    MCK(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    *body = p.conditional.phGraph_out[0];
    return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

// The whole solve on `st`, which is capturing into a graph.
cudaError_t fcg_enqueue(efs_ctx* c, cudaStream_t st) {
    MLState* m = c->ml;
    const LvView F = fine_view(c);
    const Walk wk = walk_of(c, m, 0);
    const long long N = F.V;
    const unsigned g = grid_for(N);
    const int max_it = c->prm.max_steps;
    MCK(ml_build(c, st));
    cudaGraphConditionalHandle h_loop, h_verify, h_fb;
    MCK(make_handle(st, &h_loop));
    k_fcg_init<<<g, kThreads, 0, st>>>(F, wk, c->div, m->xp, m->r, m->d, m->q, m->s, m->part, c->prm.tol_rel,
                                      c->prm.solver_threshold, max_it, h_loop);
    MCK(cudaGetLastError());

    // ---- WHILE: one FCG iteration ----
    cudaGraph_t body = nullptr;
    MCK(add_conditional(st, h_loop, cudaGraphCondTypeWhile, &body));
    {
        cudaStream_t b = m->cap1;
        MCK(cudaStreamBeginCaptureToGraph(b, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        do {
            // z = M(r), with z.q, r.z and beta at its end
            if ((e = vcycle(c, 0, m->r, m->z, m->zt, b)) != cudaSuccess) break;
            const bool quad = quad_level0(c);
            const unsigned gq = grid_for(N / 4);
            if (quad) {
                k_q_dir_matvec<<<gq, kThreads, 0, b>>>(qwalk_of(m), c->rowinfo, c->g.W, c->g.WH, m->z, m->d, m->dn, m->q, m->s, m->part);
                k_q_finish_dq<<<1, kThreads, 0, b>>>(m->part, (int)gq, m->s);
            } else {
                k_fcg_dir_matvec<<<g, kThreads, 0, b>>>(F, wk, m->z, m->d, m->dn, m->q, m->s, m->part);
            }
            if ((e = make_handle(b, &h_verify)) != cudaSuccess) break;
            if (quad) {
                k_q_update<<<gq, kThreads, 0, b>>>(qwalk_of(m), m->xp, m->r, m->d, m->dn, m->q, m->s, m->part);
                k_q_finish_rr<<<1, kThreads, 0, b>>>(m->part, (int)gq, m->s, h_verify);
            } else {
                k_fcg_update<<<g, kThreads, 0, b>>>(wk, m->xp, m->r, m->d, m->dn, m->q, m->s, m->part, h_verify);
            }
            if ((e = cudaGetLastError()) != cudaSuccess) break;
            // ---- IF: the true residual in FP64 (every 32 iterations and before stopping) ----
            cudaGraph_t vbody = nullptr;
            if ((e = add_conditional(b, h_verify, cudaGraphCondTypeIf, &vbody)) != cudaSuccess) break;
            cudaStream_t v = m->cap2;
            if ((e = cudaStreamBeginCaptureToGraph(v, vbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) break;
            k_fcg_true_resid<<<g, kThreads, 0, v>>>(F, wk, c->div, m->xp, m->d, m->dn, m->r, m->s, m->part);
            cudaError_t ve = cudaGetLastError();
            cudaGraph_t dummy = nullptr;
            cudaError_t ee = cudaStreamEndCapture(v, &dummy);
            if ((e = ve) != cudaSuccess || (e = ee) != cudaSuccess) break;
            k_fcg_loop<<<1, 32, 0, b>>>(m->s, max_it, h_loop);
            e = cudaGetLastError();
        } while (0);
        cudaGraph_t dummy = nullptr;
        cudaError_t ee = cudaStreamEndCapture(b, &dummy);
        MCK(e);
        MCK(ee);
    }

    k_fcg_flush<<<g, kThreads, 0, st>>>(wk, m->xp, m->d, m->dn, m->s);
    MCK(cudaGetLastError());
    // ---- IF: the plain-CG fallback on the residual system ----
    MCK(make_handle(st, &h_fb));
    k_fcg_post<<<1, 32, 0, st>>>(m->s, h_fb);
    MCK(cudaGetLastError());
    cudaGraph_t fbody = nullptr;
    MCK(add_conditional(st, h_fb, cudaGraphCondTypeIf, &fbody));
    {
        cudaStream_t b = m->cap1;
        MCK(cudaStreamBeginCaptureToGraph(b, fbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        do {
            k_fcg_fb_rhs<<<blocks_for(N), kThreads, 0, b>>>(F, c->div, m->xp, m->fb);
            if ((e = cudaGetLastError()) != cudaSuccess) break;
            if ((e = launch_solver_on(c, m->fb, &m->s->thr, b)) != cudaSuccess) break;
            k_fcg_fb_add<<<g, kThreads, 0, b>>>(F, wk, m->xp, c->p);
            k_fcg_fb_done<<<1, 32, 0, b>>>(m->s, c->ctl);
            e = cudaGetLastError();
        } while (0);
        cudaGraph_t dummy = nullptr;
        cudaError_t ee = cudaStreamEndCapture(b, &dummy);
        MCK(e);
        MCK(ee);
    }
    k_fcg_out<<<g, kThreads, 0, st>>>(F, wk, m->xp, c->p, c->p64);
    k_fcg_stats<<<1, 32, 0, st>>>(m->s, c->ctl);
    return cudaGetLastError();
}

}  // namespace

cudaError_t fcg_solve(efs_ctx* c) {
    if (!c->ml || c->ml->nlev != ml_resolve_levels(c)) return cudaErrorNotReady;   // ml_alloc runs before any capture
    cudaStreamCaptureStatus cs;
    MCK(cudaStreamIsCapturing(c->stream, &cs));
    if (cs == cudaStreamCaptureStatusActive) return fcg_enqueue(c, c->stream);
    MLState* m = c->ml;
    if (!m->solve_exec) {
        MCK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = fcg_enqueue(c, c->stream);
        cudaGraph_t g = nullptr;
        cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
        if (e != cudaSuccess || ee != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return e != cudaSuccess ? e : ee;
        }
        cudaGraphExec_t x = nullptr;
        e = cudaGraphInstantiate(&x, g, 0);
        if (e != cudaSuccess) { cudaGraphDestroy(g); return e; }
        m->solve_graph = g;
        m->solve_exec = x;
    }
    return cudaGraphLaunch(m->solve_exec, c->stream);
}

// Device time of one application of the preconditioner (the V-cycle, with the network or the Jacobi sweeps at the
// bottom) on r = the current divergence: `reps` applications as direct launches, then `reps` replays of one
// captured application (what a solve's loop body pays).  Builds the hierarchy from the current rowinfo first.
cudaError_t ml_time_vcycle(efs_ctx* c, int reps, float* ms_direct, float* ms_graph) {
    MLState* m = c->ml;
    cudaStream_t st = c->stream;
    const size_t bytes = (size_t)c->g.N * sizeof(float);
    MCK(ml_build(c, st));
    MCK(cudaMemcpyAsync(m->r, c->div, bytes, cudaMemcpyDeviceToDevice, st));
    MCK(cudaMemsetAsync(m->q, 0, bytes, st));   // the previous direction's A d, read by the closing sweep's dots
    MCK(vcycle(c, 0, m->r, m->z, m->zt, st));   // warm-up
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    for (int k = 0; k < reps && e == cudaSuccess; k++) e = vcycle(c, 0, m->r, m->z, m->zt, st);
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) *ms_direct = ms / reps;
    if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t ce = vcycle(c, 0, m->r, m->z, m->zt, st);
        cudaError_t ee = cudaStreamEndCapture(st, &g);
        e = ce != cudaSuccess ? ce : ee;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&x, g, 0);
    if (e == cudaSuccess) e = cudaGraphLaunch(x, st);            // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    for (int k = 0; k < reps && e == cudaSuccess; k++) e = cudaGraphLaunch(x, st);
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) *ms_graph = ms / reps;
    if (x) cudaGraphExecDestroy(x);
    if (g) cudaGraphDestroy(g);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return e;
}

// r (fine) carried down the pre-smoothing and restriction chain to the bottom level: out = the bottom residual
// (outside any capture; builds the hierarchy first)
cudaError_t ml_descend(efs_ctx* c, const float* r0, cudaStream_t st, const float** out) {
    MLState* m = c->ml;
    MCK(ml_build(c, st));
    const float* r = r0;
    for (int l = 0; l < m->nlev; l++) {
        const LvView L = level_view(c, m, l);
        float* z = (l == 0) ? m->z : m->lv[l].z;
        const LvView Cv = level_view(c, m, l + 1);
        MCK(sweep2(c, l, r, z, st));
        if (l == 0 && restrict_list(c))
            k_q_restrict<<<q_restrict_grid(m), kThreads, 0, st>>>(m->cchunks, m->s, c->rowinfo, c->g.W, c->g.H, c->g.D, r,
                                                                  z, Cv, m->lv[1].r, nullptr, m->s, m->part);
        else MCK(restrict2(c, l, r, z, (l == 0) ? m->zt : m->lv[l].t, m->lv[l + 1].r, nullptr, st));
        MCK(cudaGetLastError());
        r = m->lv[l + 1].r;
    }
    *out = r;
    return cudaSuccess;
}

// CG on level matrix L (negative definite on its rows) for L e = r from e = 0, to ||r|| <= tol ||r0||, host-driven
// (training samples only).  t1, t2, t3: scratch vectors of L.V floats.  Returns the iterations, or -1.
int ml_level_cg(efs_ctx* c, const LvView& L, const float* r0, float* e, float* t1, float* t2, float* t3, double tol,
                int maxit, cudaStream_t st) {
    MLState* m = c->ml;
    const long long n = L.V;
    const unsigned rb = grid_for(n), nb = blocks_for(n);
    float *r = t1, *d = t2, *q = t3;
    auto dot2 = [&](const float* a0, const float* b0, const float* a1, const float* b1, double& s0, double& s1) -> bool {
        k_lv_dot3<<<rb, kThreads, 0, st>>>(n, a0, b0, a1, b1, m->part);
        if (cudaMemcpyAsync(m->hpart, m->part, 3 * rb * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return false;
        if (cudaStreamSynchronize(st) != cudaSuccess) return false;
        s0 = s1 = 0;
        for (unsigned k = 0; k < rb; k++) { s0 += m->hpart[3 * k]; s1 += m->hpart[3 * k + 1]; }
        return true;
    };
    if (cudaMemsetAsync(e, 0, n * sizeof(float), st) != cudaSuccess) return -1;
    if (cudaMemcpyAsync(r, r0, n * sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess) return -1;
    if (cudaMemcpyAsync(d, r0, n * sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess) return -1;
    double rr, unused;
    if (!dot2(r, r, nullptr, nullptr, rr, unused)) return -1;
    const double thr = tol * tol * rr;
    int it = 0;
    while (it < maxit && rr > thr && rr > 0) {
        if (ml_matvec(L, d, q, st) != cudaSuccess) return -1;
        double dq;
        if (!dot2(d, q, nullptr, nullptr, dq, unused)) return -1;
        if (!(dq != 0.0)) break;
        const double a = rr / dq;
        k_lv_axpy2<<<nb, kThreads, 0, st>>>(n, e, r, d, q, a);
        double rn;
        if (!dot2(r, r, nullptr, nullptr, rn, unused)) return -1;
        k_lv_xpby<<<nb, kThreads, 0, st>>>(n, d, r, rn / rr);
        rr = rn;
        it++;
    }
    return it;
}

}  // namespace efs
