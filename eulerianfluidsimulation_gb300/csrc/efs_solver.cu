// efs_solver.cu — the pressure solve of project() as one persistent, cooperative sm_103a kernel.
//
// Restates CGSolverCPU3D::solve / CGSolverCPU2D::solve (src/simulation/solver/CGSolver.cpp:32-83, :416-465)
// with impl_mat_mul (:85-111, :467-497), and JacobiSolverCPU3D/2D::solve (src/simulation/solver/
// JacobiSolver.cpp:18-71, :154-212).  Differences from the reference, all in what is computed where:
//   - the whole iteration runs inside one kernel: phases are separated by a grid barrier (bounded spin; a
//     barrier that gives up sets DEV_ERR_BARRIER_TIMEOUT and every block returns), the stop test is made on
//     the device, and no scalar goes to the host;
//   - dot products are accumulated with FP64-class accuracy (compensated float pairs, see FSum): per-block
//     partial sums, then every block adds the partials in the same fixed order, so all blocks take the same
//     branch and results do not depend on timing;
//   - only 32-cell chunks that hold a matrix row or a non-zero right-hand side are visited, and within them
//     only the lanes that hold a row load or store.  Rows outside the matrix are the identity in the
//     reference (result = x), start at p = b and keep r = d = 0, so skipping them changes nothing;
//   - EFS_CG_MIXED_RECURRENCE (the default) runs an iteration as two passes, t = L d and a per-cell update,
//     both with 128-bit accesses when the vectors allow it, and one grid reduction; EFS_CG_MIXED and
//     EFS_CG_REFERENCE fuse d <- beta d + r into the next matrix-vector product (d double-buffered) and
//     recompute L d in the update phase instead of storing it.
// The mixed variants keep p as an FP64 accumulator plus an FP32 increment (see efs_gb300.h).
#include <cfloat>
#include <mutex>

#include "efs_internal.h"
#include "efs_pair.cuh"

namespace efs {

namespace {

// One block of 1024 threads per SM (64 registers a thread): half the grid-barrier arrivals and block partials
// of two 512-thread blocks with the same warps per SM (measured at 256^3: 40.4 against 41.4 ms per solve).
constexpr int SOLVER_THREADS = 1024;
constexpr int SOLVER_MIN_BLOCKS = 1024 / SOLVER_THREADS;      // 64 registers a thread: 1024 threads per SM
constexpr int SOLVER_WARPS = SOLVER_THREADS / 32;

constexpr unsigned long long BARRIER_TIMEOUT_NS = 2000000000ull;   // 2 s per barrier

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned atom_add_release(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Number of grid barriers this block has passed in the current launch (one per block, in shared memory).
__device__ __forceinline__ unsigned& barrier_index() {
    __shared__ unsigned s_index;
    return s_index;
}

// Grid-wide barrier for a cooperative launch (all blocks co-resident).  The arrival counter only counts up
// during a launch: at its k-th barrier a block adds 1 (a release) and waits (acquire loads) until the
// counter reaches k * gridDim.x, compared modulo 2^32.  No block resets anything, so the last arrival
// releases everyone with its own add.  Waiting is bounded by time: a block that waits longer than
// BARRIER_TIMEOUT_NS sets DEV_ERR_BARRIER_TIMEOUT and bar_abort, and every block returns false from then on.
__device__ bool grid_barrier(DevCtl* ctl) {
    __shared__ int s_ok;
    __syncthreads();
    if (gridDim.x == 1) return true;   // one block: the block barrier orders everything (small grids)
    if (threadIdx.x == 0) {
        unsigned& k = barrier_index();
        k += 1u;
        const unsigned target = k * gridDim.x;
        const unsigned old = atom_add_release(&ctl->bar_count, 1u);
        int ok = 1;
        if (old + 1u != target) {
            const unsigned long long t0 = globaltimer_ns();
            unsigned spins = 0;
            while ((int)(ld_acquire(&ctl->bar_count) - target) < 0) {
                if ((++spins & 255u) == 0) {
                    if (*(volatile int*)&ctl->bar_abort) { ok = 0; break; }
                    if (globaltimer_ns() - t0 > BARRIER_TIMEOUT_NS) {
                        atomicOr(&ctl->error, DEV_ERR_BARRIER_TIMEOUT);
                        atomicExch(&ctl->bar_abort, 1);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Dot-product accumulation.  GB300 executes FP64 at a small fraction of its FP32 rate, so sums are kept as an
// unevaluated pair of floats (s + c): every product a*b is split exactly into p + e with one FMA, and every
// addition into s is made exact with TwoSum (Knuth), the rounding error going into c.  The pair carries about
// 48 significant bits.  Threads, warps, blocks and the grid all combine pairs; only the grid total becomes a
// double (s + c).
struct FSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        const float t = s + v;
        const float z = t - s;
        c += (s - (t - z)) + (v - z);
        s = t;
    }
    __device__ __forceinline__ void add_prod(float a, float b) {
        const float p = a * b;
        const float e = fmaf(a, b, -p);
        add(p);
        c += e;
    }
    __device__ __forceinline__ void add_pair(float s2, float c2) {
        add(s2);
        c += c2;
    }
};

__device__ __forceinline__ FSum warp_sum(FSum v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_down_sync(0xffffffffu, v.s, o);
        const float c2 = __shfl_down_sync(0xffffffffu, v.c, o);
        v.add_pair(s2, c2);
    }
    return v;
}

// Sums three pairs over the block (fixed tree: lanes, then warps in order); the result is valid in warp 0.
__device__ __forceinline__ void block_sum3(FSum& a, FSum& b, FSum& c) {
    __shared__ float s_w[6][SOLVER_WARPS];
    a = warp_sum(a);
    b = warp_sum(b);
    c = warp_sum(c);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        s_w[0][warp] = a.s; s_w[1][warp] = a.c;
        s_w[2][warp] = b.s; s_w[3][warp] = b.c;
        s_w[4][warp] = c.s; s_w[5][warp] = c.c;
    }
    __syncthreads();
    if (warp == 0) {
        const bool in = lane < SOLVER_WARPS;
        a.s = in ? s_w[0][lane] : 0.f; a.c = in ? s_w[1][lane] : 0.f;
        b.s = in ? s_w[2][lane] : 0.f; b.c = in ? s_w[3][lane] : 0.f;
        c.s = in ? s_w[4][lane] : 0.f; c.c = in ? s_w[5][lane] : 0.f;
        a = warp_sum(a);
        b = warp_sum(b);
        c = warp_sum(c);
    }
}

// Grid reduction of three pair sums with two alternating partial slots.  Each block stores its three pairs
// (6 floats) in slot `slot`; after the barrier every block adds all blocks' partials in the same fixed order
// (thread k loads block k's, then block_sum3), so every block obtains bit-identical totals and takes the same
// branches.  A slot is rewritten two reductions later, after every block has passed the barrier between.
// Thread 0 also compares the first total with `below` and every thread reads the result as `lt`, so the
// stop test costs the block one integer instead of an FP64 comparison per warp.
struct Reduction {
    float* partials;           // 2 slots x gridDim.x x 6 floats
    int slot;
    double below = 0.0;
    int lt = 0;                // ta < below, for the last run
    __device__ bool run(DevCtl* ctl, FSum a, FSum b, FSum c, double& ta, double& tb, double& tc) {
        __shared__ double s_tot[3];
        __shared__ int s_lt;
        block_sum3(a, b, c);
        float* mine = partials + ((size_t)slot * gridDim.x + blockIdx.x) * 6;
        if (threadIdx.x == 0) {
            mine[0] = a.s; mine[1] = a.c; mine[2] = b.s; mine[3] = b.c; mine[4] = c.s; mine[5] = c.c;
        }
        if (!grid_barrier(ctl)) return false;
        FSum x, y, z;
        // L2 reads (the barrier's acquire orders them after every block's partial), three 8-byte pairs a block
        const float2* src = reinterpret_cast<const float2*>(partials + (size_t)slot * gridDim.x * 6);
        for (int k = threadIdx.x; k < (int)gridDim.x; k += SOLVER_THREADS) {
            const float2 p0 = __ldcg(src + 3 * k), p1 = __ldcg(src + 3 * k + 1), p2 = __ldcg(src + 3 * k + 2);
            x.add_pair(p0.x, p0.y);
            y.add_pair(p1.x, p1.y);
            z.add_pair(p2.x, p2.y);
        }
        block_sum3(x, y, z);
        if (threadIdx.x == 0) {
            s_tot[0] = (double)x.s + (double)x.c;
            s_tot[1] = (double)y.s + (double)y.c;
            s_tot[2] = (double)z.s + (double)z.c;
            s_lt = s_tot[0] < below;
        }
        __syncthreads();
        ta = s_tot[0]; tb = s_tot[1]; tc = s_tot[2];
        lt = s_lt;
        __syncthreads();
        slot ^= 1;
        return true;
    }
    __device__ bool run(DevCtl* ctl, FSum a, FSum b, int n, double& ta, double& tb, double& tc) {
        FSum c;
        c.add((float)n);
        return run(ctl, a, b, c, ta, tb, tc);
    }
};

// A float computed by thread 0 from the grid totals and read by the whole block (keeps the FP64 divisions of
// alpha = rr / dt and beta = rr / rr_old to one thread per block).
__device__ __forceinline__ float block_scalar(float v_thread0) {
    __shared__ float s_scalar;
    if (threadIdx.x == 0) s_scalar = v_thread0;
    __syncthreads();
    const float v = s_scalar;
    __syncthreads();
    return v;
}

// Neighbour order of the reference matrix-vector product: x-1, x+1, y-1, y+1, z+1, z-1 (CGSolver.cpp:489-494)
// and of the Jacobi sweep: x-1, x+1, y-1, y+1, z-1, z+1 (JacobiSolver.cpp:189-194).  rowinfo bits are
// x-1, x+1, y-1, y+1, z-1, z+1.
struct Nb {
    int o[6];
};
// In 2D (D == 1) the z offsets are 0: rowinfo never sets their bits, and the unconditional loads of the hot
// phases then stay within one row of halo.
__device__ __forceinline__ Nb cg_order(const Geo& g) {
    const int oz = (g.D > 1) ? g.WH : 0;
    return Nb{{-1, 1, -g.W, g.W, oz, -oz}};
}
__device__ __forceinline__ int cg_bit(int k) { return (k == 4) ? 5 : (k == 5 ? 4 : k); }

// L x (float, reference rounding) on row i
__device__ __forceinline__ float lap_f(const float* x, uint16_t info, int i, const Nb& nb) {
    float sum = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; k++)
        if (info & (1u << cg_bit(k))) sum += x[i + nb.o[k]];
    return sum - (float)((info >> 8) & 7) * x[i];
}
// L x in FP64 on row i
__device__ __forceinline__ double lap_d(const double* x, uint16_t info, int i, const Nb& nb) {
    double sum = 0.0;
#pragma unroll
    for (int k = 0; k < 6; k++)
        if (info & (1u << cg_bit(k))) sum += x[i + nb.o[k]];
    return sum - (double)((info >> 8) & 7) * x[i];
}

// The mixed variants' pressure accumulator as float pairs (hi + lo, about 48 significant bits) in the memory of
// a.p64, computed on the FP32 pipe with error-free transformations; GB300 runs FP64 at a small fraction of its
// FP32 rate, and the FP64 residual replacement had cost about 70 µs at 256^3 each time.  Converted to doubles in
// place at the end of the solve (efs_download_pressure_fp64).
// b - L x for the pair field x (lap_d's neighbour order), rounded to float
__device__ __forceinline__ float df_resid(float b, const float2 (&xv)[7], uint16_t f) {
    float2 sum = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 6; k++)
        if (f & (1u << cg_bit(k))) sum = df_add(sum, xv[k]);
    const float2 dc = df_mul_k(xv[6], (float)((f >> 8) & 7));
    const float2 lap = df_add(sum, df_neg(dc));
    const float2 t = df_add_f(df_neg(lap), b);
    return __fadd_rn(t.x, t.y);
}

// This block's share of the active chunks, cached in shared memory for the whole solve (the compacted list
// does not change between iterations).
struct Chunks {
    const int* ids;        // shared memory
    const unsigned* mask;  // shared memory: per chunk, bit l set when cell (chunk, lane l) is a matrix row
    int n;
};

// Iterate over this block's chunks: f(cell index) for every in-range cell.
template <typename F>
__device__ __forceinline__ void for_rows(const SolverArgs& a, const Chunks& ch, F f) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < ch.n; c += SOLVER_WARPS) {
        const int i = ch.ids[c] * 32 + lane;
        if (i < a.g.N) f(i);
    }
}

// The two hot phases of a CG iteration process U chunks per warp at once.  Neighbour addresses do not
// depend on rowinfo (they are clamped into the grid and only summed where the row's bits say so), so all
// loads of the U cells are independent and in flight together.
constexpr int U = 2;

// Phase A: d = beta * d_prev + r (it > 0) or d (it == 0), t = L d (reference float rounding), sum d.t.
__device__ __forceinline__ FSum phase_a(const SolverArgs& a, const Chunks& ch, int it, float beta,
                                        const float* __restrict__ dprev, float* __restrict__ dcur, const Nb& nb) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c0 = 0, c1 = ch.n;
    const int N = a.g.N;
    const float* __restrict__ r = a.r;
    FSum acc;
    for (int cb = c0 + warp * U; cb < c1; cb += SOLVER_WARPS * U) {
        int idx[U];
        uint16_t f[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int c = cb + u;
            idx[u] = (c < c1) ? ch.ids[c] * 32 + lane : -1;
        }
#pragma unroll
        for (int u = 0; u < U; u++) f[u] = (idx[u] >= 0 && idx[u] < N) ? a.rowinfo[idx[u]] : 0;
        float xv[U][7], rv[U][7];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = idx[u] < 0 ? 0 : idx[u];   // the vectors carry a halo: i + offset stays allocated
            xv[u][6] = (it == 0) ? dcur[i] : dprev[i];
            if (it != 0) rv[u][6] = r[i];
#pragma unroll
            for (int k = 0; k < 6; k++) {
                const int j = i + nb.o[k];
                xv[u][k] = (it == 0) ? dcur[j] : dprev[j];
                if (it != 0) rv[u][k] = r[j];
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (!(f[u] & 0x8000u)) continue;
            float sum = 0.0f;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if (f[u] & (1u << cg_bit(k))) sum += (it == 0) ? xv[u][k] : xv[u][k] * beta + rv[u][k];
            const float di = (it == 0) ? xv[u][6] : xv[u][6] * beta + rv[u][6];
            const float t = sum - (float)((f[u] >> 8) & 7) * di;
            if (it != 0) dcur[idx[u]] = di;
            acc.add_prod(di, t);
        }
    }
    return acc;
}

// Phase B: x += alpha d (x = e or p), r += (-alpha) L d, sum r.r.
__device__ __forceinline__ FSum phase_b(const SolverArgs& a, const Chunks& ch, float alpha, const float* __restrict__ dcur,
                                        float* __restrict__ x, const Nb& nb) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c0 = 0, c1 = ch.n;
    const int N = a.g.N;
    float* __restrict__ r = a.r;
    FSum acc;
    for (int cb = c0 + warp * U; cb < c1; cb += SOLVER_WARPS * U) {
        int idx[U];
        uint16_t f[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int c = cb + u;
            idx[u] = (c < c1) ? ch.ids[c] * 32 + lane : -1;
        }
#pragma unroll
        for (int u = 0; u < U; u++) f[u] = (idx[u] >= 0 && idx[u] < N) ? a.rowinfo[idx[u]] : 0;
        float dv[U][7], xo[U], ro[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int i = idx[u] < 0 ? 0 : idx[u];
            dv[u][6] = dcur[i];
            xo[u] = x[i];
            ro[u] = r[i];
#pragma unroll
            for (int k = 0; k < 6; k++) dv[u][k] = dcur[i + nb.o[k]];
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (!(f[u] & 0x8000u)) continue;
            float sum = 0.0f;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if (f[u] & (1u << cg_bit(k))) sum += dv[u][k];
            const float t = sum - (float)((f[u] >> 8) & 7) * dv[u][6];
            x[idx[u]] = xo[u] + alpha * dv[u][6];
            const float ri = ro[u] + (-alpha) * t;
            r[idx[u]] = ri;
            acc.add_prod(ri, ri);
        }
    }
    return acc;
}

// EFS_CG_MIXED_RECURRENCE, pass 1: t = L d (reference float rounding), stored; sums d.t and t.t.
constexpr int UA = 4;
__device__ __forceinline__ void phase_t(const SolverArgs& a, const Chunks& ch, const float* __restrict__ d,
                                        float* __restrict__ tout, const Nb& nb, FSum& dt, FSum& tt) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int cb = warp * UA; cb < ch.n; cb += SOLVER_WARPS * UA) {
        int idx[UA];
        bool act[UA];
        uint16_t f[UA];
#pragma unroll
        for (int u = 0; u < UA; u++) {
            const int c = cb + u;
            act[u] = c < ch.n && ((ch.mask[c] >> lane) & 1u);
            idx[u] = act[u] ? ch.ids[c] * 32 + lane : 0;
        }
#pragma unroll
        for (int u = 0; u < UA; u++) f[u] = a.rowinfo[idx[u]];
        // lanes without a row all read cell 0's neighbourhood (inside the vectors' halo): one cached line
        float xv[UA][7];
#pragma unroll
        for (int u = 0; u < UA; u++) {
            const int i = idx[u];
            xv[u][6] = d[i];
#pragma unroll
            for (int k = 0; k < 6; k++) xv[u][k] = d[i + nb.o[k]];
        }
#pragma unroll
        for (int u = 0; u < UA; u++) {
            if (!act[u]) continue;
            float sum = 0.0f;
#pragma unroll
            for (int k = 0; k < 6; k++)
                if (f[u] & (1u << cg_bit(k))) sum += xv[u][k];
            const float t = sum - (float)((f[u] >> 8) & 7) * xv[u][6];
            tout[idx[u]] = t;
            dt.add_prod(xv[u][6], t);
            tt.add_prod(t, t);
        }
    }
}

// Pass 1 with 128-bit accesses, the layout of phase_update4: lane l computes t for cells 4 (l & 7) .. +3 of
// chunk cb + l / 8.  The y and z neighbours are whole groups at +-W and +-W*H; the x neighbours inside a
// group are its own components, across groups the next lane's (warp shuffles), and at a chunk's two ends
// single loads.  A group without a row reads cell 0's neighbourhood and stores nothing.  Same per-cell
// arithmetic and neighbour order as phase_t.  Needs d and t 16-byte aligned, rowinfo 8-byte aligned and W a
// multiple of 4.
#ifndef EFS_SOLVER_UVT
#define EFS_SOLVER_UVT 1
#endif
constexpr int UVT = EFS_SOLVER_UVT;
__device__ __forceinline__ void phase_t4(const SolverArgs& a, const Chunks& ch, const Nb& nb, FSum& dt, FSum& tt) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane >> 3, q = (lane & 7) * 4;
    const float* __restrict__ d = a.d0;
    const float4* __restrict__ d4 = reinterpret_cast<const float4*>(a.d0);
    float4* __restrict__ t4 = reinterpret_cast<float4*>(a.t);
    const uint2* __restrict__ info4 = reinterpret_cast<const uint2*>(a.rowinfo);
    const int oy = nb.o[3] >> 2, oz = nb.o[4] >> 2;   // +W / 4 and +W*H / 4 (0 in 2D)
    for (int cb = warp * 4 * UVT; cb < ch.n; cb += SOLVER_WARPS * 4 * UVT) {
        unsigned m[UVT];
        int i[UVT];
        uint2 fi[UVT];
        float4 xc[UVT], ym[UVT], yp[UVT], zp[UVT], zm[UVT];
        float left[UVT], right[UVT];
#pragma unroll
        for (int v = 0; v < UVT; v++) {
            const int c = cb + 4 * v + sub;
            m[v] = c < ch.n ? (ch.mask[c] >> q) & 0xFu : 0u;
            i[v] = m[v] ? ch.ids[c] * 32 + q : 0;
            const int g = i[v] >> 2;
            fi[v] = info4[g];
            xc[v] = d4[g]; ym[v] = d4[g - oy]; yp[v] = d4[g + oy]; zp[v] = d4[g + oz]; zm[v] = d4[g - oz];
        }
#pragma unroll
        for (int v = 0; v < UVT; v++) {
            left[v] = __shfl_up_sync(0xffffffffu, xc[v].w, 1);
            right[v] = __shfl_down_sync(0xffffffffu, xc[v].x, 1);
            if ((lane & 7) == 0) left[v] = d[i[v] - 1];
            if ((lane & 7) == 7) right[v] = d[i[v] + 4];
        }
#pragma unroll
        for (int v = 0; v < UVT; v++) {
            if (!m[v]) continue;
            const float cx[4] = {xc[v].x, xc[v].y, xc[v].z, xc[v].w};
            const float cym[4] = {ym[v].x, ym[v].y, ym[v].z, ym[v].w}, cyp[4] = {yp[v].x, yp[v].y, yp[v].z, yp[v].w};
            const float czp[4] = {zp[v].x, zp[v].y, zp[v].z, zp[v].w}, czm[4] = {zm[v].x, zm[v].y, zm[v].z, zm[v].w};
            const unsigned fw[4] = {fi[v].x & 0xFFFFu, fi[v].x >> 16, fi[v].y & 0xFFFFu, fi[v].y >> 16};
            float to[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                to[k] = 0.f;
                if (!((m[v] >> k) & 1u)) continue;
                const unsigned f = fw[k];
                const float nv[6] = {k == 0 ? left[v] : cx[k > 0 ? k - 1 : 0], k == 3 ? right[v] : cx[k < 3 ? k + 1 : 3],
                                     cym[k], cyp[k], czp[k], czm[k]};
                float sum = 0.0f;
#pragma unroll
                for (int n = 0; n < 6; n++)
                    if (f & (1u << cg_bit(n))) sum += nv[n];
                const float tv = sum - (float)((f >> 8) & 7) * cx[k];
                to[k] = tv;
                dt.add_prod(cx[k], tv);
                tt.add_prod(tv, tv);
            }
            t4[i[v] >> 2] = make_float4(to[0], to[1], to[2], to[3]);
        }
    }
}

// One Jacobi sweep (JacobiSolver.cpp:176-205) with 128-bit accesses, the layout of phase_t4: dst = (sum of
// the summed neighbours of src - b) / count on rows, neighbours in the reference order x-1, x+1, y-1, y+1,
// z-1, z+1.  Cells that are not rows keep their dst value (per-cell stores in a group that is not all rows).
// Needs src, dst and b 16-byte aligned, rowinfo 8-byte aligned and W a multiple of 4.
__device__ __forceinline__ void jacobi_sweep4(const SolverArgs& a, const Chunks& ch, const float* __restrict__ src,
                                              float* __restrict__ dst) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane >> 3, q = (lane & 7) * 4;
    const float4* __restrict__ s4 = reinterpret_cast<const float4*>(src);
    const float4* __restrict__ b4 = reinterpret_cast<const float4*>(a.b);
    const uint2* __restrict__ info4 = reinterpret_cast<const uint2*>(a.rowinfo);
    const int oy = a.g.W >> 2, oz = (a.g.D > 1) ? (a.g.WH >> 2) : 0;
    for (int cb = warp * 4; cb < ch.n; cb += SOLVER_WARPS * 4) {
        const int c = cb + sub;
        const unsigned m = c < ch.n ? (ch.mask[c] >> q) & 0xFu : 0u;
        const int i = m ? ch.ids[c] * 32 + q : 0;
        const int g = i >> 2;
        const uint2 fi = info4[g];
        const float4 xc = s4[g], ym = s4[g - oy], yp = s4[g + oy], zm = s4[g - oz], zp = s4[g + oz], bv = b4[g];
        float left = __shfl_up_sync(0xffffffffu, xc.w, 1);
        float right = __shfl_down_sync(0xffffffffu, xc.x, 1);
        if ((lane & 7) == 0) left = src[i - 1];
        if ((lane & 7) == 7) right = src[i + 4];
        if (!m) continue;
        const float cx[4] = {xc.x, xc.y, xc.z, xc.w}, cb4[4] = {bv.x, bv.y, bv.z, bv.w};
        const float cym[4] = {ym.x, ym.y, ym.z, ym.w}, cyp[4] = {yp.x, yp.y, yp.z, yp.w};
        const float czm[4] = {zm.x, zm.y, zm.z, zm.w}, czp[4] = {zp.x, zp.y, zp.z, zp.w};
        const unsigned fw[4] = {fi.x & 0xFFFFu, fi.x >> 16, fi.y & 0xFFFFu, fi.y >> 16};
        float out[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const unsigned f = fw[k];
            const float nv[6] = {k == 0 ? left : cx[k > 0 ? k - 1 : 0], k == 3 ? right : cx[k < 3 ? k + 1 : 3],
                                 cym[k], cyp[k], czm[k], czp[k]};
            float sum = 0.0f;
#pragma unroll
            for (int n = 0; n < 6; n++)
                if (f & (1u << n)) sum += nv[n];
            const int cnt = (f >> 8) & 7;
            out[k] = cnt > 0 ? (sum - cb4[k]) / (float)cnt : 0.0f;
        }
        if (m == 0xFu) {
            reinterpret_cast<float4*>(dst)[g] = make_float4(out[0], out[1], out[2], out[3]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if ((m >> k) & 1u) dst[i + k] = out[k];
        }
    }
}

// EFS_CG_MIXED_RECURRENCE, pass 2 (per cell, no neighbours): what = 3: e += alpha d, r += -alpha t,
// d = d beta + r (sums r.r); what = 1: only e += alpha d; what = 2: only d = d beta + r.
template <int WHAT>
__device__ __forceinline__ FSum phase_update(const SolverArgs& a, const Chunks& ch, float alpha, float beta) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* __restrict__ d = a.d0;
    float* __restrict__ r = a.r;
    float* __restrict__ e = a.e;
    const float* __restrict__ t = a.t;
    FSum acc;
    for (int cb = warp * UA; cb < ch.n; cb += SOLVER_WARPS * UA) {
        int idx[UA];
        bool act[UA];
#pragma unroll
        for (int u = 0; u < UA; u++) {
            const int c = cb + u;
            act[u] = c < ch.n && ((ch.mask[c] >> lane) & 1u);
            idx[u] = act[u] ? ch.ids[c] * 32 + lane : 0;
        }
        float dv[UA], tv[UA], rv[UA], ev[UA];
#pragma unroll
        for (int u = 0; u < UA; u++) {
            const int i = idx[u];   // 0 for lanes without a row: one cached line
            dv[u] = d[i];
            if (WHAT & 1) { tv[u] = t[i]; ev[u] = e[i]; }
            rv[u] = r[i];
        }
#pragma unroll
        for (int u = 0; u < UA; u++) {
            if (!act[u]) continue;
            const int i = idx[u];
            if (WHAT & 1) e[i] = ev[u] + alpha * dv[u];
            if (WHAT == 3) {
                const float rn = rv[u] + (-alpha) * tv[u];
                r[i] = rn;
                d[i] = dv[u] * beta + rn;
                acc.add_prod(rn, rn);
            } else if (WHAT == 2) {
                d[i] = dv[u] * beta + rv[u];
            }
        }
    }
    return acc;
}

// Pass 2 (what = 3) with 128-bit accesses: lane l handles cells 4 (l & 7) .. 4 (l & 7) + 3 of chunk
// cb + l / 8, so one warp instruction covers four chunks.  A group of four cells without a row reads cell 0's
// group (one cached line) and stores nothing; in a group with rows, the cells that are not rows are written back
// as read.  Same per-cell arithmetic as phase_update<3>.  Needs d, t, r and e 16-byte aligned.
#ifndef EFS_SOLVER_UV
#define EFS_SOLVER_UV 2
#endif
constexpr int UV = EFS_SOLVER_UV;
template <int WHAT = 3>
__device__ __forceinline__ FSum phase_update4(const SolverArgs& a, const Chunks& ch, float alpha, float beta) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = lane >> 3, q = (lane & 7) * 4;
    float4* __restrict__ d = reinterpret_cast<float4*>(a.d0);
    float4* __restrict__ r = reinterpret_cast<float4*>(a.r);
    float4* __restrict__ e = reinterpret_cast<float4*>(a.e);
    const float4* __restrict__ t = reinterpret_cast<const float4*>(a.t);
    FSum acc;
    for (int cb = warp * UV * 4; cb < ch.n; cb += SOLVER_WARPS * UV * 4) {
        int idx[UV];
        unsigned m[UV];
#pragma unroll
        for (int v = 0; v < UV; v++) {
            const int c = cb + v * 4 + sub;
            m[v] = c < ch.n ? (ch.mask[c] >> q) & 0xFu : 0u;
            idx[v] = m[v] ? (ch.ids[c] * 32 + q) >> 2 : 0;
        }
        float4 dv[UV], tv[UV], rv[UV], ev[UV];
#pragma unroll
        for (int v = 0; v < UV; v++) {
            dv[v] = d[idx[v]];
            if (WHAT == 3) tv[v] = t[idx[v]];
            if (WHAT & 2) rv[v] = r[idx[v]];
            if (WHAT & 1) ev[v] = e[idx[v]];
        }
#pragma unroll
        for (int v = 0; v < UV; v++) {
            if (!m[v]) continue;
            float* dd = &dv[v].x;
            float* tt = &tv[v].x;
            float* rr = &rv[v].x;
            float* ee = &ev[v].x;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                if (!((m[v] >> k) & 1u)) continue;
                if (WHAT & 1) ee[k] = ee[k] + alpha * dd[k];
                if (WHAT == 3) {
                    const float rn = rr[k] + (-alpha) * tt[k];
                    rr[k] = rn;
                    dd[k] = dd[k] * beta + rn;
                    acc.add_prod(rn, rn);
                } else if (WHAT == 2) {
                    dd[k] = dd[k] * beta + rr[k];
                }
            }
            if (WHAT & 1) e[idx[v]] = ev[v];
            if (WHAT == 3) r[idx[v]] = rv[v];
            if (WHAT & 2) d[idx[v]] = dv[v];
        }
    }
    return acc;
}

// Residual replacement of the mixed-precision variants, in rounds of several chunks per warp whose loads do not
// depend on rowinfo (a chunk at a time, each row's loads waiting for its rowinfo, made every replacement a
// chain of dependent L2 round trips: about 145 µs at 256^3, 16 times a solve): p += e, e = 0, then r = b - L p
// with the neighbours summed in order, p as float pairs (df_resid).
#ifndef EFS_SOLVER_UR
#define EFS_SOLVER_UR 1
#endif
constexpr int UR = EFS_SOLVER_UR;   // chunks per round of the FP64 residual (7 doubles a row: more would spill)
__device__ __forceinline__ void fold_rows(const SolverArgs& a, const Chunks& ch) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int cb = warp * UA; cb < ch.n; cb += SOLVER_WARPS * UA) {
        int idx[UA];
        bool act[UA];
#pragma unroll
        for (int u = 0; u < UA; u++) {
            const int c = cb + u;
            act[u] = c < ch.n && ((ch.mask[c] >> lane) & 1u);
            idx[u] = act[u] ? ch.ids[c] * 32 + lane : 0;
        }
        float2* pp = reinterpret_cast<float2*>(a.p64);
        float2 pv[UA];
        float ev[UA];
#pragma unroll
        for (int u = 0; u < UA; u++) { pv[u] = pp[idx[u]]; ev[u] = a.e[idx[u]]; }
#pragma unroll
        for (int u = 0; u < UA; u++) {
            if (!act[u]) continue;
            pp[idx[u]] = df_add_f(pv[u], ev[u]);
            a.e[idx[u]] = 0.f;
        }
    }
}
__device__ __forceinline__ FSum residual_rows(const SolverArgs& a, const Chunks& ch, const Nb& nb) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    FSum acc;
    for (int cb = warp * UR; cb < ch.n; cb += SOLVER_WARPS * UR) {
        int idx[UR];
        bool act[UR];
#pragma unroll
        for (int u = 0; u < UR; u++) {
            const int c = cb + u;
            act[u] = c < ch.n && ((ch.mask[c] >> lane) & 1u);
            idx[u] = act[u] ? ch.ids[c] * 32 + lane : 0;
        }
        const float2* pp = reinterpret_cast<const float2*>(a.p64);
        uint16_t f[UR];
        float bv[UR];
        float2 xv[UR][7];
#pragma unroll
        for (int u = 0; u < UR; u++) {
            const int i = idx[u];
            f[u] = a.rowinfo[i];
            bv[u] = a.b[i];
            xv[u][6] = pp[i];
#pragma unroll
            for (int k = 0; k < 6; k++) xv[u][k] = pp[i + nb.o[k]];
        }
#pragma unroll
        for (int u = 0; u < UR; u++) {
            if (!act[u]) continue;
            const float ri = df_resid(bv[u], xv[u], f[u]);
            a.r[idx[u]] = ri;
            acc.add_prod(ri, ri);
        }
    }
    return acc;
}

// Two floats and a flag computed by thread 0 and read by the whole block.
__device__ __forceinline__ void block_scalars(float& v0, float& v1, int* flag = nullptr) {
    __shared__ float s2[2];
    __shared__ int s_flag;
    if (threadIdx.x == 0) { s2[0] = v0; s2[1] = v1; s_flag = flag ? *flag : 0; }
    __syncthreads();
    v0 = s2[0];
    v1 = s2[1];
    if (flag) *flag = s_flag;
    __syncthreads();
}

// A per-thread FP64 sum as a float pair (about 48 significant bits), for the pair reductions.
__device__ __forceinline__ FSum pair_of(double v) {
    FSum f;
    f.s = (float)v;
    f.c = (float)(v - (double)f.s);
    return f;
}

// EFS_CG_FP64: the reference CG iteration (CGSolver.cpp:416-465: p0 = b, r = b - L p, d = r; true residual
// when (i & 63) == 0; stop on r.r < threshold) with p, r, d and t = L d all in FP64 and the threshold
// tol_rel^2 b.b kept in FP64.  A study solver: it gives the FP64 pressure of the same right-hand side that the
// FP32 solvers are measured against.  Rows outside the matrix keep p = b, as in the other variants.
__device__ __forceinline__ void cg_fp64(const SolverArgs& a, const Chunks& ch, const Nb& nb, Reduction& red, int M) {
    DevCtl* ctl = a.ctl;
    const float* b = a.b;
    const uint16_t* info = a.rowinfo;
    double* p = a.p64;
    double* r = a.r64;
    double* d = a.d64;
    double* t = a.t64;
    double u1, u2, rr, bb, nrows;
    for_rows(a, ch, [&](int i) { p[i] = (double)b[i]; });
    if (!grid_barrier(ctl)) return;
    {
        double acc_rr = 0.0, acc_bb = 0.0;
        int rows = 0;
        for_rows(a, ch, [&](int i) {
            const double bi = (double)b[i];
            acc_bb += bi * bi;
            const uint16_t f = info[i];
            if (!(f & 0x8000u)) return;
            rows += 1;
            const double ri = bi - lap_d(p, f, i, nb);
            r[i] = ri;
            d[i] = ri;
            acc_rr += ri * ri;
        });
        if (!red.run(ctl, pair_of(acc_rr), pair_of(acc_bb), rows, rr, bb, nrows)) return;
    }
    const double thr = a.tol_rel > 0 ? (double)a.tol_rel * (double)a.tol_rel * bb : (double)a.solver_threshold;
    int conv = rr < thr, it = 0;
    if (!conv) {
        for (it = 0; it < a.max_steps; it++) {
            double acc = 0.0;
            for_rows(a, ch, [&](int i) {
                const uint16_t f = info[i];
                if (!(f & 0x8000u)) return;
                const double ti = lap_d(d, f, i, nb);
                t[i] = ti;
                acc += d[i] * ti;
            });
            double dt;
            if (!red.run(ctl, pair_of(acc), FSum(), 0, dt, u1, u2)) return;
            if (!(dt != 0.0) || !isfinite(rr / dt)) break;   // breakdown: stop, not converged
            const double alpha = rr / dt;
            const double old = rr;
            acc = 0.0;
            if (it & 0x3F) {
                for_rows(a, ch, [&](int i) {
                    if (!(info[i] & 0x8000u)) return;
                    p[i] += alpha * d[i];
                    const double ri = r[i] - alpha * t[i];
                    r[i] = ri;
                    acc += ri * ri;
                });
            } else {
                for_rows(a, ch, [&](int i) {
                    if (info[i] & 0x8000u) p[i] += alpha * d[i];
                });
                if (!grid_barrier(ctl)) return;
                for_rows(a, ch, [&](int i) {
                    const uint16_t f = info[i];
                    if (!(f & 0x8000u)) return;
                    const double ri = (double)b[i] - lap_d(p, f, i, nb);
                    r[i] = ri;
                    acc += ri * ri;
                });
            }
            if (!red.run(ctl, pair_of(acc), FSum(), 0, rr, u1, u2)) return;
            if (rr < thr) { conv = 1; break; }
            const double beta = rr / old;
            for_rows(a, ch, [&](int i) {
                if (info[i] & 0x8000u) d[i] = r[i] + beta * d[i];
            });
            if (!grid_barrier(ctl)) return;
        }
        it += 1;
    }
    for_rows(a, ch, [&](int i) {
        if (info[i] & 0x8000u) a.p[i] = (float)p[i];
    });
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->converged = conv;
        ctl->iterations = it;
        ctl->rr = rr;
        ctl->bb = bb;
        ctl->thr = thr;
        ctl->active_chunks = M;
        ctl->active_cells = (long long)nrows;
        ctl->total_iterations += it;
        ctl->solves += 1;
        ctl->precond_iterations = 0;
        ctl->sum_iter_rows += (double)it * nrows;
        ctl->sum_rows += nrows;
    }
}

// Start of both solver kernels: ordered compaction of the active chunks into a.chunk_list (two grid
// barriers), then this block's share of the list cached in shared memory.  M = active chunks.
__device__ __forceinline__ bool solver_prologue(const SolverArgs& a, Chunks& ch, int& M) {
    if (threadIdx.x == 0) barrier_index() = 0u;
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
    if (!grid_barrier(a.ctl)) return false;
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
    M = s_total;
    if (!grid_barrier(a.ctl)) return false;
    extern __shared__ int s_chunks[];
    {
        const int per = (M + gridDim.x - 1) / gridDim.x;
        const int c0 = blockIdx.x * per, c1 = min(M, c0 + per);
        ch.ids = s_chunks;
        ch.n = max(0, c1 - c0);
        for (int k = threadIdx.x; k < ch.n; k += SOLVER_THREADS) s_chunks[k] = ((volatile int*)a.chunk_list)[c0 + k];
        __syncthreads();
        // Row lanes of every chunk (rowinfo is fixed during the solve).  The hot passes load and store only
        // these lanes, so the sectors of a chunk that hold no row are never fetched: a liquid region whose x
        // extent ends inside a chunk costs its touched 32-byte sectors, not the whole chunk.
        unsigned* s_mask = reinterpret_cast<unsigned*>(s_chunks + ch.n);
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int c = warp; c < ch.n; c += SOLVER_WARPS) {
            const int i = s_chunks[c] * 32 + lane;
            const bool row = i < a.g.N && (a.rowinfo[i] & 0x8000u);
            const unsigned m = __ballot_sync(0xffffffffu, row);
            if (lane == 0) s_mask[c] = m;
        }
        ch.mask = s_mask;
        __syncthreads();
    }

    return true;
}

__global__ void __launch_bounds__(SOLVER_THREADS, SOLVER_MIN_BLOCKS) k_solver(SolverArgs a) {
    DevCtl* ctl = a.ctl;
    Chunks ch;
    int M = 0;
    if (!solver_prologue(a, ch, M)) return;
    const Nb nb = cg_order(a.g);
    const float* __restrict__ b = a.b;
    const uint16_t* __restrict__ info = a.rowinfo;

    Reduction red{reinterpret_cast<float*>(a.partials), 0};
    double u1, u2;

    // ---- Jacobi ---------------------------------------------------------------------------------------
    if (a.solver == EFS_SOLVER_JACOBI) {
        const int iters = a.max_steps / 2;
        const int jo[6] = {-1, 1, -a.g.W, a.g.W, -a.g.WH, a.g.WH};
        int rows = 0;
        for_rows(a, ch, [&](int i) { if (info[i] & 0x8000u) rows += 1; });
        double nrows;
        if (!red.run(ctl, FSum(), FSum(), rows, u1, u2, nrows)) return;
        const bool vec4 = ((reinterpret_cast<uintptr_t>(a.p) | reinterpret_cast<uintptr_t>(a.e) |
                            reinterpret_cast<uintptr_t>(a.b)) & 15u) == 0 &&
                          (reinterpret_cast<uintptr_t>(a.rowinfo) & 7u) == 0 && (a.g.W & 3) == 0;
        for (int it = 0; it < iters; it++) {
            const float* src = (it & 1) ? a.e : a.p;
            float* dst = (it & 1) ? a.p : a.e;
            if (vec4) {
                jacobi_sweep4(a, ch, src, dst);
                if (!grid_barrier(ctl)) return;
                continue;
            }
            for_rows(a, ch, [&](int i) {
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
            for_rows(a, ch, [&](int i) { if (info[i] & 0x8000u) a.p[i] = a.e[i]; });
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctl->converged = 1; ctl->iterations = iters; ctl->rr = 0; ctl->bb = 0; ctl->thr = 0;
            ctl->active_chunks = M; ctl->active_cells = (long long)nrows;
            ctl->total_iterations += iters; ctl->solves += 1; ctl->precond_iterations = 0;
            ctl->sum_iter_rows += (double)iters * nrows; ctl->sum_rows += nrows;
        }
        return;
    }

    // ---- CG ---------------------------------------------------------------------------------------------
    const bool mixed = a.cg_variant == EFS_CG_MIXED || a.cg_variant == EFS_CG_MIXED_RECURRENCE;
    float* __restrict__ r = a.r;
    float* __restrict__ e = a.e;
    double* __restrict__ p64 = a.p64;
    float* __restrict__ p = a.p;

    // initial residual r = b - L p0 with p0 = b (CGSolver.cpp:425-434); d = r
    double rr, bb, nrows;
    {
        FSum rr_p, bb_p;
        int rows = 0;
        for_rows(a, ch, [&](int i) {
            const float bi = b[i];
            bb_p.add_prod(bi, bi);
            const uint16_t f = info[i];
            if (!(f & 0x8000u)) return;
            rows += 1;
            float ri;
            if (mixed) {
                reinterpret_cast<float2*>(p64)[i] = make_float2(bi, 0.f);
                e[i] = 0.f;
                float2 bv[7];
#pragma unroll
                for (int k = 0; k < 6; k++) bv[k] = make_float2(b[i + nb.o[k]], 0.f);
                bv[6] = make_float2(bi, 0.f);
                ri = df_resid(bi, bv, f);
            } else {
                ri = bi - lap_f(b, f, i, nb);
            }
            r[i] = ri;
            a.d0[i] = ri;
            rr_p.add_prod(ri, ri);
        });
        if (!red.run(ctl, rr_p, bb_p, rows, rr, bb, nrows)) return;
    }
    float thr_f;
    if (a.thr_dev) {
        thr_f = (float)*a.thr_dev;
    } else if (a.tol_rel > 0) {
        thr_f = (float)((double)a.tol_rel * (double)a.tol_rel * bb);
        if (!(thr_f > 0)) thr_f = FLT_MIN;
    } else {
        thr_f = a.solver_threshold;
    }
    const double thr = (double)thr_f;
    red.below = thr;

    // residual recomputation (CGSolver.cpp:447-451): fold e into the pair accumulator and r = b - L p in float
    // pairs (mixed), or
    // r = b - L p in FP32 (reference)
    auto replace = [&](double& rr_out) -> bool {
        // the fold reads e with its own chunk-to-warp mapping: every warp's update of e comes first
        __syncthreads();
        if (mixed) fold_rows(a, ch);
        if (!grid_barrier(ctl)) return false;
        FSum rp;
        if (mixed) {
            rp = residual_rows(a, ch, nb);
        } else {
            for_rows(a, ch, [&](int i) {
                const uint16_t f = info[i];
                if (!(f & 0x8000u)) return;
                const float ri = b[i] - lap_f(p, f, i, nb);
                r[i] = ri;
                rp.add_prod(ri, ri);
            });
        }
        return red.run(ctl, rp, FSum(), 0, rr_out, u1, u2);
    };

    int conv = rr < thr;
    int iters = 0;
    float beta = 0.f;
    if (!conv && a.cg_variant == EFS_CG_MIXED_RECURRENCE) {
        // Pass 1 (t = L d; d.t, t.t) and pass 2 (e, r, d per cell; exact r.r) alternate.  The r.r of pass 2
        // only feeds the stop test, so its block partial travels with the next pass 1's reduction: one
        // reduction and one plain barrier per iteration.  The stop test of iteration k is therefore taken
        // after the pass 1 of iteration k+1, whose t is then unused; e, r and p are unaffected.
        double dt, tt, u3;
        // 128-bit passes when the vectors allow them (always for the context's own allocations)
        const bool vec4 = ((reinterpret_cast<uintptr_t>(a.d0) | reinterpret_cast<uintptr_t>(a.r) |
                            reinterpret_cast<uintptr_t>(a.e) | reinterpret_cast<uintptr_t>(a.t)) & 15u) == 0 &&
                          (reinterpret_cast<uintptr_t>(a.rowinfo) & 7u) == 0 && (a.g.W & 3) == 0;
        {
            FSum dtp, ttp;
            if (vec4) phase_t4(a, ch, nb, dtp, ttp); else phase_t(a, ch, a.d0, a.t, nb, dtp, ttp);
            if (!red.run(ctl, FSum(), dtp, ttp, u3, dt, tt)) return;
        }
        int it;
        for (it = 0; it < a.max_steps; it++) {
            // The FP64 scalar work of an iteration is thread 0's: GB300 runs FP64 at a small fraction of its
            // FP32 rate, and a division in every thread cost the whole block microseconds per iteration.
            float alpha = 0.f, bet = 0.f;
            int recur = 0;
            if (threadIdx.x == 0) {
                const double ad = div_fast(rr, dt);
                if (!(dt != 0.0) || !isfinite(ad)) {
                    recur = -1;   // breakdown (a singular block: a liquid region with no air neighbour)
                } else {
                    alpha = (float)ad;
                    const double est = ad * ad * tt * div_fast(1.0, rr) - 1.0;   // r'.r' / r.r from the recurrence
                    recur = (it & 0x3F) && est > 0.0;
                    bet = (float)est;
                }
            }
            block_scalars(alpha, bet, &recur);
            if (recur < 0) break;   // stop, not converged
            const double old = rr;
            if (recur) {
                const FSum rp = vec4 ? phase_update4(a, ch, alpha, bet) : phase_update<3>(a, ch, alpha, bet);
                if (!grid_barrier(ctl)) return;
                FSum dtp, ttp;
                if (vec4) phase_t4(a, ch, nb, dtp, ttp); else phase_t(a, ch, a.d0, a.t, nb, dtp, ttp);
                if (!red.run(ctl, rp, dtp, ttp, rr, dt, tt)) return;
                if (red.lt) {
                    // confirm on the recomputed residual; if that is above the threshold, the direction (formed
                    // from the recurrence residual, so r.d != r.r now) restarts from it: d = r, t = L d
                    if (!replace(rr)) return;
                    if (red.lt) { conv = 1; break; }
                    for_rows(a, ch, [&](int i) { if (info[i] & 0x8000u) a.d0[i] = r[i]; });
                    if (!grid_barrier(ctl)) return;
                    FSum dtp2, ttp2;
                    if (vec4) phase_t4(a, ch, nb, dtp2, ttp2); else phase_t(a, ch, a.d0, a.t, nb, dtp2, ttp2);
                    if (!red.run(ctl, FSum(), dtp2, ttp2, u3, dt, tt)) return;
                }
            } else {
                if (vec4) phase_update4<1>(a, ch, alpha, 0.f); else phase_update<1>(a, ch, alpha, 0.f);
                __syncthreads();   // replace() folds e with another cell-to-thread mapping
                if (!replace(rr)) return;
                if (red.lt) { conv = 1; break; }
                float b2 = 0.f, unused = 0.f;
                if (threadIdx.x == 0) b2 = (float)(rr / old);
                block_scalars(b2, unused);
                if (vec4) phase_update4<2>(a, ch, 0.f, b2); else phase_update<2>(a, ch, 0.f, b2);
                if (!grid_barrier(ctl)) return;
                FSum dtp, ttp;
                if (vec4) phase_t4(a, ch, nb, dtp, ttp); else phase_t(a, ch, a.d0, a.t, nb, dtp, ttp);
                if (!red.run(ctl, FSum(), dtp, ttp, u3, dt, tt)) return;
            }
        }
        iters = it + 1;
    } else if (!conv) {
        int it;
        for (it = 0; it < a.max_steps; it++) {
            float* dcur = (it & 1) ? a.d1 : a.d0;
            const float* dprev = (it & 1) ? a.d0 : a.d1;
            // A: d = beta d + r (it > 0; CGSolver.cpp:458-460), t = L d, d.t
            const FSum dt_p = phase_a(a, ch, it, beta, dprev, dcur, nb);
            double dt;
            if (!red.run(ctl, dt_p, FSum(), 0, dt, u1, u2)) return;
            float alpha = 0.f, unused = 0.f;
            int brk = 0;
            if (threadIdx.x == 0) {
                const double q = rr / dt;
                if (!(dt != 0.0) || !isfinite(q)) brk = 1; else alpha = (float)q;
            }
            block_scalars(alpha, unused, &brk);
            if (brk) break;   // breakdown: stop, not converged
            // B: p (or e) += alpha d; r -= alpha L d, or the true residual every 64 iterations (:442-451)
            const double old = rr;
            bool replaced = false;
            if (it & 0x3F) {
                const FSum rp = phase_b(a, ch, alpha, dcur, mixed ? e : p, nb);
                if (!red.run(ctl, rp, FSum(), 0, rr, u1, u2)) return;
            } else {
                for_rows(a, ch, [&](int i) {
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
            beta = block_scalar(threadIdx.x == 0 ? (float)(rr / old) : 0.f);
        }
        iters = it + 1;
    }
    if (mixed) {
        // fold the increment and convert the pairs in place: p64 then holds the FP64 solution
        // (efs_download_pressure_fp64)
        for_rows(a, ch, [&](int i) {
            if (!(info[i] & 0x8000u)) return;
            const float2 pv = reinterpret_cast<const float2*>(p64)[i];
            const double v = ((double)pv.x + (double)pv.y) + (double)e[i];
            p64[i] = v;
            e[i] = 0.f;
            p[i] = (float)v;
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
        ctl->precond_iterations = 0;
        ctl->sum_iter_rows += (double)iters * nrows;
        ctl->sum_rows += nrows;
    }
}

// EFS_CG_FP64 runs in its own kernel so that the study solver does not weigh on k_solver's registers.
__global__ void __launch_bounds__(SOLVER_THREADS, SOLVER_MIN_BLOCKS) k_solver_fp64(SolverArgs a) {
    Chunks ch;
    int M = 0;
    if (!solver_prologue(a, ch, M)) return;
    Reduction red{reinterpret_cast<float*>(a.partials), 0};
    cg_fp64(a, ch, cg_order(a.g), red, M);
}

// The dynamic shared-memory limit is an attribute of the kernel for the whole process: raise it when a grid
// needs more than the 48 KB default, and never lower it (other contexts may need the larger value).
std::mutex g_smem_mutex;
size_t g_smem_limit = 48 * 1024;

// The shared-memory carveout is set so that two blocks with this dynamic size fit on one SM (the driver's
// default carveout held only one block of the 256^3 chunk cache); it too only rises.
int g_carveout_pct = 0;

cudaError_t ensure_solver_smem(size_t bytes) {
    std::lock_guard<std::mutex> lock(g_smem_mutex);
    const size_t per_block = bytes + 4096 + 1024;   // dynamic + static + reserved, rounded up
    const int pct = (int)std::min<size_t>(100, (2 * per_block * 100 + 228 * 1024 - 1) / (228 * 1024) + 1);
    if (pct > g_carveout_pct) {
        for (auto k : {k_solver, k_solver_fp64}) {
            cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
            if (e != cudaSuccess) return e;
        }
        g_carveout_pct = pct;
    }
    if (bytes <= g_smem_limit) return cudaSuccess;
    for (auto k : {k_solver, k_solver_fp64}) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e != cudaSuccess) return e;
    }
    g_smem_limit = bytes;
    return cudaSuccess;
}

}  // namespace

// Blocks per SM and the chunk-cache size: two blocks per SM when two blocks, each caching its share of the
// chunks, fit (registers, threads, shared memory); otherwise one.  Small grids get fewer blocks (about four
// chunks per warp) so barrier cost stays proportionate.
cudaError_t solver_shape(int n_chunks, int sm_count, int* blocks_out, size_t* smem_out) {
    int blocks = sm_count;
    for (int bps = 2; bps >= 1; bps--) {
        const size_t smem = (size_t)((n_chunks + bps * sm_count - 1) / (bps * sm_count)) * 2 * sizeof(int);
        cudaError_t e = ensure_solver_smem(smem);
        if (e != cudaSuccess) return e;
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_solver, SOLVER_THREADS, smem);
        if (e != cudaSuccess) return e;
        if (occ >= bps) { blocks = bps * sm_count; break; }
        if (bps == 1 && occ < 1) return cudaErrorLaunchOutOfResources;
    }
    // Small grids get fewer blocks (about four chunks per warp) so that barrier cost stays proportionate, and
    // one block (block barriers instead of grid barriers) up to kOneBlockChunks chunks: at 2D 128^2 (512 chunks)
    // a pass of one block's 32 warps takes less than a grid barrier of four blocks.
    constexpr int kOneBlockChunks = 640;
    const int want = n_chunks <= kOneBlockChunks ? 1 : (n_chunks + SOLVER_WARPS * 4 - 1) / (SOLVER_WARPS * 4);
    blocks = std::max(1, std::min(blocks, want));
    *blocks_out = blocks;
    *smem_out = (size_t)((n_chunks + blocks - 1) / blocks) * 2 * sizeof(int);   // chunk ids and row masks
    return ensure_solver_smem(*smem_out);
}

cudaError_t solver_configure(efs_ctx* c) {
    const int n_chunks = (c->g.N + 31) / 32;
    c->solver_threads = SOLVER_THREADS;
    return solver_shape(n_chunks, c->sm_count, &c->solver_blocks, &c->solver_smem);
}

namespace {
SolverArgs context_solver_args(efs_ctx* c) {
    SolverArgs a{};
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
    a.t = c->t;
    a.r64 = c->r64;
    a.d64 = c->d64;
    a.t64 = c->t64;
    a.partials = c->partials;
    a.ctl = c->ctl;
    a.thr_dev = nullptr;
    return a;
}

cudaError_t launch_context_solver(efs_ctx* c, const SolverArgs& a, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c->solver_blocks);
    cfg.blockDim = dim3(SOLVER_THREADS);
    cfg.dynamicSmemBytes = c->solver_smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // a fresh barrier for this launch (a previous launch may have aborted mid-barrier)
    cudaError_t e = cudaMemsetAsync(c->ctl, 0, 2 * sizeof(int), st);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, a.cg_variant == EFS_CG_FP64 && a.solver == EFS_SOLVER_CG ? k_solver_fp64 : k_solver, a);
}
}  // namespace

cudaError_t launch_solver(efs_ctx* c) {
    if (c->prm.solver == EFS_SOLVER_FCG_UNET) return fcg_solve(c);
    return launch_context_solver(c, context_solver_args(c), c->stream);
}

cudaError_t launch_solver_on(efs_ctx* c, const float* b, const double* thr_dev, cudaStream_t st) {
    SolverArgs a = context_solver_args(c);
    a.solver = EFS_SOLVER_CG;
    a.cg_variant = EFS_CG_MIXED_RECURRENCE;
    a.b = b;
    a.thr_dev = thr_dev;
    return launch_context_solver(c, a, st);
}

// Launch shape of the solver for a grid of n_chunks 32-cell chunks (the same rule as solver_configure),
// for callers that hold their own SolverArgs.
cudaError_t solver_launch_shape(int n_chunks, int sm_count, int* blocks_out, size_t* smem_out) {
    return solver_shape(n_chunks, sm_count, blocks_out, smem_out);
}

// Cooperative launch of the solver with caller-provided arguments and shape (no allocation).
cudaError_t launch_solver_args(const SolverArgs& a, int blocks, size_t smem, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(SOLVER_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_solver, a);
}

}  // namespace efs
