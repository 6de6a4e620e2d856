// efs_batch.cu — many independent 2D scenes of uneven sizes advanced together (efs_batch_* entry points).
//
// Every scene is a full reference 2D simulation (CPUSimulator2D: the seven stages of ISimulator::update,
// include/simulation/simulator/ISimulator.h:12-38, and CGSolverCPU2D::solve, src/simulation/solver/
// CGSolver.cpp:32-111) with its own grid size and cell size; the batch shares one set of parameters except
// GRAVITY_FORCE, which is per scene (9.81 / dx in cells/s^2).  One step of all scenes is one CUDA graph: each
// stage kernel is a single persistent launch over a table of (scene, block) entries (efs_stages.cu), and the
// pressure solves are one persistent launch in which each block, or each thread-block cluster, solves whole
// scenes (scenes in descending size), so no scene waits on another and no grid-wide barrier is needed.  The
// tile shape of the stage kernels, their blocks per SM and the solver's block and cluster size are chosen by
// efs_batch_autotune from timed trial steps.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include <cooperative_groups.h>

#include "efs_batch.h"

namespace cg = cooperative_groups;

using namespace efs;

struct efs_batch {
    int n = 0;
    efs_params prm{};
    int device = 0, sm_count = 0;
    cudaStream_t stream = nullptr;
    std::vector<BScene> sc;
    BScene* d_sc = nullptr;
    std::vector<int> order;            // scenes by descending cell count (solver assignment)
    int* d_order = nullptr;
    long long total = 0;
    BFields F{};
    double* p64 = nullptr;
    float *r = nullptr, *d = nullptr, *t = nullptr, *e = nullptr;
    std::vector<void*> allocs;
    BEntry* d_tab[5] = {};
    int ntab[5] = {};
    // tuning
    int bx = 32, by = 8, bps = 4, cg_threads = 512, cg_cluster = 1;
    int cg_clusters_max = 0;           // co-resident clusters of k_batch_cg_cluster at the current tuning
    unsigned* fetch = nullptr;         // k_batch_cg*: next scene
    cudaGraphExec_t graph = nullptr;
    cudaGraph_t graph_def = nullptr;
    unsigned graph_stages = 0;
    int graph_kernels = 0;
    int64_t frames = 0;
    std::string err;
};

namespace {

std::string g_batch_create_error;

int bfail(efs_batch* b, int status, const std::string& msg) {
    if (b) b->err = msg; else g_batch_create_error = msg;
    return status;
}
int bcuda(efs_batch* b, cudaError_t e, const char* what) {
    return bfail(b, EFS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define BCK(call, what) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return bcuda(b, e_, what); } while (0)

template <typename T>
cudaError_t balloc(efs_batch* b, T** p, long long count) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), (size_t)std::max<long long>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    b->allocs.push_back(*p);
    return cudaMemset(*p, 0, (size_t)std::max<long long>(count, 1) * sizeof(T));
}

// ---- group-level CG: EFS_CG_MIXED_RECURRENCE on one scene per block or per thread-block cluster
// (CGSolver.cpp:32-83 with the mixed precision and recurrence of the persistent solver; see efs_gb300.h).
// Dot products are compensated float pairs summed by fixed shuffle trees; FP64 appears only in the group
// totals, the scalars thread 0 derives from them, and the residual replacement every 64 iterations. --------
struct BSum {
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
    __device__ __forceinline__ double total() const { return (double)s + (double)c; }
};

// Pair sum over a warp (fixed tree), valid in lane 0.
__device__ __forceinline__ BSum warp_bsum(BSum v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float s2 = __shfl_down_sync(0xffffffffu, v.s, o);
        const float c2 = __shfl_down_sync(0xffffffffu, v.c, o);
        v.add_pair(s2, c2);
    }
    return v;
}

// Block pair sums of up to three pair sums, valid in thread 0 only: lanes by a fixed tree, then the warps'
// partials by a second tree in warp 0.  All in float pairs: GB300 runs FP64 at a small fraction of its FP32
// rate, and a serial chain of FP64 additions on one thread held every other warp at the next barrier.  One
// block barrier; the next call writes `sw` only after a barrier every thread reaches after this one's reads.
__device__ void block_pairs3(BSum& a, BSum& b, BSum& c) {
    __shared__ float sw[6][32];
    a = warp_bsum(a);
    b = warp_bsum(b);
    c = warp_bsum(c);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0) {
        sw[0][warp] = a.s; sw[1][warp] = a.c;
        sw[2][warp] = b.s; sw[3][warp] = b.c;
        sw[4][warp] = c.s; sw[5][warp] = c.c;
    }
    __syncthreads();
    if (warp == 0) {
        const bool in = lane < nw;
        a.s = in ? sw[0][lane] : 0.f; a.c = in ? sw[1][lane] : 0.f;
        b.s = in ? sw[2][lane] : 0.f; b.c = in ? sw[3][lane] : 0.f;
        c.s = in ? sw[4][lane] : 0.f; c.c = in ? sw[5][lane] : 0.f;
        a = warp_bsum(a);
        b = warp_bsum(b);
        c = warp_bsum(c);
    }
}

// No work for thread 0 between a reduction and its broadcast.
struct NoEpilogue {
    __device__ __forceinline__ void operator()(double, double, double) const {}
};

__device__ __forceinline__ float lap2_f(const float* x, uint16_t f, int i, int W) {
    float s = 0.f;
    if (f & 1u) s += x[i - 1];
    if (f & 2u) s += x[i + 1];
    if (f & 4u) s += x[i - W];
    if (f & 8u) s += x[i + W];
    return s - (float)((f >> 8) & 7) * x[i];
}
template <typename T>
__device__ __forceinline__ double lap2_d(const T* x, uint16_t f, int i, int W) {
    double s = 0.0;
    if (f & 1u) s += (double)x[i - 1];
    if (f & 2u) s += (double)x[i + 1];
    if (f & 4u) s += (double)x[i - W];
    if (f & 8u) s += (double)x[i + W];
    return s - (double)((f >> 8) & 7) * (double)x[i];
}

struct BCGArgs {
    const BScene* sc;
    const int* order;
    int n;
    BFields F;
    double* p64;
    float *r, *d, *t, *e;
    int max_steps;
    float tol_rel, solver_threshold;
    unsigned* fetch;      // next scene to take (reset to 0 before every launch)
};

// The threads that solve one scene: one block, or the CTAs of one thread-block cluster.  A pass that reads
// stencil neighbours written by another thread of the group is preceded by sync().  reduce3 returns the same
// group totals to every thread (block partials added in rank order); before the block barrier that publishes
// them, thread 0 of every CTA runs `t0` on the totals, so scalars it derives and stores in shared memory
// are published by the same barrier.  `tot` is written again only after the next reduction's first block
// barrier, which every thread reaches after reading it.
struct BlockGroup {
    __device__ __forceinline__ int rank() const { return 0; }
    __device__ __forceinline__ int ranks() const { return 1; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    template <class T0>
    __device__ __forceinline__ void reduce3(BSum a, BSum b, BSum c, double& x, double& y, double& z, T0&& t0) {
        __shared__ double tot[3];
        block_pairs3(a, b, c);
        if (threadIdx.x == 0) {
            const double bx = a.total(), by = b.total(), bz = c.total();
            t0(bx, by, bz);
            tot[0] = bx; tot[1] = by; tot[2] = bz;
        }
        __syncthreads();
        x = tot[0]; y = tot[1]; z = tot[2];
    }
    __device__ __forceinline__ void reduce3(BSum a, BSum b, BSum c, double& x, double& y, double& z) {
        reduce3(a, b, c, x, y, z, NoEpilogue());
    }
    __device__ __forceinline__ int next_scene(unsigned* fetch) {
        __shared__ int s_k;
        if (threadIdx.x == 0) s_k = (int)atomicAdd(fetch, 1u);
        __syncthreads();
        const int k = s_k;
        __syncthreads();
        return k;
    }
    __device__ __forceinline__ void finish() const {}
};

struct ClusterGroup {
    float* slots;         // this CTA's shared memory: 2 x 3 float pairs (alternating per reduction)
    int* next;            // this CTA's shared memory: 2 ints (alternating per fetch)
    int parity = 0, fparity = 0;
    __device__ __forceinline__ int rank() const { return (int)cg::this_cluster().block_rank(); }
    __device__ __forceinline__ int ranks() const { return (int)cg::this_cluster().num_blocks(); }
    __device__ __forceinline__ void sync() const { cg::this_cluster().sync(); }
    // The slot written at one reduction is written again two reductions later, after a cluster barrier that
    // every CTA reaches only once it has read the slot.  Lane r of warp 0 loads rank r's pairs (all loads in
    // flight together) and a fixed shuffle tree adds them, so every CTA gets bit-identical totals.
    template <class T0>
    __device__ void reduce3(BSum a, BSum b, BSum c, double& x, double& y, double& z, T0&& t0) {
        __shared__ double tot[3];
        block_pairs3(a, b, c);
        cg::cluster_group cl = cg::this_cluster();
        if (threadIdx.x == 0) {
            float* sl = slots + 6 * parity;
            sl[0] = a.s; sl[1] = a.c;
            sl[2] = b.s; sl[3] = b.c;
            sl[4] = c.s; sl[5] = c.c;
        }
        cl.sync();
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            BSum px, py, pz;
            if (lane < (int)cl.num_blocks()) {
                const float* rs = cl.map_shared_rank(slots + 6 * parity, lane);
                px.s = rs[0]; px.c = rs[1];
                py.s = rs[2]; py.c = rs[3];
                pz.s = rs[4]; pz.c = rs[5];
            }
            px = warp_bsum(px);
            py = warp_bsum(py);
            pz = warp_bsum(pz);
            if (lane == 0) {
                const double X = px.total(), Y = py.total(), Z = pz.total();
                t0(X, Y, Z);
                tot[0] = X; tot[1] = Y; tot[2] = Z;
            }
        }
        __syncthreads();
        x = tot[0]; y = tot[1]; z = tot[2];
        parity ^= 1;
    }
    __device__ __forceinline__ void reduce3(BSum a, BSum b, BSum c, double& x, double& y, double& z) {
        reduce3(a, b, c, x, y, z, NoEpilogue());
    }
    // The slot written at one fetch is written again two fetches later, after a cluster barrier that every
    // CTA reaches only once it has read the slot.
    __device__ int next_scene(unsigned* fetch) {
        cg::cluster_group cl = cg::this_cluster();
        if (cl.block_rank() == 0 && threadIdx.x == 0) next[fparity] = (int)atomicAdd(fetch, 1u);
        cl.sync();
        const int k = *cl.map_shared_rank(next + fparity, 0);
        fparity ^= 1;
        return k;
    }
    // no CTA leaves while another may still read its shared memory
    __device__ __forceinline__ void finish() const { cg::this_cluster().sync(); }
};

// CG (EFS_CG_MIXED_RECURRENCE) of one scene by group G (CGSolver.cpp:32-83 with the mixed precision and
// recurrence of the persistent solver; see efs_gb300.h).
template <class G>
__device__ void solve_scene(const BCGArgs& A, int s, G& grp) {
    const BScene S = A.sc[s];
    const long long o = S.base;
    const int N = S.g.N, W = S.g.W;
    const float* b = A.F.div + o;
    const uint16_t* info = A.F.rowinfo + o;
    float* p = A.F.p + o;
    double* p64 = A.p64 + o;
    float *r = A.r + o, *d = A.d + o, *t = A.t + o, *e = A.e + o;
    DevCtl* ctl = A.F.sctl + s;
    const int i0 = grp.rank() * blockDim.x + threadIdx.x, stride = grp.ranks() * blockDim.x;
    // r = b - L p0 with p0 = b (CGSolver.cpp:63-72), in FP64; d = r
    BSum rr_p, bb_p, rows_p;
    for (int i = i0; i < N; i += stride) {
        const float bi = b[i];
        bb_p.add_prod(bi, bi);
        const uint16_t f = info[i];
        if (!(f & 0x8000u)) continue;
        rows_p.add(1.f);
        p64[i] = (double)bi;
        e[i] = 0.f;
        const float ri = (float)((double)bi - lap2_d(b, f, i, W));
        r[i] = ri;
        d[i] = ri;
        rr_p.add_prod(ri, ri);
    }
    double rr, bb, rows;
    grp.reduce3(rr_p, bb_p, rows_p, rr, bb, rows);
    float thr_f = A.tol_rel > 0 ? (float)((double)A.tol_rel * (double)A.tol_rel * bb) : A.solver_threshold;
    if (A.tol_rel > 0 && !(thr_f > 0)) thr_f = FLT_MIN;
    const double thr = (double)thr_f;
    // true residual: fold e into p64, r = b - L p64 in FP64 (CGSolver.cpp:46-50)
    auto replace = [&](double& rr_out) {
        for (int i = i0; i < N; i += stride) {
            if (!(info[i] & 0x8000u)) continue;
            p64[i] += (double)e[i];
            e[i] = 0.f;
        }
        grp.sync();
        BSum rp;
        for (int i = i0; i < N; i += stride) {
            const uint16_t f = info[i];
            if (!(f & 0x8000u)) continue;
            const float ri = (float)((double)b[i] - lap2_d(p64, f, i, W));
            r[i] = ri;
            rp.add_prod(ri, ri);
        }
        double u1, u2;
        grp.reduce3(rp, BSum(), BSum(), rr_out, u1, u2);
    };
    int conv = rr < thr, it = 0;
    // 128-bit passes: a thread takes groups of four cells (consecutive lanes, consecutive groups), x
    // neighbours across groups by warp shuffles.  Needs W (so N) a multiple of 4 and 16-byte aligned vectors.
    const bool vec4 = (W & 3) == 0 && ((reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(t) |
                                       reinterpret_cast<uintptr_t>(r) | reinterpret_cast<uintptr_t>(e)) & 15u) == 0 &&
                      (reinterpret_cast<uintptr_t>(info) & 7u) == 0;
    const int N4 = N >> 2, W4 = W >> 2, lane = threadIdx.x & 31;
    // t = L d on rows (same neighbour order and rounding as lap2_f), d.t and t.t
    auto tpass = [&](BSum& dtp, BSum& ttp) {
        if (vec4) {
            const float4* d4 = reinterpret_cast<const float4*>(d);
            float4* t4 = reinterpret_cast<float4*>(t);
            for (int gb = i0 - lane; gb < N4; gb += stride) {
                const int g = gb + lane;
                const uint2 fi = g < N4 ? reinterpret_cast<const uint2*>(info)[g] : make_uint2(0u, 0u);
                const unsigned fw[4] = {fi.x & 0xFFFFu, fi.x >> 16, fi.y & 0xFFFFu, fi.y >> 16};
                const bool any = ((fw[0] | fw[1] | fw[2] | fw[3]) & 0x8000u) != 0;
                float4 xc = make_float4(0.f, 0.f, 0.f, 0.f), ym = xc, yp = xc;
                if (any) { xc = d4[g]; ym = d4[g - W4]; yp = d4[g + W4]; }   // rows are interior cells
                float left = __shfl_up_sync(0xffffffffu, xc.w, 1);
                float right = __shfl_down_sync(0xffffffffu, xc.x, 1);
                if (lane == 0 && (fw[0] & 0x8000u) && (fw[0] & 1u)) left = d[4 * g - 1];
                if (lane == 31 && (fw[3] & 0x8000u) && (fw[3] & 2u)) right = d[4 * g + 4];
                if (!any) continue;
                const float cx[4] = {xc.x, xc.y, xc.z, xc.w};
                const float cym[4] = {ym.x, ym.y, ym.z, ym.w}, cyp[4] = {yp.x, yp.y, yp.z, yp.w};
                float to[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    to[k] = 0.f;
                    const unsigned f = fw[k];
                    if (!(f & 0x8000u)) continue;
                    float sm = 0.f;
                    if (f & 1u) sm += (k == 0) ? left : cx[k > 0 ? k - 1 : 0];
                    if (f & 2u) sm += (k == 3) ? right : cx[k < 3 ? k + 1 : 3];
                    if (f & 4u) sm += cym[k];
                    if (f & 8u) sm += cyp[k];
                    const float ti = sm - (float)((f >> 8) & 7) * cx[k];
                    to[k] = ti;
                    dtp.add_prod(cx[k], ti);
                    ttp.add_prod(ti, ti);
                }
                t4[g] = make_float4(to[0], to[1], to[2], to[3]);
            }
        } else {
            for (int i = i0; i < N; i += stride) {
                const uint16_t f = info[i];
                if (!(f & 0x8000u)) continue;
                const float ti = lap2_f(d, f, i, W);
                t[i] = ti;
                dtp.add_prod(d[i], ti);
                ttp.add_prod(ti, ti);
            }
        }
    };
    // The FP64 scalar work of an iteration is thread 0's (GB300 runs FP64 divisions slowly; in every thread
    // they cost the scene's group microseconds per iteration), done on the totals of the t pass's reduction
    // and published by its barrier.  Every CTA of a cluster computes the same values from the same totals.
    __shared__ float s_sc[2];
    __shared__ int s_mode;
    auto scalars = [&](double rr_, double dt_, double tt_, int it_) {
        int mode = 0;
        float al = 0.f, be = 0.f;
        const double ad = div_fast(rr_, dt_);
        if (!(dt_ != 0.0) || !isfinite(ad)) {
            mode = -1;                                 // breakdown (singular block): not converged
        } else {
            al = (float)ad;
            const double est = ad * ad * tt_ - rr_;    // r'.r' from the CG recurrence
            if ((it_ & 0x3F) && est > 0.0) { mode = 1; be = (float)div_fast(est, rr_); }
        }
        s_sc[0] = al;
        s_sc[1] = be;
        s_mode = mode;
    };
    if (!conv) {
        // Pass 1 (t = L d; d.t, t.t) and pass 2 (e, r, d per cell; exact r.r) alternate.  The r.r of pass 2
        // travels with the next pass 1's reduction: one reduction and one group barrier per iteration.  The
        // stop test of iteration k is therefore taken after the pass 1 of iteration k+1, whose t is then
        // unused; e, r and p are unaffected.
        double dt, tt, u3;
        {
            BSum dtp, ttp;
            tpass(dtp, ttp);
            grp.reduce3(BSum(), dtp, ttp, u3, dt, tt, [&](double, double y, double z) { scalars(rr, y, z, 0); });
        }
        for (it = 0; it < A.max_steps; it++) {
            const int mode = s_mode;
            const float alpha = s_sc[0];
            if (mode < 0) break;
            const double old = rr;
            if (mode == 1) {
                const float beta = s_sc[1];
                BSum rp;
                if (vec4) {
                    for (int g = i0; g < N4; g += stride) {
                        const uint2 fi = reinterpret_cast<const uint2*>(info)[g];
                        const unsigned rows = ((fi.x >> 15) & 1u) | ((fi.x >> 30) & 2u) | (((fi.y >> 15) & 1u) << 2) |
                                              ((fi.y >> 31) << 3);
                        if (!rows) continue;
                        float4 dv = reinterpret_cast<float4*>(d)[g], ev = reinterpret_cast<float4*>(e)[g];
                        float4 rv = reinterpret_cast<float4*>(r)[g];
                        const float4 tv = reinterpret_cast<const float4*>(t)[g];
                        float* dd = &dv.x;
                        float* ee = &ev.x;
                        float* rr4 = &rv.x;
                        const float* tt4 = &tv.x;
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            if (!((rows >> k) & 1u)) continue;
                            const float di = dd[k];
                            ee[k] += alpha * di;
                            const float rn = rr4[k] + (-alpha) * tt4[k];
                            rr4[k] = rn;
                            dd[k] = di * beta + rn;
                            rp.add_prod(rn, rn);
                        }
                        reinterpret_cast<float4*>(e)[g] = ev;
                        reinterpret_cast<float4*>(r)[g] = rv;
                        reinterpret_cast<float4*>(d)[g] = dv;
                    }
                } else {
                    for (int i = i0; i < N; i += stride) {
                        if (!(info[i] & 0x8000u)) continue;
                        const float di = d[i];
                        e[i] += alpha * di;
                        const float rn = r[i] + (-alpha) * t[i];
                        r[i] = rn;
                        d[i] = di * beta + rn;
                        rp.add_prod(rn, rn);
                    }
                }
                grp.sync();
                BSum dtp, ttp;
                tpass(dtp, ttp);
                grp.reduce3(rp, dtp, ttp, rr, dt, tt, [&](double x, double y, double z) { scalars(x, y, z, it + 1); });
                if (rr < thr) {
                    replace(rr);
                    if (rr < thr) { conv = 1; break; }
                    // d was formed from the recurrence residual: restart it from the recomputed one
                    for (int i = i0; i < N; i += stride)
                        if (info[i] & 0x8000u) d[i] = r[i];
                    grp.sync();
                    BSum dtp2, ttp2;
                    tpass(dtp2, ttp2);
                    grp.reduce3(BSum(), dtp2, ttp2, u3, dt, tt, [&](double, double y, double z) { scalars(rr, y, z, it + 1); });
                }
            } else {
                for (int i = i0; i < N; i += stride)
                    if (info[i] & 0x8000u) e[i] += alpha * d[i];
                grp.sync();
                replace(rr);
                if (rr < thr) { conv = 1; break; }
                __shared__ float s_b2;
                if (threadIdx.x == 0) s_b2 = (float)(rr / old);
                __syncthreads();
                const float beta = s_b2;
                for (int i = i0; i < N; i += stride)
                    if (info[i] & 0x8000u) d[i] = d[i] * beta + r[i];
                grp.sync();
                BSum dtp, ttp;
                tpass(dtp, ttp);
                grp.reduce3(BSum(), dtp, ttp, u3, dt, tt, [&](double, double y, double z) { scalars(rr, y, z, it + 1); });
            }
        }
        it = min(it + 1, A.max_steps);
    }
    // p = p64 + e (FP64 accumulator folded), rows only
    for (int i = i0; i < N; i += stride) {
        if (!(info[i] & 0x8000u)) continue;
        const double v = p64[i] + (double)e[i];
        p64[i] = v;
        e[i] = 0.f;
        p[i] = (float)v;
    }
    if (grp.rank() == 0 && threadIdx.x == 0) {
        ctl->converged = conv;
        ctl->iterations = it;
        ctl->rr = rr;
        ctl->bb = bb;
        ctl->thr = thr;
        ctl->active_cells = (long long)rows;
        ctl->total_iterations += it;
        ctl->solves += 1;
        ctl->precond_iterations = 0;
    }
    grp.sync();
}

// One block per scene; blocks take scenes largest first.
__global__ void __launch_bounds__(1024) k_batch_cg(BCGArgs A) {
    BlockGroup grp;
    for (;;) {
        const int k = grp.next_scene(A.fetch);
        if (k >= A.n) break;
        solve_scene(A, A.order[k], grp);
    }
}

// One thread-block cluster per scene; clusters take scenes largest first.
__global__ void __launch_bounds__(1024) k_batch_cg_cluster(BCGArgs A) {
    __shared__ float slots[12];
    __shared__ int next[2];
    ClusterGroup grp;
    grp.slots = slots;
    grp.next = next;
    for (;;) {
        const int k = grp.next_scene(A.fetch);
        if (k >= A.n) break;
        solve_scene(A, A.order[k], grp);
    }
    grp.finish();
}

// ---- host side --------------------------------------------------------------------------------------------
void build_tables(efs_batch* b, std::vector<BEntry> (&tab)[5]) {
    for (auto& t : tab) t.clear();
    for (int s = 0; s < b->n; s++) {
        const Geo& g = b->sc[s].g;
        const int ix = (g.W - 2 + b->bx - 1) / b->bx, iy = (g.H - 2 + b->by - 1) / b->by;
        for (int y = 0; y < iy; y++)
            for (int x = 0; x < ix; x++) tab[0].push_back(BEntry{s, x, y, 0});
        const int px = (g.W - 1 + b->bx - 1) / b->bx, py = (g.H - 1 + b->by - 1) / b->by;
        for (int y = 0; y < py; y++)
            for (int x = 0; x < px; x++) tab[1].push_back(BEntry{s, x, y, 0});
        const int nl = (((g.N + 31) / 32) * 32 + 255) / 256;
        for (int x = 0; x < nl; x++) tab[2].push_back(BEntry{s, x, 0, 0});
        for (int x = 0; x < (g.H - 2 + 127) / 128; x++) tab[3].push_back(BEntry{s, x, 0, 0});
        for (int x = 0; x < (g.W - 2 + 127) / 128; x++) tab[4].push_back(BEntry{s, x, 0, 0});
    }
}

int upload_tables(efs_batch* b) {
    std::vector<BEntry> tab[5];
    build_tables(b, tab);
    for (int k = 0; k < 5; k++) {
        if (b->d_tab[k]) cudaFree(b->d_tab[k]);
        b->d_tab[k] = nullptr;
        BCK(cudaMalloc(reinterpret_cast<void**>(&b->d_tab[k]), std::max<size_t>(1, tab[k].size()) * sizeof(BEntry)), "cudaMalloc table");
        if (!tab[k].empty())
            BCK(cudaMemcpy(b->d_tab[k], tab[k].data(), tab[k].size() * sizeof(BEntry), cudaMemcpyHostToDevice), "upload table");
        b->ntab[k] = (int)tab[k].size();
    }
    return EFS_OK;
}

BLaunch launch_of(const efs_batch* b) {
    BLaunch L{};
    L.interior = BView{b->d_tab[0], b->ntab[0], b->d_sc};
    L.post = BView{b->d_tab[1], b->ntab[1], b->d_sc};
    L.linear = BView{b->d_tab[2], b->ntab[2], b->d_sc};
    L.dx = BView{b->d_tab[3], b->ntab[3], b->d_sc};
    L.dy = BView{b->d_tab[4], b->ntab[4], b->d_sc};
    L.bx_dim = b->bx;
    L.by_dim = b->by;
    L.grid = b->sm_count * b->bps;
    L.list_grid = b->sm_count * 4;
    L.total_cells = b->total;
    L.F = b->F;
    L.dt = b->prm.dt;
    L.vel_decay = b->prm.vel_decay;
    L.rho_d = b->prm.rho_d;
    L.thrL = b->prm.liquid_threshold;
    L.lp = b->prm.lambda_plus;
    L.lm = b->prm.lambda_minus;
    L.eta = b->prm.eta;
    L.gravity = b->prm.gravity_enabled ? 1 : 0;
    L.stream = b->stream;
    return L;
}

cudaError_t launch_cg(const efs_batch* b) {
    BCGArgs A;
    A.sc = b->d_sc;
    A.order = b->d_order;
    A.n = b->n;
    A.F = b->F;
    A.p64 = b->p64;
    A.r = b->r; A.d = b->d; A.t = b->t; A.e = b->e;
    A.max_steps = b->prm.max_steps;
    A.tol_rel = b->prm.tol_rel;
    A.solver_threshold = b->prm.solver_threshold;
    A.fetch = b->fetch;
    cudaError_t e = cudaMemsetAsync(b->fetch, 0, sizeof(unsigned), b->stream);
    if (e != cudaSuccess) return e;
    if (b->cg_cluster <= 1) {
        const int grid = std::min(b->n, b->sm_count * (1024 / b->cg_threads));
        k_batch_cg<<<std::max(1, grid), b->cg_threads, 0, b->stream>>>(A);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)b->cg_cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(b->cg_cluster * std::max(1, std::min(b->n, b->cg_clusters_max))));
    cfg.blockDim = dim3((unsigned)b->cg_threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = b->stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_batch_cg_cluster, A);
}

cudaError_t enqueue_stage(const efs_batch* b, int stage, bool fuse, bool chain = false) {
    const BLaunch L = launch_of(b);
    if (stage == EFS_STAGE_PROJECT) {
        cudaError_t e = batch_project_pre(L);
        if (e != cudaSuccess) return e;
        if ((e = launch_cg(b)) != cudaSuccess) return e;
        return batch_project_post(L);
    }
    return batch_stage(L, stage, fuse, chain);
}

cudaError_t enqueue_step(const efs_batch* b, unsigned stages) {
    const bool fuse = (stages & EFS_STAGE_BIT(EFS_STAGE_VEL_ADVECT)) && (stages & EFS_STAGE_BIT(EFS_STAGE_ADD_FORCE));
    const bool chain = (stages & EFS_STAGE_BIT(EFS_STAGE_RHO_ADVECT)) && (stages & EFS_STAGE_BIT(EFS_STAGE_VEL_ADVECT));
    for (int s = 0; s < EFS_STAGE_COUNT; s++) {
        if (!(stages & EFS_STAGE_BIT(s))) continue;
        if (s == EFS_STAGE_ADD_FORCE && fuse) continue;
        cudaError_t e = enqueue_stage(b, s, s == EFS_STAGE_VEL_ADVECT && fuse, chain);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void drop_graph(efs_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->graph_def) cudaGraphDestroy(b->graph_def);
    b->graph = nullptr;
    b->graph_def = nullptr;
}

int build_graph(efs_batch* b) {
    const unsigned stages = EFS_STAGES_ALL & ~b->prm.disable_mask;
    if (b->graph && b->graph_stages == stages) return EFS_OK;
    drop_graph(b);
    cudaGraph_t g = nullptr;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    cudaError_t le = enqueue_step(b, stages);
    cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess) { if (g) cudaGraphDestroy(g); return bcuda(b, le, "batch step capture"); }
    if (ce != cudaSuccess) return bcuda(b, ce, "cudaStreamEndCapture");
    size_t n = 0;
    cudaGraphGetNodes(g, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) cudaGraphGetNodes(g, nodes.data(), &n);
    int kernels = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) kernels++;
    }
    cudaGraphExec_t ex = nullptr;
    cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
    if (ie != cudaSuccess) { cudaGraphDestroy(g); return bcuda(b, ie, "cudaGraphInstantiate"); }
    b->graph = ex;
    b->graph_def = g;
    b->graph_stages = stages;
    b->graph_kernels = kernels;
    return EFS_OK;
}

int check_status(efs_batch* b) {
    BCK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    DevCtl h;
    BCK(cudaMemcpy(&h, b->F.ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost), "read device status");
    if (h.error) return bfail(b, EFS_ERR_DEVICE_FAULT, "device error word " + std::to_string(h.error));
    return EFS_OK;
}

bool field_ok(int f) {
    return f == EFS_FIELD_VEL || f == EFS_FIELD_RHO || f == EFS_FIELD_GAMMA || f == EFS_FIELD_BETA ||
           f == EFS_FIELD_DIVERGENCE || f == EFS_FIELD_PRESSURE || f == EFS_FIELD_FORCES || f == EFS_FIELD_BOUNDARY;
}

float* scalar_field(efs_batch* b, int f) {
    switch (f) {
        case EFS_FIELD_RHO: return b->F.rho;
        case EFS_FIELD_GAMMA: return b->F.gamma;
        case EFS_FIELD_BETA: return b->F.beta;
        case EFS_FIELD_DIVERGENCE: return b->F.div;
        case EFS_FIELD_PRESSURE: return b->F.p;
        default: return nullptr;
    }
}

}  // namespace

extern "C" {

const char* efs_batch_last_error(const efs_batch* b) { return b ? b->err.c_str() : g_batch_create_error.c_str(); }

void efs_batch_destroy(efs_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    for (auto& t : b->d_tab) if (t) cudaFree(t);
    for (void* p : b->allocs) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int efs_batch_create(int n_scenes, const int* widths, const int* heights, const efs_params* params,
                     const float* gravity_force, efs_batch** out) {
    if (!out) return bfail(nullptr, EFS_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n_scenes < 1 || !widths || !heights || !params) return bfail(nullptr, EFS_ERR_ARG, "n_scenes >= 1 and non-NULL arrays");
    if (params->solver != EFS_SOLVER_CG || params->cg_variant != EFS_CG_MIXED_RECURRENCE)
        return bfail(nullptr, EFS_ERR_ARG, "batched scenes use the CG solver (EFS_CG_MIXED_RECURRENCE)");
    if (params->re_calc_div) return bfail(nullptr, EFS_ERR_ARG, "RE_CALC_DIV is not supported in batches");
    if (params->sharpen_mode != EFS_SHARPEN_PARALLEL)
        return bfail(nullptr, EFS_ERR_ARG, "batched scenes sharpen in EFS_SHARPEN_PARALLEL mode only");
    if (params->max_steps < 0 || !std::isfinite(params->dt)) return bfail(nullptr, EFS_ERR_ARG, "bad params");
    for (int s = 0; s < n_scenes; s++)
        if (widths[s] < 4 || heights[s] < 4 || (long long)widths[s] * heights[s] > (1LL << 26))
            return bfail(nullptr, EFS_ERR_ARG, "scene sizes must be 4..2^26 cells");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return bfail(nullptr, EFS_ERR_NO_DEVICE, "no CUDA device");
    efs_batch* b = new efs_batch();
    b->n = n_scenes;
    b->prm = *params;
    cudaGetDevice(&b->device);
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device);
    cudaError_t e;
    auto bail = [&](cudaError_t er, const char* what) {
        const int st = bcuda(nullptr, er, what);
        efs_batch_destroy(b);
        return st;
    };
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "cudaStreamCreate");
    long long off = 0;
    for (int s = 0; s < n_scenes; s++) {
        BScene S{};
        S.g = Geo{widths[s], heights[s], 1, widths[s] * heights[s], widths[s] * heights[s]};
        S.base = off;
        S.gforce = gravity_force ? gravity_force[s] : params->gravity_force;
        off += ((long long)S.g.N + 31) / 32 * 32;
        b->sc.push_back(S);
    }
    b->total = off;
    b->order.resize(n_scenes);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return b->sc[x].g.N > b->sc[y].g.N; });
    const long long T = b->total;
    BFields& F = b->F;
#define BA(ptr, cnt) if ((e = balloc(b, &(ptr), (cnt))) != cudaSuccess) return bail(e, "cudaMalloc " #ptr)
    BA(b->d_sc, n_scenes); BA(b->d_order, n_scenes);
    BA(F.u, T); BA(F.v, T); BA(F.rho, T); BA(F.gamma, T); BA(F.beta, T); BA(F.div, T); BA(F.p, T); BA(F.fx, T); BA(F.fy, T);
    BA(F.solid, T); BA(F.tu, T); BA(F.tv, T); BA(F.validA, T); BA(F.validB, T);
    BA(F.wb, 4 * T); BA(F.wf, 4 * T); BA(F.bb, T); BA(F.fb, T); BA(F.bsum, T); BA(F.gsum, T); BA(F.rho_acc, T);
    BA(F.sh_idx, T); BA(F.sh_sid, T); BA(F.sh_val, T); BA(F.sh_end, 3 * T);
    BA(F.rowinfo, T); BA(F.chunk_flag, T / 32 + 1); BA(F.ctl, 1); BA(F.sctl, n_scenes);
    BA(b->p64, T); BA(b->r, T); BA(b->d, T); BA(b->t, T); BA(b->e, T); BA(b->fetch, 1);
#undef BA
    F.list_cap = (int)std::min<long long>(T, 1LL << 30);
    if ((e = cudaMemcpy(b->d_sc, b->sc.data(), n_scenes * sizeof(BScene), cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e, "upload scenes");
    if ((e = cudaMemcpy(b->d_order, b->order.data(), n_scenes * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e, "upload order");
    // Grid2D constructor state (Grid2D.cpp:11-66): zero fields, gamma = 1, solid border
    std::vector<float> ones(T, 1.f);
    std::vector<uint8_t> solid(T, 0);
    for (const auto& S : b->sc)
        for (int y = 0; y < S.g.H; y++)
            for (int x = 0; x < S.g.W; x++)
                if (x == 0 || y == 0 || x == S.g.W - 1 || y == S.g.H - 1) solid[S.base + (long long)y * S.g.W + x] = 1;
    if ((e = cudaMemcpy(F.gamma, ones.data(), T * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e, "init");
    if ((e = cudaMemcpy(F.solid, solid.data(), T, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e, "init");
    const int ts = upload_tables(b);
    if (ts != EFS_OK) { efs_batch_destroy(b); return ts; }
    *out = b;
    return EFS_OK;
}

int efs_batch_scene_count(const efs_batch* b, int* n) {
    if (!b || !n) return EFS_ERR_ARG;
    *n = b->n;
    return EFS_OK;
}

int efs_batch_upload_field(efs_batch* b, int scene, int field, const float* host) {
    if (!b) return EFS_ERR_ARG;
    if (scene < 0 || scene >= b->n || !field_ok(field) || !host) return bfail(b, EFS_ERR_ARG, "bad scene, field or pointer");
    const BScene& S = b->sc[scene];
    const long long N = S.g.N, o = S.base;
    BCK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    if (field == EFS_FIELD_VEL || field == EFS_FIELD_FORCES) {
        std::vector<float> a(N), c(N);
        for (long long i = 0; i < N; i++) { a[i] = host[2 * i]; c[i] = host[2 * i + 1]; }
        float* da = field == EFS_FIELD_VEL ? b->F.u : b->F.fx;
        float* dc = field == EFS_FIELD_VEL ? b->F.v : b->F.fy;
        BCK(cudaMemcpy(da + o, a.data(), N * sizeof(float), cudaMemcpyHostToDevice), "upload");
        BCK(cudaMemcpy(dc + o, c.data(), N * sizeof(float), cudaMemcpyHostToDevice), "upload");
    } else if (field == EFS_FIELD_BOUNDARY) {
        std::vector<uint8_t> s8(N);
        for (long long i = 0; i < N; i++) {
            if (host[i] != 0.f && host[i] != 1.f) return bfail(b, EFS_ERR_ARG, "boundary values must be 0.0 or 1.0");
            s8[i] = host[i] == 1.f ? 1 : 0;
        }
        BCK(cudaMemcpy(b->F.solid + o, s8.data(), N, cudaMemcpyHostToDevice), "upload");
    } else {
        BCK(cudaMemcpy(scalar_field(b, field) + o, host, N * sizeof(float), cudaMemcpyHostToDevice), "upload");
    }
    return EFS_OK;
}

int efs_batch_download_field(efs_batch* b, int scene, int field, float* host) {
    if (!b) return EFS_ERR_ARG;
    if (scene < 0 || scene >= b->n || !field_ok(field) || !host) return bfail(b, EFS_ERR_ARG, "bad scene, field or pointer");
    const BScene& S = b->sc[scene];
    const long long N = S.g.N, o = S.base;
    const int st = check_status(b);
    if (st != EFS_OK) return st;
    if (field == EFS_FIELD_VEL || field == EFS_FIELD_FORCES) {
        std::vector<float> a(N), c(N);
        const float* da = field == EFS_FIELD_VEL ? b->F.u : b->F.fx;
        const float* dc = field == EFS_FIELD_VEL ? b->F.v : b->F.fy;
        BCK(cudaMemcpy(a.data(), da + o, N * sizeof(float), cudaMemcpyDeviceToHost), "download");
        BCK(cudaMemcpy(c.data(), dc + o, N * sizeof(float), cudaMemcpyDeviceToHost), "download");
        for (long long i = 0; i < N; i++) { host[2 * i] = a[i]; host[2 * i + 1] = c[i]; }
    } else if (field == EFS_FIELD_BOUNDARY) {
        std::vector<uint8_t> s8(N);
        BCK(cudaMemcpy(s8.data(), b->F.solid + o, N, cudaMemcpyDeviceToHost), "download");
        for (long long i = 0; i < N; i++) host[i] = s8[i] ? 1.f : 0.f;
    } else {
        BCK(cudaMemcpy(host, scalar_field(b, field) + o, N * sizeof(float), cudaMemcpyDeviceToHost), "download");
    }
    return EFS_OK;
}

int efs_batch_stage(efs_batch* b, int stage) {
    if (!b) return EFS_ERR_ARG;
    if (stage < 0 || stage >= EFS_STAGE_COUNT) return bfail(b, EFS_ERR_ARG, "unknown stage");
    BCK(enqueue_stage(b, stage, false), "batch stage");
    return EFS_OK;
}

int efs_batch_step(efs_batch* b, int n_steps) {
    if (!b) return EFS_ERR_ARG;
    if (n_steps < 0) return bfail(b, EFS_ERR_ARG, "n_steps < 0");
    if (n_steps == 0) return EFS_OK;
    const int s = build_graph(b);
    if (s != EFS_OK) return s;
    for (int k = 0; k < n_steps; k++) BCK(cudaGraphLaunch(b->graph, b->stream), "cudaGraphLaunch");
    b->frames += n_steps;
    return EFS_OK;
}

int efs_batch_time_steps(efs_batch* b, int n_steps, float* ms) {
    if (!b || !ms) return EFS_ERR_ARG;
    if (n_steps < 1) return bfail(b, EFS_ERR_ARG, "n_steps >= 1");
    const int s = build_graph(b);
    if (s != EFS_OK) return s;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0), "cudaEventCreate");
    BCK(cudaEventCreate(&e1), "cudaEventCreate");
    BCK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    BCK(cudaEventRecord(e0, b->stream), "cudaEventRecord");
    for (int k = 0; k < n_steps; k++) BCK(cudaGraphLaunch(b->graph, b->stream), "cudaGraphLaunch");
    BCK(cudaEventRecord(e1, b->stream), "cudaEventRecord");
    BCK(cudaEventSynchronize(e1), "cudaEventSynchronize");
    BCK(cudaEventElapsedTime(ms, e0, e1), "cudaEventElapsedTime");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->frames += n_steps;
    return check_status(b);
}

int efs_batch_synchronize(efs_batch* b) {
    if (!b) return EFS_ERR_ARG;
    return check_status(b);
}

int efs_batch_stats(efs_batch* b, int scene, efs_stats* out) {
    if (!b || !out) return EFS_ERR_ARG;
    if (scene < 0 || scene >= b->n) return bfail(b, EFS_ERR_ARG, "bad scene");
    const int st = check_status(b);
    if (st != EFS_OK) return st;
    DevCtl h, g;
    BCK(cudaMemcpy(&h, b->F.sctl + scene, sizeof(DevCtl), cudaMemcpyDeviceToHost), "download stats");
    BCK(cudaMemcpy(&g, b->F.ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost), "download stats");
    std::memset(out, 0, sizeof(*out));
    out->frames = b->frames;
    out->solve_steps = h.iterations;
    out->converged = h.converged;
    out->paused = h.paused;
    out->device_error = g.error;
    out->rr = h.rr;
    out->bb = h.bb;
    out->threshold = h.thr;
    out->active_cells = h.active_cells;
    out->total_solve_steps = h.total_iterations;
    out->solves = h.solves;
    return EFS_OK;
}

int efs_batch_kernel_count(efs_batch* b, int* count) {
    if (!b || !count) return EFS_ERR_ARG;
    const int s = build_graph(b);
    if (s != EFS_OK) return s;
    *count = b->graph_kernels;
    return EFS_OK;
}

int efs_batch_get_tuning(const efs_batch* b, efs_batch_tuning* t) {
    if (!b || !t) return EFS_ERR_ARG;
    t->tile_x = b->bx;
    t->tile_y = b->by;
    t->blocks_per_sm = b->bps;
    t->solver_threads = b->cg_threads;
    t->solver_cluster = b->cg_cluster;
    t->ms_per_step = 0.f;
    return EFS_OK;
}

int efs_batch_set_tuning(efs_batch* b, const efs_batch_tuning* t) {
    if (!b || !t) return EFS_ERR_ARG;
    if (t->tile_x < 1 || t->tile_y < 1 || t->tile_x * t->tile_y > 1024 || (t->tile_x * t->tile_y) % 32 != 0 ||
        t->blocks_per_sm < 1 || t->blocks_per_sm > 32 ||
        (t->solver_threads != 128 && t->solver_threads != 256 && t->solver_threads != 512 && t->solver_threads != 1024) ||
        (t->solver_cluster != 1 && t->solver_cluster != 2 && t->solver_cluster != 4 && t->solver_cluster != 8 &&
         t->solver_cluster != 16))
        return bfail(b, EFS_ERR_ARG, "tile_x * tile_y a multiple of 32 up to 1024; blocks_per_sm 1..32; solver_threads "
                                     "128..1024 (power of 2); solver_cluster 1, 2, 4, 8 or 16");
    BCK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    int clusters = 0;
    if (t->solver_cluster > 1) {
        if (t->solver_cluster > 8)
            BCK(cudaFuncSetAttribute(k_batch_cg_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1), "cluster size attribute");
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)t->solver_cluster;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3((unsigned)t->solver_cluster);
        cfg.blockDim = dim3((unsigned)t->solver_threads);
        cfg.attrs = at;
        cfg.numAttrs = 1;
        BCK(cudaOccupancyMaxActiveClusters(&clusters, k_batch_cg_cluster, &cfg), "cudaOccupancyMaxActiveClusters");
        if (clusters < 1) return bfail(b, EFS_ERR_ARG, "this solver cluster shape cannot be resident on the device");
    }
    b->bx = t->tile_x;
    b->by = t->tile_y;
    b->bps = t->blocks_per_sm;
    b->cg_threads = t->solver_threads;
    b->cg_cluster = t->solver_cluster;
    b->cg_clusters_max = clusters;
    drop_graph(b);
    return upload_tables(b);
}

// Coordinate search over the tile shape, the blocks per SM of the stage kernels and the solver's block size:
// each candidate runs `trial_steps` timed steps from the same saved state (the state is restored after every
// trial), and the fastest is kept.
int efs_batch_autotune(efs_batch* b, int trial_steps, efs_batch_tuning* best_out) {
    if (!b) return EFS_ERR_ARG;
    if (trial_steps < 1) return bfail(b, EFS_ERR_ARG, "trial_steps >= 1");
    BCK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    const long long T = b->total;
    // save the state every step reads or writes across steps
    struct Saved { void* dev; size_t bytes; std::vector<unsigned char> host; };
    std::vector<Saved> sv = {{b->F.u, (size_t)T * 4, {}}, {b->F.v, (size_t)T * 4, {}}, {b->F.rho, (size_t)T * 4, {}},
                             {b->F.gamma, (size_t)T * 4, {}}, {b->F.beta, (size_t)T * 4, {}}, {b->F.p, (size_t)T * 4, {}},
                             {b->F.div, (size_t)T * 4, {}}, {b->F.sctl, (size_t)b->n * sizeof(DevCtl), {}}};
    for (auto& x : sv) {
        x.host.resize(x.bytes);
        BCK(cudaMemcpy(x.host.data(), x.dev, x.bytes, cudaMemcpyDeviceToHost), "save state");
    }
    const int64_t frames0 = b->frames;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0), "cudaEventCreate");
    BCK(cudaEventCreate(&e1), "cudaEventCreate");
    auto restore = [&]() -> int {
        for (auto& x : sv) BCK(cudaMemcpy(x.dev, x.host.data(), x.bytes, cudaMemcpyHostToDevice), "restore state");
        b->frames = frames0;
        return EFS_OK;
    };
    auto trial = [&](const efs_batch_tuning& t, float& ms) -> int {
        int s = efs_batch_set_tuning(b, &t);
        if (s != EFS_OK) return s;
        if ((s = restore()) != EFS_OK) return s;
        if ((s = efs_batch_step(b, 1)) != EFS_OK) return s;   // warm-up and graph build
        BCK(cudaEventRecord(e0, b->stream), "cudaEventRecord");
        if ((s = efs_batch_step(b, trial_steps)) != EFS_OK) return s;
        BCK(cudaEventRecord(e1, b->stream), "cudaEventRecord");
        BCK(cudaEventSynchronize(e1), "cudaEventSynchronize");
        BCK(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        ms /= trial_steps;
        return check_status(b);
    };
    efs_batch_tuning best{b->bx, b->by, b->bps, b->cg_threads, b->cg_cluster, 0.f};
    float best_ms = FLT_MAX;
    int s = trial(best, best_ms);
    if (s != EFS_OK) return s;
    const int tiles[][2] = {{32, 8}, {32, 4}, {64, 4}, {16, 8}, {32, 16}, {128, 2}};
    for (const auto& tl : tiles) {
        efs_batch_tuning c = best;
        c.tile_x = tl[0];
        c.tile_y = tl[1];
        float ms;
        if ((s = trial(c, ms)) != EFS_OK) return s;
        if (ms < best_ms) { best_ms = ms; best = c; }
    }
    for (int bps : {2, 4, 8, 16}) {
        efs_batch_tuning c = best;
        c.blocks_per_sm = bps;
        float ms;
        if ((s = trial(c, ms)) != EFS_OK) return s;
        if (ms < best_ms) { best_ms = ms; best = c; }
    }
    for (int cl : {1, 4, 8, 16}) {
        for (int th : {256, 512, 1024}) {
            efs_batch_tuning c = best;
            c.solver_threads = th;
            c.solver_cluster = cl;
            float ms;
            s = trial(c, ms);
            if (s == EFS_ERR_ARG && cl > 1) continue;      // shape not resident on this device
            if (s != EFS_OK) return s;
            if (ms < best_ms) { best_ms = ms; best = c; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if ((s = efs_batch_set_tuning(b, &best)) != EFS_OK) return s;
    if ((s = restore()) != EFS_OK) return s;
    best.ms_per_step = best_ms;
    if (best_out) *best_out = best;
    return EFS_OK;
}

}  // extern "C"
