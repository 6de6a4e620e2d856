// efs_tc.cuh — 5th-generation tensor-core (tcgen05) building blocks for sm_103a and the two GEMM-shaped
// kernels of the U-Net preconditioner: the implicit-GEMM 3x3x3 convolution (forward, and input gradient
// with flipped/transposed weights) and the weight-gradient GEMM.
//
// Operand staging.  Both operands of every tcgen05.mma are K-major BF16 tiles in shared memory in the
// canonical no-swizzle layout: 8-row x 16-byte core matrices (8 rows of 8 BF16 along K, 128 contiguous
// bytes).  A tile of R rows x 16 K-elements (one MMA K-step) is R/8 row groups x 2 K groups; core matrix
// (row group g, K group k) sits at g * 256 + k * 128 bytes, i.e. leading (K) byte offset 128 and stride
// (row group) byte offset 256 in the shared-memory descriptor.  Accumulators are FP32 in tensor memory
// (TMEM): row i of the M = 128 tile is TMEM lane i, output channel n is column n.
//
// Every wait on an mbarrier is bounded in time; on expiry the kernel records an error, waits (bounded
// again) for its own MMAs, frees its TMEM and returns.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_bf16.h>

namespace efs {
namespace tc {

constexpr unsigned long long kWaitNs = 2000000000ull;   // 2 s

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- mbarrier -------------------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Waits until the phase with the given parity has completed; false after kWaitNs.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    if (mbar_test(bar, parity)) return true;
    const unsigned long long t0 = now_ns();
    while (!mbar_test(bar, parity)) {
        if (now_ns() - t0 > kWaitNs) return false;
    }
    return true;
}

// ---- tensor memory ----------------------------------------------------------------------------------------
// Allocation by one whole warp; the TMEM address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory writes (plain stores, cp.async) made visible to the tensor cores' async proxy.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes: thread l of the warp gets lane (base + l).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// ---- MMA ---------------------------------------------------------------------------------------------------
// Shared-memory matrix descriptor: no swizzle, K-major, byte offsets as described at the top of this file.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version of the sm_100 family; base offset 0; layout: no swizzle
    return d;
}
// Instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 accumulator, shape M x N (x K = 16).
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// D (TMEM) = A * B^T (+ D when accumulate != 0), issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The mbarrier receives one arrival when every tcgen05 operation this thread issued so far has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// ---- cp.async ----------------------------------------------------------------------------------------------
// 16 bytes global -> shared; zero-filled when !valid (src must still be a mapped address).
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(sdst)), "l"(gsrc), "r"(valid ? 16u : 0u)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// ---- TMA and bulk copies ------------------------------------------------------------------------------------
// The arrival of this thread plus `bytes` of expected transaction count on the mbarrier.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Tiled 4D tensor load (box of the tensor map) into shared memory; elements outside the tensor read as zero.
// The innermost coordinate c0 is always 0 here (whole 16-byte channel groups).
__device__ __forceinline__ void tma_load_4d(void* sdst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
        ::"r"(smem_u32(sdst)), "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}
// Contiguous global -> shared copy (addresses and size multiples of 16 bytes).
__device__ __forceinline__ void bulk_load(void* sdst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(sdst)), "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Byte offset of element (row, k) (k < 16) in a K-major no-swizzle tile (see the top of this file).
__host__ __device__ __forceinline__ uint32_t tile_off(int row, int k) {
    return (uint32_t)((row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// ============================================================================================================
// Implicit-GEMM 3x3x3 convolution, zero padding ("same"), channel-last BF16 tensors.
//   out[v][n] = sum_{tap, c} in[v + off(tap)][c] * w[tap][c][n]   (+ bias, ReLU, + skip)
// GEMM view per block: M = 128 voxels (linear index v = (z*H + y)*W + x), N = COUT, K = 27 * CIN in steps of
// one tap x 16 channels.  Weights are pre-arranged as wt[tap][c/16][n][16] (BF16) so a K-step's B tile is
// COUT rows of 32 contiguous bytes.  Two operand buffers: the loads of step s+1 fly while MMA s runs.
// ============================================================================================================
struct ConvArgs {
    const __nv_bfloat16* in;    // [V][cin]
    const __nv_bfloat16* wt;    // [27][cin/16][COUT][16]
    const float* bias;          // [COUT] or null
    const __nv_bfloat16* skip;  // [V][COUT] added after the activation, or null
    __nv_bfloat16* out;         // [V][COUT] (BF16) or null
    float* out32;               // [V] FP32: output channel 0 only, or null
    __nv_bfloat16* pre;         // [V][COUT] pre-activation (BF16, for the ReLU mask of the backward pass) or null
    int D, H, W, cin;
    int relu;
    int* err;                   // error word: bit 0 = an mbarrier wait gave up
    // split over the K steps (taps x 16-channel chunks): CTA (x, y) runs steps [y * split_per, (y + 1) * split_per)
    // and stores its raw FP32 accumulators in partial[y][V][COUT]; k_conv_split_reduce finishes the layer.
    // partial null: one CTA per 128 voxels runs every step and finishes the layer itself.
    float* partial;
    int split_per;
    // up != 0: the input is the grid of half the resolution (ceil(W/2) x ceil(H/2) x ceil(D/2) voxels) read as its
    // nearest up-sampling: voxel (x, y, z) takes the input voxel (x/2, y/2, z/2)
    int up;
    // k_conv3_slab with two z slabs: the 2x2x2 mean of the outputs ([ceil(D/2)][ceil(H/2)][ceil(W/2)][COUT]), or null
    __nv_bfloat16* pool;
    // k_conv3_slab: the weights already in its shared-memory order (step s's B tile at s * COUT * 32 bytes), read
    // by one bulk copy; null: the kernel arranges `wt` itself
    const __nv_bfloat16* wslab;
};

constexpr int kConvThreads = 128;
constexpr int kConvSmem = 32 * 1024;   // also caps residency at 7 blocks/SM: 7 x 64 TMEM columns <= 512
constexpr int kConvStages = 4;         // operand buffers of k_conv3_tc
constexpr int kConvAhead = 2;          // steps its gathers run ahead of its MMAs
static_assert(kConvAhead == 2 && kConvStages == kConvAhead + 2, "the refill waits for the MMA two steps back");

template <int COUT>
__global__ void __launch_bounds__(kConvThreads) k_conv3_tc(ConvArgs a) {
    static_assert(COUT == 16 || COUT == 32 || COUT == 64, "COUT");
    constexpr int kABytes = 128 * 32, kBBytes = COUT * 32;
    constexpr uint32_t kCols = COUT < 32 ? 32 : COUT;
    static_assert(kConvStages * (kABytes + kBBytes + 8) + 4 <= kConvSmem, "stages fit the shared memory");
    extern __shared__ __align__(1024) unsigned char smem[];
    auto bufA = [&](int b) { return smem + b * kABytes; };
    auto bufB = [&](int b) { return smem + kConvStages * kABytes + b * kBBytes; };
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + kConvStages * (kABytes + kBBytes));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + kConvStages);

    const int tid = threadIdx.x, warp = tid >> 5;
    const int V = a.D * a.H * a.W;
    const int v = blockIdx.x * 128 + tid;
    const bool vin = v < V;
    const int x = vin ? v % a.W : 0, y = vin ? (v / a.W) % a.H : 0, z = vin ? v / (a.W * a.H) : 0;
    const int chunks = a.cin >> 4;
    const int s_all = 27 * chunks;
    const int s0 = a.partial ? (int)blockIdx.y * a.split_per : 0;
    const int S = a.partial ? min(a.split_per, s_all - s0) : s_all;   // >= 1: the host sizes the split so

    if (warp == 0) tmem_alloc(tslot, kCols);
    if (tid == 0) {
        for (int b = 0; b < kConvStages; b++) mbar_init(&mbar[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    // The gathers walk the K steps in order, so a cursor carries the step's tap offset (dx, dy, dz), channel
    // chunk and weight tile from one gather to the next instead of decomposing the step index each time.
    const int clog = __ffs(chunks) - 1;   // chunks = cin / 16 is 1, 2 or 4
    const int tap0 = s0 >> clog;
    int ccur = s0 & (chunks - 1), dz = tap0 / 9 - 1, dy = (tap0 / 3) % 3 - 1, dx = tap0 % 3 - 1;
    // which of the three offsets along each axis stay inside the grid (bit d + 1)
    const unsigned mx = vin ? ((x > 0) | 2u | ((x < a.W - 1) << 2)) : 0u;
    const unsigned my = (y > 0) | 2u | ((y < a.H - 1) << 2), mz = (z > 0) | 2u | ((z < a.D - 1) << 2);
    const int PW = (a.W + 1) >> 1, PH = (a.H + 1) >> 1;
    const uint32_t aoff0 = tile_off(tid, 0), aoff8 = tile_off(tid, 8);
    const int wn = tid >> 1, wkg = tid & 1;
    const __nv_bfloat16* wcur = a.wt + ((size_t)s0 * COUT + wn) * 16 + wkg * 8;
    auto load = [&](int bi) {
        const bool ok = (mx >> (dx + 1)) & (my >> (dy + 1)) & (mz >> (dz + 1)) & 1u;
        const int nx = x + dx, ny = y + dy, nz = z + dz;
        const int iv = a.up ? (((nz >> 1) * PH + (ny >> 1)) * PW + (nx >> 1)) : ((nz * a.H + ny) * a.W + nx);
        const __nv_bfloat16* src = ok ? a.in + ((size_t)iv * a.cin + ccur * 16) : a.in;
        cp_async16(bufA(bi) + aoff0, src, ok);
        cp_async16(bufA(bi) + aoff8, src + 8, ok);
        if (tid < 2 * COUT) cp_async16(bufB(bi) + tile_off(wn, wkg * 8), wcur, true);
        cp_async_commit();
        // advance the cursor by one step
        wcur += COUT * 16;
        if (++ccur == chunks) {
            ccur = 0;
            if (++dx > 1) {
                dx = -1;
                if (++dy > 1) { dy = -1; ++dz; }
            }
        }
    };

    // kConvStages buffers, the gathers kConvAhead steps ahead: while MMA s runs the gathers of steps s + 1 ..
    // s + kConvAhead fly, and a buffer is refilled two steps after its MMA was issued, so a CTA does not wait for
    // each MMA's completion in turn.  Buffer b serves steps b, b + kConvStages, ...; its mbarrier completes once
    // per step, when that step's MMA has read it.  Thread 0 alone polls that mbarrier; the step's barrier tells
    // the others.
    bool ok = true;
    for (int p = 0; p < kConvAhead && p < S; p++) load(p);
    for (int s = 0; s < S; s++) {
        const int b = s % kConvStages;
        // step s's gather is complete when at most the later steps' gathers already issued are pending
        if (s + 1 < S) cp_async_wait<kConvAhead - 1>();
        else cp_async_wait<0>();
        fence_async_smem();
        const int next = s + kConvAhead, prev = next - kConvStages;
        const bool gave_up = tid == 0 && next < S && prev >= 0 &&
                             !mbar_wait(&mbar[next % kConvStages], (uint32_t)((prev / kConvStages) & 1));
        if (__syncthreads_or(gave_up)) { ok = false; break; }
        if (tid == 0) {
            tc_fence_after();
            const uint64_t ad = sdesc(smem_u32(bufA(b)), 128, 256);
            const uint64_t bd = sdesc(smem_u32(bufB(b)), 128, 256);
            mma_bf16(tmem, ad, bd, idesc_bf16(128, COUT), s > 0 ? 1u : 0u);
            mma_commit(&mbar[b]);
        }
        if (next < S) load(next % kConvStages);
    }
    cp_async_wait<0>();
    // all MMAs (the last commit covers every earlier one), and every buffer's last arrival
    const int last = S - 1;
    for (int b = 0; b < kConvStages && ok; b++) {
        const int sl = last - ((last - b) % kConvStages + kConvStages) % kConvStages;   // last step on buffer b
        if (sl >= 0 && !mbar_wait(&mbar[b], (uint32_t)((sl / kConvStages) & 1))) ok = false;
    }
    if (!ok) {
        if (tid == 0) atomicOr(a.err, 1);
        // bounded: let MMAs in flight finish before freeing TMEM
        mbar_wait(&mbar[last % kConvStages], (uint32_t)((last / kConvStages) & 1));
    }
    tc_fence_after();
    if (ok && a.partial) {
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float acc[16];
            tmem_ld16(tmem + lane_base + (uint32_t)c0, acc);
            if (vin) {
                float4* dst = reinterpret_cast<float4*>(a.partial + ((size_t)blockIdx.y * V + v) * COUT + c0);
#pragma unroll
                for (int q = 0; q < 4; q++) dst[q] = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
            }
        }
    } else if (ok) {
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float acc[16];
            tmem_ld16(tmem + lane_base + (uint32_t)c0, acc);
            if (vin) {
                __align__(16) __nv_bfloat16 o[16], pr[16];
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    float t = acc[j] + (a.bias ? a.bias[c0 + j] : 0.f);
                    pr[j] = __float2bfloat16(t);
                    if (a.relu) t = fmaxf(t, 0.f);
                    if (a.skip) t += __bfloat162float(a.skip[(size_t)v * COUT + c0 + j]);
                    o[j] = __float2bfloat16(t);
                    if (a.out32 && c0 + j == 0) a.out32[v] = t;
                }
                if (a.out) {
                    uint4* dst = reinterpret_cast<uint4*>(a.out + (size_t)v * COUT + c0);
                    dst[0] = reinterpret_cast<const uint4*>(o)[0];
                    dst[1] = reinterpret_cast<const uint4*>(o)[1];
                }
                if (a.pre) {
                    uint4* dst = reinterpret_cast<uint4*>(a.pre + (size_t)v * COUT + c0);
                    dst[0] = reinterpret_cast<const uint4*>(pr)[0];
                    dst[1] = reinterpret_cast<const uint4*>(pr)[1];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kCols);
}

// Finishes a split convolution: per voxel and 4 channels, LANES lanes of one warp sum the splits k = lane,
// lane + LANES, ... in order, then a fixed butterfly over the LANES lanes (every lane ends with the same sum);
// bias, ReLU, the skip addition and the stores of k_conv3_tc's epilogue.  With many splits (the coarse layers run
// 27-54 over a few thousand items) 8 lanes keep 8 loads in flight per item; with few, one lane per item.
template <int LANES>
__host__ __device__ constexpr int split_lanes_ok() { return LANES == 1 || LANES == 8; }
inline int split_lanes(int splits) { return splits >= 16 ? 8 : 1; }
template <int COUT, int LANES>
__global__ void k_conv_split_reduce(const float* __restrict__ partial, int splits, int V, const float* __restrict__ bias,
                                    const __nv_bfloat16* __restrict__ skip, __nv_bfloat16* __restrict__ out,
                                    float* __restrict__ out32, int relu) {
    static_assert(split_lanes_ok<LANES>(), "LANES");
    const long long item = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / LANES;
    const int lane = (int)(threadIdx.x % LANES);
    const bool live = item < (long long)V * (COUT / 4);
    const int v = live ? (int)(item / (COUT / 4)) : 0, c0 = live ? (int)(item % (COUT / 4)) * 4 : 0;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (live) {
#pragma unroll 4
        for (int k = lane; k < splits; k += LANES) {
            const float4 p = *reinterpret_cast<const float4*>(partial + ((size_t)k * V + v) * COUT + c0);
            acc.x += p.x; acc.y += p.y; acc.z += p.z; acc.w += p.w;
        }
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
        acc.z += __shfl_xor_sync(0xffffffffu, acc.z, o);
        acc.w += __shfl_xor_sync(0xffffffffu, acc.w, o);
    }
    if (!live || lane != 0) return;
    const float a4[4] = {acc.x, acc.y, acc.z, acc.w};
    __align__(8) __nv_bfloat16 o[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        float t = a4[j] + (bias ? bias[c0 + j] : 0.f);
        if (relu) t = fmaxf(t, 0.f);
        if (skip) t += __bfloat162float(skip[(size_t)v * COUT + c0 + j]);
        o[j] = __float2bfloat16(t);
        if (out32 && c0 + j == 0) out32[v] = t;
    }
    if (out) *reinterpret_cast<uint2*>(out + (size_t)v * COUT + c0) = *reinterpret_cast<const uint2*>(o);
}

// ============================================================================================================
// Slab 3x3x3 convolution for narrow grids: the same function as k_conv3_tc.  A CTA computes ZS slabs of M = 128
// voxels, each 8 (x) x 16 (y) x 1 (z); slabs reaching past the grid compute zeros there and store only the
// voxels inside.  It copies their input with a one-voxel halo (10 x 18 x (ZS + 2) voxels; zero outside the grid;
// with `up`, voxel (x, y, z) of the half-resolution input at (x/2, y/2, z/2)) into shared memory once, as planes
// of 8 channels ([cin/8][z][y][x] x 16 bytes, each padded to 128 bytes), together with every K step's weight
// tile.  The planes arrive by one tensor load each (SlabMaps) or, for an up-sampled input, by a cp.async gather;
// the weights, pre-packed in this order (ConvArgs::wslab), by one bulk copy.  The A operand of step
// (tap, chunk) of slab k is a descriptor into that copy: 8 x-consecutive voxels of one y row are a 128-byte core
// matrix, the slab's 16 rows follow at the row pitch (stride byte offset 160), and the chunk's upper 8 channels
// one plane further (leading byte offset).  A tap or a slab only moves the start address, so one thread issues
// all ZS x 27 x cin/16 MMAs back to back, slab k into TMEM columns k COUT .. k COUT + COUT - 1: no gathers
// between the MMAs and no split of the steps over CTAs.  M row m = TMEM lane m is voxel (x0 + m % 8, y0 + m / 8)
// of each slab.
// With ZS = 2 and `pool`, the epilogue also writes the 2x2x2 mean of the stored (BF16) outputs in k_pool's
// order (z, then y, then x), taking the x and y neighbours from lanes m ^ 1 and m ^ 8 of the same warp.
// ============================================================================================================
constexpr int kSlabX = 8, kSlabY = 16;
constexpr int kSlabHX = kSlabX + 2, kSlabHY = kSlabY + 2;
constexpr uint32_t kSlabRow = kSlabHX * 16;               // bytes of one brick row: the A stride byte offset
constexpr uint32_t kSlabZ = kSlabHY * kSlabRow;           // bytes of one z plane of one channel plane
__host__ __device__ constexpr int slab_vox(int zs) { return kSlabHX * kSlabHY * (zs + 2); }
// bytes of one 8-channel plane of the brick, padded to 128 (the alignment of a tensor copy's destination)
__host__ __device__ constexpr uint32_t slab_plane(int zs) { return ((uint32_t)slab_vox(zs) * 16 + 127) / 128 * 128; }
__host__ __device__ constexpr size_t slab_smem_bytes(int cin, int cout, int zs) {
    return (size_t)(cin / 8) * slab_plane(zs) + (size_t)27 * (cin / 16) * cout * 32 + 32;
}
__host__ __device__ constexpr bool slab_fits(int cin) { return cin == 16 || cin == 32 || cin == 64; }
__host__ __device__ constexpr long long slab_count(int W, int H, int D, int zs) {
    return (long long)((W + kSlabX - 1) / kSlabX) * ((H + kSlabY - 1) / kSlabY) * ((D + zs - 1) / zs);
}

// TMA maps of the input's 8-channel planes for k_conv3_slab (n = cin / 8 maps, box 8 x 10 x 18 x (ZS + 2) at
// (0, x0 - 1, y0 - 1, z0 - 1), zero outside the grid); n = 0: the brick is gathered by cp.async (the up-sampled
// inputs, which no tensor map describes)
struct SlabMaps {
    CUtensorMap map[8];
    int n;
};

template <int COUT, int ZS>
__global__ void __launch_bounds__(kConvThreads) k_conv3_slab(ConvArgs a, const __grid_constant__ SlabMaps m) {
    static_assert(COUT == 16 || COUT == 32 || COUT == 64, "COUT");
    static_assert(ZS == 1 || ZS == 2, "ZS");
    constexpr uint32_t kCols = ZS * COUT < 32 ? 32 : ZS * COUT;
    constexpr int kVox = slab_vox(ZS);
    constexpr uint32_t kPlane = slab_plane(ZS);            // bytes of one 8-channel plane of the brick
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int chunks = a.cin >> 4, planes = a.cin >> 3;
    const int S = 27 * chunks;
    unsigned char* brick = smem;
    unsigned char* wsm = smem + (size_t)planes * kPlane;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(wsm + (size_t)S * COUT * 32);   // [0] the MMAs, [1] the weights
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 2);
    const uint32_t wbytes = (uint32_t)S * COUT * 32;

    const int nsx = (a.W + kSlabX - 1) / kSlabX, nsy = (a.H + kSlabY - 1) / kSlabY;
    const int x0 = (blockIdx.x % nsx) * kSlabX, y0 = ((blockIdx.x / nsx) % nsy) * kSlabY;
    const int z0 = (blockIdx.x / (nsx * nsy)) * ZS;
    const bool tma = m.n == planes;
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // the packed weights (one bulk copy) and the brick's planes (one tensor load each), complete on mbar[1]
        // (a tensor load delivers its box, kVox x 16 bytes, into a plane padded to kPlane)
        const uint32_t tx = (a.wslab ? wbytes : 0u) + (tma ? (uint32_t)planes * (uint32_t)(kVox * 16) : 0u);
        if (tx) {
            mbar_expect_tx(&mbar[1], tx);
            if (a.wslab) bulk_load(wsm, a.wslab, wbytes, &mbar[1]);
            if (tma)
                for (int pl = 0; pl < planes; pl++)
                    tma_load_4d(brick + (size_t)pl * kPlane, &m.map[pl], 0, x0 - 1, y0 - 1, z0 - 1, &mbar[1]);
        }
    }
    const int PW = (a.W + 1) >> 1, PH = (a.H + 1) >> 1;

    // without tensor maps, the brick by cp.async: piece p = voxel * planes + plane (the planes of one voxel are
    // adjacent in global memory)
    const int pieces = tma ? 0 : kVox * planes;
    for (int p = tid; p < pieces; p += kConvThreads) {
        const int vox = p / planes, pl = p - vox * planes;
        const int hx = vox % kSlabHX, hy = (vox / kSlabHX) % kSlabHY, hz = vox / (kSlabHX * kSlabHY);
        const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
        const bool ok = gx >= 0 && gx < a.W && gy >= 0 && gy < a.H && gz >= 0 && gz < a.D;
        const int iv = a.up ? (((gz >> 1) * PH + (gy >> 1)) * PW + (gx >> 1)) : ((gz * a.H + gy) * a.W + gx);
        const __nv_bfloat16* src = ok ? a.in + ((size_t)iv * a.cin + pl * 8) : a.in;
        cp_async16(brick + (size_t)pl * kPlane + (size_t)vox * 16, src, ok);
    }
    // without packed weights: every step's weight tile in k_conv3_tc's B layout, step s's tile at s * COUT * 32
    // bytes, one 16-byte piece at a time
    const int wpieces = a.wslab ? 0 : S * COUT * 2;
    for (int q = tid; q < wpieces; q += kConvThreads) {
        const int s = q / (2 * COUT), r = q - s * 2 * COUT, n = r >> 1, kh = r & 1;
        cp_async16(wsm + (size_t)s * COUT * 32 + tile_off(n, kh * 8), a.wt + ((size_t)(s * COUT + n) * 16 + kh * 8),
                   true);
    }
    cp_async_commit();
    if (warp == 0) tmem_alloc(tslot, kCols);
    cp_async_wait<0>();
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    if (tid == 0) {
        // steps in k_conv3_tc's order: s = tap * chunks + chunk, tap = ((dz + 1) * 3 + dy + 1) * 3 + dx + 1
        const uint32_t b0 = smem_u32(brick), w0 = smem_u32(wsm);
        const int clog = __ffs(chunks) - 1;
        // the bulk and tensor copies (bounded); without them no MMA is issued, the error word says why, and the
        // commit below still completes mbar[0]
        const bool wok = !(a.wslab || tma) || mbar_wait(&mbar[1], 0);
        if (!wok) atomicOr(a.err, 1);
        tc_fence_after();
#pragma unroll
        for (int k = 0; k < (wok ? ZS : 0); k++) {
            for (int s = 0; s < S; s++) {
                const int tap = s >> clog, c = s & (chunks - 1);
                const int hz = tap / 9 + k, hy = (tap / 3) % 3, hx = tap % 3;   // the tap's offsets + 1, slab k
                const uint32_t aaddr = b0 + (uint32_t)(2 * c) * kPlane + (uint32_t)hz * kSlabZ + (uint32_t)hy * kSlabRow +
                                       (uint32_t)hx * 16;
                mma_bf16(tmem + (uint32_t)(k * COUT), sdesc(aaddr, kPlane, kSlabRow),
                         sdesc(w0 + (uint32_t)s * COUT * 32, 128, 256), idesc_bf16(128, COUT), s > 0 ? 1u : 0u);
            }
        }
        mma_commit(&mbar[0]);
    }
    bool ok = mbar_wait(&mbar[0], 0);
    if (!ok) {
        if (tid == 0) atomicOr(a.err, 1);
        // bounded: let MMAs in flight finish before freeing TMEM
        mbar_wait(&mbar[0], 0);
    }
    tc_fence_after();
    const int vx = x0 + (tid & 7), vy = y0 + (tid >> 3);
    if (ok) {
        const bool vin = vx < a.W && vy < a.H;
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        const bool pool = ZS == 2 && a.pool != nullptr;
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float st[ZS][16];   // the stored values, for the pooling
#pragma unroll
            for (int k = 0; k < ZS; k++) {
                float acc[16];
                tmem_ld16(tmem + lane_base + (uint32_t)(k * COUT + c0), acc);   // every lane of the warp takes part
                const bool in = vin && z0 + k < a.D;
                const size_t v = in ? ((size_t)(z0 + k) * a.H + vy) * a.W + vx : 0;
                __align__(16) __nv_bfloat16 o[16], pr[16];
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    float t = acc[j] + (a.bias ? a.bias[c0 + j] : 0.f);
                    pr[j] = __float2bfloat16(t);
                    if (a.relu) t = fmaxf(t, 0.f);
                    if (in && a.skip) t += __bfloat162float(a.skip[v * COUT + c0 + j]);
                    o[j] = __float2bfloat16(t);
                    st[k][j] = __bfloat162float(o[j]);
                    if (in && a.out32 && c0 + j == 0) a.out32[v] = t;
                }
                if (in && a.out) {
                    uint4* dst = reinterpret_cast<uint4*>(a.out + v * COUT + c0);
                    dst[0] = reinterpret_cast<const uint4*>(o)[0];
                    dst[1] = reinterpret_cast<const uint4*>(o)[1];
                }
                if (in && a.pre) {
                    uint4* dst = reinterpret_cast<uint4*>(a.pre + v * COUT + c0);
                    dst[0] = reinterpret_cast<const uint4*>(pr)[0];
                    dst[1] = reinterpret_cast<const uint4*>(pr)[1];
                }
            }
            if (pool) {
                // the pooled voxel of the lane at even (x, y): its own value, then x + 1, y + 1, x + 1 and y + 1,
                // for z0 and then z0 + 1, as k_pool sums them
                const bool hx1 = vx + 1 < a.W, hy1 = vy + 1 < a.H, hz1 = z0 + 1 < a.D;
                const float inv = 1.f / (float)((hx1 ? 2 : 1) * (hy1 ? 2 : 1) * (hz1 ? 2 : 1));
                __align__(16) __nv_bfloat16 po[16];
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    float sum = 0.f;
#pragma unroll
                    for (int k = 0; k < ZS; k++) {
                        const float sx = __shfl_xor_sync(0xffffffffu, st[k][j], 1);
                        const float sy = __shfl_xor_sync(0xffffffffu, st[k][j], 8);
                        const float sxy = __shfl_xor_sync(0xffffffffu, st[k][j], 9);
                        if (k == 1 && !hz1) continue;
                        sum += st[k][j];
                        if (hx1) sum += sx;
                        if (hy1) sum += sy;
                        if (hx1 && hy1) sum += sxy;
                    }
                    po[j] = __float2bfloat16(sum * inv);
                }
                if (vin && !(vx & 1) && !(vy & 1)) {
                    const size_t pv = ((size_t)(z0 >> 1) * PH + (vy >> 1)) * PW + (vx >> 1);
                    uint4* dst = reinterpret_cast<uint4*>(a.pool + pv * COUT + c0);
                    dst[0] = reinterpret_cast<const uint4*>(po)[0];
                    dst[1] = reinterpret_cast<const uint4*>(po)[1];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kCols);
}

// ============================================================================================================
// Weight gradient:  dw[tap][c][n] += sum_v in[v + off(tap)][c] * g[v][n]
// GEMM view: M = 27 * CIN rows (row = tap * CIN + c), tiles of 128 (blockIdx.x); N = COUT; K = voxels, in
// steps of 16, over the voxel range of blockIdx.y.  Operands are transposed into the K-major tiles with
// plain shared stores.  Each block adds its FP32 partial into dw with atomics.
// ============================================================================================================
struct WgradArgs {
    const __nv_bfloat16* in;   // [V][cin]
    const __nv_bfloat16* g;    // [V][COUT]
    float* dw;                 // [27 * cin][COUT] FP32, accumulated
    int D, H, W, cin;
    int vox_per_block;         // multiple of 16
    int* err;
};

template <int COUT>
__global__ void __launch_bounds__(kConvThreads) k_wgrad3_tc(WgradArgs a) {
    static_assert(COUT == 16 || COUT == 32 || COUT == 64, "COUT");
    constexpr int kABytes = 128 * 32, kBBytes = COUT * 32;
    constexpr uint32_t kCols = COUT < 32 ? 32 : COUT;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* bufA[2] = {smem, smem + kABytes};
    unsigned char* bufB[2] = {smem + 2 * kABytes, smem + 2 * kABytes + kBBytes};
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + 2 * kABytes + 2 * kBBytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 2);

    const int tid = threadIdx.x, warp = tid >> 5;
    const int V = a.D * a.H * a.W;
    const int rows = 27 * a.cin;
    const int row = blockIdx.x * 128 + tid;          // this thread's A row
    const bool rin = row < rows;
    const int tap = rin ? row / a.cin : 0, c = rin ? row - tap * a.cin : 0;
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const int v0 = blockIdx.y * a.vox_per_block;
    const int v1 = min(V, v0 + a.vox_per_block);
    const int S = (v1 > v0) ? (v1 - v0 + 15) / 16 : 0;

    if (warp == 0) tmem_alloc(tslot, kCols);
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    bool ok = true;
    for (int s = 0; s < S && ok; s++) {
        const int b = s & 1;
        const int vs = v0 + s * 16;
        // gather this step's operands into registers before waiting for the buffer
        __align__(16) __nv_bfloat16 av[16];
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int vv = vs + j;
            __nv_bfloat16 t = __float2bfloat16(0.f);
            if (rin && vv < v1) {
                const int x = vv % a.W, y = (vv / a.W) % a.H, z = vv / (a.W * a.H);
                const int nx = x + dx, ny = y + dy, nz = z + dz;
                if (nx >= 0 && nx < a.W && ny >= 0 && ny < a.H && nz >= 0 && nz < a.D)
                    t = a.in[(size_t)((nz * a.H + ny) * a.W + nx) * a.cin + c];
            }
            av[j] = t;
        }
        __align__(16) __nv_bfloat16 bv[16];
        if (tid < COUT) {
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int vv = vs + j;
                bv[j] = (vv < v1) ? a.g[(size_t)vv * COUT + tid] : __float2bfloat16(0.f);
            }
        }
        if (s >= 2 && !mbar_wait(&mbar[b], ((s - 2) >> 1) & 1)) { ok = false; break; }
        *reinterpret_cast<uint4*>(bufA[b] + tile_off(tid, 0)) = reinterpret_cast<const uint4*>(av)[0];
        *reinterpret_cast<uint4*>(bufA[b] + tile_off(tid, 8)) = reinterpret_cast<const uint4*>(av)[1];
        if (tid < COUT) {
            *reinterpret_cast<uint4*>(bufB[b] + tile_off(tid, 0)) = reinterpret_cast<const uint4*>(bv)[0];
            *reinterpret_cast<uint4*>(bufB[b] + tile_off(tid, 8)) = reinterpret_cast<const uint4*>(bv)[1];
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint64_t ad = sdesc(smem_u32(bufA[b]), 128, 256);
            const uint64_t bd = sdesc(smem_u32(bufB[b]), 128, 256);
            mma_bf16(tmem, ad, bd, idesc_bf16(128, COUT), s > 0 ? 1u : 0u);
            mma_commit(&mbar[b]);
        }
    }
    if (S > 0) {
        const int last = S - 1;
        if (ok && !mbar_wait(&mbar[last & 1], (last >> 1) & 1)) ok = false;
        if (ok && last >= 1 && !mbar_wait(&mbar[(last - 1) & 1], ((last - 1) >> 1) & 1)) ok = false;
        if (!ok) {
            if (tid == 0) atomicOr(a.err, 1);
            mbar_wait(&mbar[last & 1], (last >> 1) & 1);
        }
    }
    tc_fence_after();
    if (ok && S > 0) {
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            float acc[16];
            tmem_ld16(tmem + lane_base + (uint32_t)c0, acc);
            if (rin) {
#pragma unroll
                for (int j = 0; j < 16; j++) atomicAdd(&a.dw[(size_t)row * COUT + c0 + j], acc[j]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kCols);
}

// ============================================================================================================
// Halo-tile 3x3x3 convolution (k_conv3_halo_ws below): the same function as k_conv3_tc, for grids at least
// one tile wide.
// A CTA computes kHaloRows output rows (2 in y x 2 in z) of one 128-voxel segment along x.  Per 16 input
// channels it loads, with two TMA tensor copies (one per 8-channel group), the input box of
// 130 x 4 x 4 voxels that covers those rows and their one-voxel halo (zero outside the grid), and with one
// bulk copy the 27 weight tiles of those channels.  Every tap of every row is then one tcgen05.mma whose A
// operand starts at the tap's shifted voxel inside the box: shared memory holds each channel group as
// [z][y][x][8 channels], so 8 consecutive x voxels of one group are one 128-byte core matrix (SBO 128 B
// between voxel groups, LBO = one group plane between the two K halves).  Each input voxel is staged once
// per CTA instead of once per tap.  Row r accumulates in TMEM columns [r * COUT, (r + 1) * COUT).
// ============================================================================================================
constexpr int kHaloSeg = 128, kHaloX = kHaloSeg + 2, kHaloRY = 2, kHaloRZ = 2, kHaloRows = kHaloRY * kHaloRZ;
constexpr int kHaloBoxY = kHaloRY + 2, kHaloBoxZ = kHaloRZ + 2;
constexpr int kHaloPlane = 16 * kHaloX * kHaloBoxY * kHaloBoxZ;     // bytes of one 8-channel group box
constexpr int kHaloMaxGroups = 8;                                    // cin <= 64

struct HaloArgs {
    CUtensorMap map[kHaloMaxGroups];   // input group g: dims (8 channels, W, H, D), base in + 8 g
    const __nv_bfloat16* wh;           // [cin/16][27][COUT x 16 in the K-major core-matrix order]
    const float* bias;
    const __nv_bfloat16* skip;
    __nv_bfloat16* out;
    float* out32;                      // [V] FP32: output channel 0 only, or null
    __nv_bfloat16* pre;
    int D, H, W, cin;
    int relu;
    int* err;
};

// ---- persistent, warp-specialised halo convolution ---------------------------------------------------------
// One CTA per SM walking tiles blockIdx.x, blockIdx.x + gridDim.x, ...
// Roles: warp 0 (one lane) streams (tile, 16-channel chunk) items into kWsStages shared-memory stages with TMA;
// warp 1 (one lane) issues each item's 108 MMAs into one of two TMEM accumulator buffers; warps 2-5 (one per
// TMEM lane quarter) run a tile's epilogue while the next tile's MMAs run.  full/empty mbarriers hand stages
// between producer and MMA warp, acc_full/acc_empty accumulator buffers between MMA warp and epilogue.  Every
// wait is bounded and also gives up as soon as another role has given up (shared abort flag), so a failure
// ends the kernel within one wait limit; the MMA warp then drains its MMAs and the producer its copies before
// TMEM is freed.
constexpr int kWsThreads = 192;

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// mbar_wait that also returns false as soon as *abort is set; sets *abort itself when it gives up.
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, uint32_t parity, volatile int* abort) {
    if (mbar_test(bar, parity)) return true;
    const unsigned long long t0 = now_ns();
    while (!mbar_test(bar, parity)) {
        if (*abort) return false;
        if (now_ns() - t0 > kWaitNs) { *abort = 1; return false; }
    }
    return true;
}

template <int COUT> __host__ __device__ constexpr int ws_stages() { return COUT == 64 ? 1 : 2; }
template <int COUT> __host__ __device__ constexpr int ws_stage_bytes() { return 2 * kHaloPlane + 27 * COUT * 32; }
template <int COUT> __host__ __device__ constexpr int ws_smem_bytes() { return ws_stages<COUT>() * ws_stage_bytes<COUT>() + 128; }

template <int COUT>
__global__ void __launch_bounds__(kWsThreads, 1) k_conv3_halo_ws(const __grid_constant__ HaloArgs a) {
    static_assert(COUT == 16 || COUT == 32 || COUT == 64, "COUT");
    constexpr int S = ws_stages<COUT>();
    constexpr int kStage = ws_stage_bytes<COUT>();
    constexpr int kWBytes = 27 * COUT * 32;
    constexpr uint32_t kAcc = kHaloRows * COUT;       // TMEM columns of one accumulator buffer
    constexpr uint32_t kCols = 2 * kAcc;              // 128, 256 or 512
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * kStage);
    uint64_t* full = bars;              // [2]
    uint64_t* empty = bars + 2;         // [2]
    uint64_t* acc_full = bars + 4;      // [2]
    uint64_t* acc_empty = bars + 6;     // [2]
    uint64_t* drained = bars + 8;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 10);
    __shared__ int s_abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nx = (a.W + kHaloSeg - 1) / kHaloSeg, ny = (a.H + kHaloRY - 1) / kHaloRY;
    const int nz = (a.D + kHaloRZ - 1) / kHaloRZ;
    const int ntiles = nx * ny * nz;
    const int chunks = a.cin >> 4;
    const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    if (warp == 0) tmem_alloc(tslot, kCols);
    if (tid == 0) {
        for (int q = 0; q < 2; q++) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], 1);
            mbar_init(&acc_full[q], 1);
            mbar_init(&acc_empty[q], 4);
        }
        mbar_init(drained, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    volatile int* abort = &s_abort;
    auto origin = [&](int j, int& x0, int& y0, int& z0) {
        const int t = (int)blockIdx.x + j * (int)gridDim.x;
        x0 = (t % nx) * kHaloSeg;
        y0 = ((t / nx) % ny) * kHaloRY;
        z0 = (t / (nx * ny)) * kHaloRZ;
    };

    if (warp == 0 && lane == 0) {
        // ---- producer ----
        int k = 0;
        for (int j = 0; j < my_tiles && !*abort; j++) {
            int x0, y0, z0;
            origin(j, x0, y0, z0);
            bool ok = true;
            for (int c = 0; c < chunks; c++) {
                const int s = k % S;
                if (k >= S && !mbar_wait_or_abort(&empty[s], ((k / S) - 1) & 1, abort)) { ok = false; break; }
                unsigned char* box = smem + s * kStage;
                mbar_expect_tx(&full[s], 2 * kHaloPlane + kWBytes);
                tma_load_4d(box, &a.map[2 * c], 0, x0 - 1, y0 - 1, z0 - 1, &full[s]);
                tma_load_4d(box + kHaloPlane, &a.map[2 * c + 1], 0, x0 - 1, y0 - 1, z0 - 1, &full[s]);
                bulk_load(box + 2 * kHaloPlane, a.wh + (size_t)c * 27 * COUT * 16, kWBytes, &full[s]);
                k++;
            }
            if (!ok) break;
        }
        // the last S items' copies have landed before the CTA may exit (bounded; no-ops when consumed)
        for (int q = k - S; q < k; q++)
            if (q >= 0) mbar_wait(&full[q % S], (q / S) & 1);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issue ----
        int k = 0;
        for (int j = 0; j < my_tiles && !*abort; j++) {
            const int ab = j & 1;
            if (j >= 2 && !mbar_wait_or_abort(&acc_empty[ab], ((j / 2) - 1) & 1, abort)) break;
            tc_fence_after();
            const uint32_t acc = tmem + (uint32_t)ab * kAcc;
            bool ok = true;
            for (int c = 0; c < chunks; c++) {
                const int s = k % S;
                if (!mbar_wait_or_abort(&full[s], (k / S) & 1, abort)) { ok = false; break; }
                tc_fence_after();
                const uint32_t sbox = smem_u32(smem + s * kStage), swts = sbox + 2 * kHaloPlane;
                // all 108 operand addresses are constant offsets from the two base descriptors (the start
                // address field is addr >> 4 and shared memory stays below 256 KB, so the addition cannot carry)
                const uint64_t abase = sdesc(sbox, (uint32_t)kHaloPlane, 128), bbase = sdesc(swts, 128, 256);
                const uint32_t first = c > 0 ? 1u : 0u;
#pragma unroll
                for (int r = 0; r < kHaloRows; r++) {
#pragma unroll
                    for (int tap = 0; tap < 27; tap++) {
                        const int ry = r % kHaloRY, rz = r / kHaloRY;
                        const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
                        const uint32_t off = (uint32_t)((((rz + dz) * kHaloBoxY + (ry + dy)) * kHaloX + dx) * 16);
                        mma_bf16(acc + (uint32_t)(r * COUT), abase + (off >> 4), bbase + (uint32_t)((tap * COUT * 32) >> 4),
                                 idesc_bf16(128, COUT), tap > 0 ? 1u : first);
                    }
                }
                mma_commit(&empty[s]);
                k++;
            }
            if (!ok) break;
            mma_commit(&acc_full[ab]);
        }
        mma_commit(drained);                 // arrives when every MMA issued above has completed
        mbar_wait(drained, 0);
    } else if (warp >= 2) {
        // ---- epilogue: warp w reads TMEM lanes 32 * (w % 4) .. + 31 ----
        const int quarter = warp & 3;
        const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
        for (int j = 0; j < my_tiles; j++) {
            const int ab = j & 1;
            if (!mbar_wait_or_abort(&acc_full[ab], (j / 2) & 1, abort)) break;
            tc_fence_after();
            int x0, y0, z0;
            origin(j, x0, y0, z0);
            const int x = x0 + quarter * 32 + lane;
#pragma unroll 1
            for (int r = 0; r < kHaloRows; r++) {
                const int y = y0 + r % kHaloRY, z = z0 + r / kHaloRY;
                const bool vin = x < a.W && y < a.H && z < a.D;
                const size_t v = ((size_t)z * a.H + y) * a.W + x;
#pragma unroll
                for (int c0 = 0; c0 < COUT; c0 += 16) {
                    float accv[16];
                    tmem_ld16(tmem + lane_base + (uint32_t)ab * kAcc + (uint32_t)(r * COUT + c0), accv);
                    if (vin) {
                        __align__(16) __nv_bfloat16 o[16], pr[16];
#pragma unroll
                        for (int q = 0; q < 16; q++) {
                            float t = accv[q] + (a.bias ? a.bias[c0 + q] : 0.f);
                            pr[q] = __float2bfloat16(t);
                            if (a.relu) t = fmaxf(t, 0.f);
                            if (a.skip) t += __bfloat162float(a.skip[v * COUT + c0 + q]);
                            o[q] = __float2bfloat16(t);
                            if (a.out32 && c0 + q == 0) a.out32[v] = t;
                        }
                        if (a.out) {
                            uint4* dst = reinterpret_cast<uint4*>(a.out + v * COUT + c0);
                            dst[0] = reinterpret_cast<const uint4*>(o)[0];
                            dst[1] = reinterpret_cast<const uint4*>(o)[1];
                        }
                        if (a.pre) {
                            uint4* dst = reinterpret_cast<uint4*>(a.pre + v * COUT + c0);
                            dst[0] = reinterpret_cast<const uint4*>(pr)[0];
                            dst[1] = reinterpret_cast<const uint4*>(pr)[1];
                        }
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[ab]);
        }
    }
    __syncthreads();
    if (tid == 0 && *abort) atomicOr(a.err, 1);
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, kCols);
}

// Weights wt[tap][cin/16][cout][16] (the k_conv3_tc layout) -> wh[cin/16][27][core-matrix tile of cout x 16].
__global__ void k_pack_halo_weights(const __nv_bfloat16* __restrict__ wt, int cin, int cout, __nv_bfloat16* __restrict__ wh) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 27 * cin * cout) return;
    const int chunks = cin >> 4;
    const int k = i & 15, n = (i >> 4) % cout, cc = (i / (16 * cout)) % chunks, tap = i / (16 * cout * chunks);
    const size_t dst = ((size_t)cc * 27 + tap) * cout * 16 + tile_off(n, k) / 2;
    wh[dst] = wt[i];
}

}  // namespace tc
}  // namespace efs
