// efs_unet.cu — the learned preconditioner: a 3-level 3D convolutional U-Net (16/32/64 channels, BF16
// weights and activations, FP32 accumulation in tensor memory) and its training on the GPU with the
// project's own forward and backward kernels.  FCG applies it as the coarsest-level solve of its multilevel
// preconditioner (efs_mlfcg.cu).
//
// No counterpart in the reference (its solvers are CGSolverCPU3D / JacobiSolverCPU3D,
// src/simulation/solver/CGSolver.cpp:416-497, JacobiSolver.cpp:154-212).
//
// The network works on one level of FCG's hierarchy (the bottom one; level 0 is the pressure matrix's own
// grid).  Network (all convolutions 3x3x3, zero padding; network level k has that grid's dimensions halved k
// times, rounded up):
//   x0  = [r / rms(r), row mask, geometry, 0...]          network level 0, 16 channels (BF16); geometry (only
//                                                        above hierarchy level 0): -diag / (6 4^l) and the six
//                                                        face weights / 4^l of the level-l matrix
//   e0  = relu(conv0(x0))            16 -> 16              level 0
//   e1  = relu(conv1(pool(e0)))      16 -> 32              level 1 (pool: 2x2x2 mean)
//   e2  = relu(conv2(pool(e1)))      32 -> 64              level 2
//   d1  = relu(conv3(up(e2))) + e1   64 -> 32              level 1 (up: nearest)
//   d0  = relu(conv4(up(d1))) + e0   32 -> 16              level 0
//   y   = conv5(d0)[channel 0]       16 -> 16 (FP32)       level 0
// Parameters: layer k's weights w[tap][cin][cout] then its bias[cout], layers in order (FP32 master copy;
// BF16 copies in the tcgen05 operand layouts).  The preconditioner is z = y on matrix rows, 0 elsewhere.
// FCG is invariant to the scale of z, so neither the input normalisation nor the output scale matters to it.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "efs_internal.h"
#include "efs_tc.cuh"

using bf16 = __nv_bfloat16;

namespace efs {

namespace {

constexpr int kLayers = 6;
struct LayerSpec {
    int cin, cout, level;
};
constexpr LayerSpec kSpec[kLayers] = {{16, 16, 0}, {16, 32, 1}, {32, 64, 2}, {64, 32, 1}, {32, 16, 0}, {16, 16, 0}};

long long param_count_host() {
    long long n = 0;
    for (const auto& s : kSpec) n += 27LL * s.cin * s.cout + s.cout;
    return n;
}

struct Level {
    int D, H, W;
    long long V;
};

}  // namespace

struct UNetState {
    int level = 0;               // hierarchy level the network works on (0: the context's grid)
    int sm = 0;                  // SMs of the device (the split convolutions' target CTA count)
    int slab_smem = 0;           // dynamic shared memory k_conv3_slab may take (0: the slab kernel is not used)
    float* split = nullptr;      // FP32 partial sums of split convolutions
    long long split_cap = 0;     // floats in split
    Level L[3];
    long long woff[kLayers], boff[kLayers], nparam = 0;
    float *w32 = nullptr, *grad = nullptr, *am = nullptr, *av = nullptr;
    int adam_t = 0;
    bf16 *wf[kLayers] = {}, *wb[kLayers] = {};
    bf16 *wsf[kLayers] = {}, *wsb[kLayers] = {};   // wf, wb in k_conv3_slab's shared-memory order
    bf16* wh = nullptr;          // weights of the convolution in flight, packed for k_conv3_halo_ws
    // activations (level of each in brackets)
    bf16 *x0 = nullptr, *e0 = nullptr, *p0 = nullptr, *e1 = nullptr, *p1 = nullptr, *e2 = nullptr, *u2 = nullptr,
         *d1 = nullptr, *u1 = nullptr, *d0 = nullptr;
    float* y32 = nullptr;        // network output, channel 0 (FP32)
    // training: pre-activations and gradients
    bool train_ready = false;
    bf16 *a0 = nullptr, *a1 = nullptr, *a2 = nullptr, *a3 = nullptr, *a4 = nullptr;
    bf16 *g5 = nullptr, *gd0 = nullptr, *ga4 = nullptr, *gu1 = nullptr, *gd1 = nullptr, *ga3 = nullptr, *gu2 = nullptr,
         *ge2 = nullptr, *ga2 = nullptr, *gp1 = nullptr, *ge1 = nullptr, *ga1 = nullptr, *gp0 = nullptr, *ge0 = nullptr,
         *ga0 = nullptr;
    // scalars and reductions
    double* dscal = nullptr;     // [0] sum, [1] count, [2] 1/rms (input); [3..5] the same for the target; [8..10] dots
    double* dpart = nullptr;     // block partials
    double* dloss = nullptr;     // [0] loss
    int* err = nullptr;
    // training set per sample: input r, its exact correction e (A e = r), row info and, above level 0, the
    // level's matrix (face weights, diagonal)
    int cap = 0, count = 0, next = 0;
    float *sb = nullptr, *sp = nullptr;
    uint16_t* srow = nullptr;
    uint8_t* sw = nullptr;
    float* sdiag = nullptr;
    float* tmp_in = nullptr;     // one scalar field: input staging
    float* tmp_t = nullptr;
    float *tz = nullptr, *tq = nullptr;   // training: z = net output and L z (energy loss)
    float *c1 = nullptr, *c2 = nullptr, *c3 = nullptr;   // bottom-level CG vectors (training samples)
    std::vector<void*> allocs;
};

namespace {

constexpr int kRedBlocks = 512;

// ---- small kernels -------------------------------------------------------------------------------------------
// sum of x^2 and count over matrix rows -> block partials [2 * blockIdx]
__global__ void k_sumsq_rows(const float* __restrict__ x, const uint16_t* __restrict__ rowinfo, long long n,
                             double* __restrict__ part) {
    double s = 0, c = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (rowinfo[i] & 0x8000u) {
            const double v = x[i];
            s += v * v;
            c += 1;
        }
    }
    __shared__ double ss[256], sc[256];
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) { ss[threadIdx.x] += ss[threadIdx.x + o]; sc[threadIdx.x] += sc[threadIdx.x + o]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = ss[0]; part[2 * blockIdx.x + 1] = sc[0]; }
}
// out[0] = sum, out[1] = count, out[2] = 1 / sqrt(sum / count) (1 when the sum is 0)
__global__ void k_finish_scale(const double* __restrict__ part, int nb, double* __restrict__ out) {
    __shared__ double ss[256], sc[256];
    double s = 0, c = 0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) { s += part[2 * b]; c += part[2 * b + 1]; }
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) { ss[threadIdx.x] += ss[threadIdx.x + o]; sc[threadIdx.x] += sc[threadIdx.x + o]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = ss[0];
        out[1] = sc[0];
        out[2] = (ss[0] > 0 && sc[0] > 0) ? 1.0 / sqrt(ss[0] / sc[0]) : 1.0;
    }
}

// x0[v] = [r * inv, mask, geometry, 0...] on rows, 0 elsewhere; geometry (gw non-null: a level above 0) is
// -diag * gnorm / 6 and the six face weights * gnorm, gnorm = 4^-level
__global__ void k_pack(const float* __restrict__ r, const uint16_t* __restrict__ rowinfo, const double* __restrict__ scal,
                       long long n, bf16* __restrict__ x0, const uint8_t* __restrict__ gw, const float* __restrict__ gdiag,
                       float gnorm) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= n) return;
    const bool row = rowinfo[v] & 0x8000u;
    __align__(16) bf16 o[16];
#pragma unroll
    for (int j = 0; j < 16; j++) o[j] = __float2bfloat16(0.f);
    if (row) {
        o[0] = __float2bfloat16((float)((double)r[v] * scal[2]));
        o[1] = __float2bfloat16(1.f);
        if (gw) {
            o[2] = __float2bfloat16(-gdiag[v] * gnorm * (1.f / 6.f));
#pragma unroll
            for (int k = 0; k < 6; k++) o[3 + k] = __float2bfloat16((float)gw[k * n + v] * gnorm);
        }
    }
    uint4* dst = reinterpret_cast<uint4*>(x0 + v * 16);
    dst[0] = reinterpret_cast<const uint4*>(o)[0];
    dst[1] = reinterpret_cast<const uint4*>(o)[1];
}

__device__ __forceinline__ void unpack8(uint4 u, float (&f)[8]) {
    const bf16* b = reinterpret_cast<const bf16*>(&u);
#pragma unroll
    for (int j = 0; j < 8; j++) f[j] = __bfloat162float(b[j]);
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
    __align__(16) bf16 b[8];
#pragma unroll
    for (int j = 0; j < 8; j++) b[j] = __float2bfloat16(f[j]);
    return *reinterpret_cast<const uint4*>(b);
}

// 2x2x2 mean over the children that exist; one thread per (parent voxel, 8 channels)
__global__ void k_pool(const bf16* __restrict__ in, Level lc, bf16* __restrict__ out, Level lp, int C) {
    const int g8 = C / 8;
    const long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (item >= lp.V * g8) return;
    const long long pv = item / g8;
    const int g = (int)(item - pv * g8);
    const int px = (int)(pv % lp.W), py = (int)((pv / lp.W) % lp.H), pz = (int)(pv / ((long long)lp.W * lp.H));
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int cnt = 0;
    for (int dz = 0; dz < 2; dz++)
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                const int x = 2 * px + dx, y = 2 * py + dy, z = 2 * pz + dz;
                if (x >= lc.W || y >= lc.H || z >= lc.D) continue;
                float f[8];
                unpack8(*reinterpret_cast<const uint4*>(in + (((long long)z * lc.H + y) * lc.W + x) * C + g * 8), f);
#pragma unroll
                for (int j = 0; j < 8; j++) acc[j] += f[j];
                cnt++;
            }
    const float inv = 1.f / (float)cnt;
#pragma unroll
    for (int j = 0; j < 8; j++) acc[j] *= inv;
    *reinterpret_cast<uint4*>(out + pv * C + g * 8) = pack8(acc);
}
// nearest up-sampling: out[child] = in[parent]
__global__ void k_up(const bf16* __restrict__ in, Level lp, bf16* __restrict__ out, Level lc, int C) {
    const int g8 = C / 8;
    const long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (item >= lc.V * g8) return;
    const long long v = item / g8;
    const int g = (int)(item - v * g8);
    const int x = (int)(v % lc.W), y = (int)((v / lc.W) % lc.H), z = (int)(v / ((long long)lc.W * lc.H));
    const long long pv = ((long long)(z >> 1) * lp.H + (y >> 1)) * lp.W + (x >> 1);
    *reinterpret_cast<uint4*>(out + v * C + g * 8) = *reinterpret_cast<const uint4*>(in + pv * C + g * 8);
}
// gradient of k_up: parent gets the sum of its children's gradients
__global__ void k_up_bwd(const bf16* __restrict__ gc, Level lc, bf16* __restrict__ gp, Level lp, int C) {
    const int g8 = C / 8;
    const long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (item >= lp.V * g8) return;
    const long long pv = item / g8;
    const int g = (int)(item - pv * g8);
    const int px = (int)(pv % lp.W), py = (int)((pv / lp.W) % lp.H), pz = (int)(pv / ((long long)lp.W * lp.H));
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dz = 0; dz < 2; dz++)
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) {
                const int x = 2 * px + dx, y = 2 * py + dy, z = 2 * pz + dz;
                if (x >= lc.W || y >= lc.H || z >= lc.D) continue;
                float f[8];
                unpack8(*reinterpret_cast<const uint4*>(gc + (((long long)z * lc.H + y) * lc.W + x) * C + g * 8), f);
#pragma unroll
                for (int j = 0; j < 8; j++) acc[j] += f[j];
            }
    *reinterpret_cast<uint4*>(gp + pv * C + g * 8) = pack8(acc);
}
// gradient of k_pool: child gets parent's gradient / (parent's child count), plus an optional skip gradient
__global__ void k_pool_bwd(const bf16* __restrict__ gp, Level lp, bf16* __restrict__ gc, Level lc, int C,
                           const bf16* __restrict__ skip) {
    const int g8 = C / 8;
    const long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (item >= lc.V * g8) return;
    const long long v = item / g8;
    const int g = (int)(item - v * g8);
    const int x = (int)(v % lc.W), y = (int)((v / lc.W) % lc.H), z = (int)(v / ((long long)lc.W * lc.H));
    const int px = x >> 1, py = y >> 1, pz = z >> 1;
    const int nx = min(2, lc.W - 2 * px), ny = min(2, lc.H - 2 * py), nz = min(2, lc.D - 2 * pz);
    const float inv = 1.f / (float)(nx * ny * nz);
    float f[8];
    unpack8(*reinterpret_cast<const uint4*>(gp + (((long long)pz * lp.H + py) * lp.W + px) * C + g * 8), f);
#pragma unroll
    for (int j = 0; j < 8; j++) f[j] *= inv;
    if (skip) {
        float s[8];
        unpack8(*reinterpret_cast<const uint4*>(skip + v * C + g * 8), s);
#pragma unroll
        for (int j = 0; j < 8; j++) f[j] += s[j];
    }
    *reinterpret_cast<uint4*>(gc + v * C + g * 8) = pack8(f);
}
// out = g where pre > 0, else 0
__global__ void k_relu_bwd(const bf16* __restrict__ g, const bf16* __restrict__ pre, long long n8, bf16* __restrict__ out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n8) return;
    float f[8], p[8];
    unpack8(reinterpret_cast<const uint4*>(g)[i], f);
    unpack8(reinterpret_cast<const uint4*>(pre)[i], p);
#pragma unroll
    for (int j = 0; j < 8; j++) f[j] = p[j] > 0.f ? f[j] : 0.f;
    reinterpret_cast<uint4*>(out)[i] = pack8(f);
}
// db[c] += sum over voxels of g[v][c]
__global__ void k_bias_grad(const bf16* __restrict__ g, long long V, int C, float* __restrict__ db) {
    __shared__ float acc[256];
    const int lanes = 256 / C;                           // voxels processed side by side per block
    const int c = threadIdx.x % C, l = threadIdx.x / C;
    float s = 0.f;
    for (long long v = blockIdx.x * (long long)lanes + l; v < V; v += (long long)gridDim.x * lanes)
        s += __bfloat162float(g[v * C + c]);
    acc[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.f;
        for (int k = 0; k < lanes; k++) t += acc[k * C + threadIdx.x];
        atomicAdd(&db[threadIdx.x], t);
    }
}
// loss = sum_rows (y - t)^2 / rows with t = p / rms(p); g5 = dloss/dy (channel 0), 0 on the other channels
__global__ void k_loss(const float* __restrict__ y32, const float* __restrict__ p, const uint16_t* __restrict__ rowinfo,
                       const double* __restrict__ tscal, long long n, bf16* __restrict__ g5, double* __restrict__ part) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double l = 0;
    __align__(16) bf16 o[16];
#pragma unroll
    for (int j = 0; j < 16; j++) o[j] = __float2bfloat16(0.f);
    if (v < n) {
        if (rowinfo[v] & 0x8000u) {
            const double t = (double)p[v] * tscal[2];
            const double d = (double)y32[v] - t;
            l = d * d;
            o[0] = __float2bfloat16((float)(2.0 * d / tscal[1]));
        }
        uint4* dst = reinterpret_cast<uint4*>(g5 + v * 16);
        dst[0] = reinterpret_cast<const uint4*>(o)[0];
        dst[1] = reinterpret_cast<const uint4*>(o)[1];
    }
    __shared__ double s[256];
    s[threadIdx.x] = l;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}
// Energy-norm alignment loss of the preconditioner output z (channel 0 of y32, on rows) for input r and
// error e (L e = r):  loss = 1 - (z.r)^2 / ((z.Lz) (e.r)), the fraction of the error's energy norm that a
// line search along z leaves.  dots = (a, c, k) = (z.r, z.Lz, e.r); q = L z.
__global__ void k_energy_grad(const float* __restrict__ r, const float* __restrict__ q, const uint16_t* __restrict__ rowinfo,
                              const double* __restrict__ dots, long long n, bf16* __restrict__ g5) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= n) return;
    __align__(16) bf16 o[16];
#pragma unroll
    for (int j = 0; j < 16; j++) o[j] = __float2bfloat16(0.f);
    const double a = dots[0], cz = dots[1], k = dots[2];
    if ((rowinfo[v] & 0x8000u) && cz != 0.0 && k != 0.0) {
        const double g = -2.0 * a / (cz * k) * (double)r[v] + 2.0 * a * a / (cz * cz * k) * (double)q[v];
        o[0] = __float2bfloat16((float)g);
    }
    uint4* dst = reinterpret_cast<uint4*>(g5 + v * 16);
    dst[0] = reinterpret_cast<const uint4*>(o)[0];
    dst[1] = reinterpret_cast<const uint4*>(o)[1];
}
__global__ void k_energy_loss(const double* __restrict__ dots, double* __restrict__ out) {
    const double a = dots[0], cz = dots[1], k = dots[2];
    out[0] += (cz != 0.0 && k != 0.0) ? 1.0 - a * a / (cz * k) : 1.0;
}

__global__ void k_sum_partials(const double* __restrict__ part, int nb, const double* __restrict__ tscal, double* out) {
    __shared__ double s[256];
    double a = 0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) a += part[b];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] += (tscal[1] > 0 ? s[0] / tscal[1] : 0.0);
}
// FP32 master weights -> BF16 operand layouts: forward wf[tap][cin/16][cout][16]; input gradient
// wb[tap'][cout/16][cin][16] with tap' = 26 - tap (negated offsets) and the channel roles swapped.
// wf: the forward weights [tap][cin/16][cout][16]; wb: the input gradient's (taps flipped, cin and cout swapped)
// [26 - tap][cout/16][cin][16]; wsf, wsb: the same as k_conv3_slab keeps them in shared memory, step s's
// K-major no-swizzle B tile (rows = output channels) at s * rows * 16 elements
__global__ void k_w_to_bf16(const float* __restrict__ w, int cin, int cout, bf16* __restrict__ wf, bf16* __restrict__ wb,
                            bf16* __restrict__ wsf, bf16* __restrict__ wsb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 27 * cin * cout) return;
    const int co = i % cout, ci = (i / cout) % cin, tap = i / (cout * cin);
    const bf16 v = __float2bfloat16(w[i]);
    const size_t sf = (size_t)tap * (cin / 16) + ci / 16, sb = (size_t)(26 - tap) * (cout / 16) + co / 16;
    wf[(sf * cout + co) * 16 + ci % 16] = v;
    wb[(sb * cin + ci) * 16 + co % 16] = v;
    wsf[sf * cout * 16 + tc::tile_off(co, ci % 16) / 2] = v;
    wsb[sb * cin * 16 + tc::tile_off(ci, co % 16) / 2] = v;
}
__global__ void k_adam(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2, float gscale) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * gscale;
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}
// He-normal initial weights from a counter-based hash (Box-Muller), biases 0
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__global__ void k_init(float* __restrict__ w, long long n, long long nw, float stdv, unsigned long long seed,
                       unsigned long long salt) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i >= nw) { w[i] = 0.f; return; }
    const unsigned long long h = mix64(seed ^ (salt << 32) ^ (unsigned long long)i);
    const double u1 = ((h >> 11) + 1.0) * (1.0 / 9007199254740993.0);
    const double u2 = (mix64(h) >> 11) * (1.0 / 9007199254740992.0);
    w[i] = (float)(stdv * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
}
// Synthetic training pair: a random error field e on the rows, the sum over lattice spacings s of
// amp[k] * (trilinear interpolation of hash values on the lattice of spacing s); r = L e is formed after.
__device__ __forceinline__ float lattice_value(unsigned long long seed, int k, int ix, int iy, int iz) {
    const unsigned long long h = mix64(seed ^ ((unsigned long long)k << 56) ^ ((unsigned long long)(unsigned)ix << 36) ^
                                       ((unsigned long long)(unsigned)iy << 18) ^ (unsigned long long)(unsigned)iz);
    return (float)((h >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
}
struct SynthAmp {
    float a[5];
};
__global__ void k_synth_error(Level L, const uint16_t* __restrict__ rowinfo, unsigned long long seed, SynthAmp amp,
                              float* __restrict__ e) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= L.V) return;
    if (!(rowinfo[v] & 0x8000u)) { e[v] = 0.f; return; }
    const int x = (int)(v % L.W), y = (int)((v / L.W) % L.H), z = (int)(v / ((long long)L.W * L.H));
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int s = 1 << k;
        const float fx = (float)x / s, fy = (float)y / s, fz = (float)z / s;
        const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
        const float tx = fx - ix, ty = fy - iy, tz = fz - iz;
        float c = 0.f;
#pragma unroll
        for (int corner = 0; corner < 8; corner++) {
            const int dx = corner & 1, dy = (corner >> 1) & 1, dz = corner >> 2;
            const float w = (dx ? tx : 1.f - tx) * (dy ? ty : 1.f - ty) * (dz ? tz : 1.f - tz);
            c += w * lattice_value(seed, k, ix + dx, iy + dy, iz + dz);
        }
        acc += amp.a[k] * c;
    }
    e[v] = acc;
}

// z = y (channel 0) on rows, 0 elsewhere
__global__ void k_unpack(const float* __restrict__ y32, const uint16_t* __restrict__ rowinfo, long long n, float* __restrict__ z) {
    const long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (v >= n) return;
    z[v] = (rowinfo[v] & 0x8000u) ? y32[v] : 0.f;
}

// three dot products at once (pairs (a0,b0), (a1,b1), (a2,b2); null pairs give 0) -> block partials
__global__ void k_dots3(const float* a0, const float* b0, const float* a1, const float* b1, const float* a2, const float* b2,
                        long long n, double* __restrict__ part) {
    double s0 = 0, s1 = 0, s2 = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (a0) s0 += (double)a0[i] * b0[i];
        if (a1) s1 += (double)a1[i] * b1[i];
        if (a2) s2 += (double)a2[i] * b2[i];
    }
    __shared__ double sh[3][256];
    sh[0][threadIdx.x] = s0;
    sh[1][threadIdx.x] = s1;
    sh[2][threadIdx.x] = s2;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + k];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + k];
            sh[2][threadIdx.x] += sh[2][threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = sh[0][0];
        part[3 * blockIdx.x + 1] = sh[1][0];
        part[3 * blockIdx.x + 2] = sh[2][0];
    }
}
__global__ void k_dots3_finish(const double* __restrict__ part, int nb, double* __restrict__ out) {
    __shared__ double sh[3][256];
    double s0 = 0, s1 = 0, s2 = 0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) { s0 += part[3 * b]; s1 += part[3 * b + 1]; s2 += part[3 * b + 2]; }
    sh[0][threadIdx.x] = s0;
    sh[1][threadIdx.x] = s1;
    sh[2][threadIdx.x] = s2;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) {
            sh[0][threadIdx.x] += sh[0][threadIdx.x + k];
            sh[1][threadIdx.x] += sh[1][threadIdx.x + k];
            sh[2][threadIdx.x] += sh[2][threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[0] = sh[0][0]; out[1] = sh[1][0]; out[2] = sh[2][0]; }
}
// ---- host helpers -------------------------------------------------------------------------------------------
inline unsigned nblk(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

template <typename T>
cudaError_t ualloc(UNetState* u, T** p, long long count) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), (size_t)count * sizeof(T));
    if (e == cudaSuccess) u->allocs.push_back(*p);
    return e;
}

// network level l of a network on hierarchy level `base` (grid sides halved base + l times, rounded up)
Level level_of(const efs_ctx* c, int base, int l) {
    Level L{c->g.D, c->g.H, c->g.W, 0};
    for (int k = 0; k < base + l; k++) L = Level{(L.D + 1) / 2, (L.H + 1) / 2, (L.W + 1) / 2, 0};
    L.V = (long long)L.D * L.H * L.W;
    return L;
}


// cuTensorMapEncodeTiled from the driver, through the runtime (no link against the driver library).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// Grids this wide or wider use the halo-tile convolution (a CTA covers 128 voxels along x).
constexpr int kHaloMinWidth = 96;

template <int COUT>
cudaError_t launch_halo(const tc::HaloArgs& a, int W, int H, int D, int sm_count, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(tc::k_conv3_halo_ws<COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             tc::ws_smem_bytes<COUT>());
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long long tiles = (long long)((W + tc::kHaloSeg - 1) / tc::kHaloSeg) * ((H + tc::kHaloRY - 1) / tc::kHaloRY) *
                            ((D + tc::kHaloRZ - 1) / tc::kHaloRZ);
    const unsigned grid = (unsigned)std::max(1LL, std::min<long long>(tiles, sm_count));
    tc::k_conv3_halo_ws<COUT><<<grid, tc::kWsThreads, tc::ws_smem_bytes<COUT>(), st>>>(a);
    return cudaGetLastError();
}

cudaError_t conv_halo(UNetState* u, const bf16* in, const bf16* wt, int cin, int cout, const Level& L, const float* bias,
                      const bf16* skip, bf16* out, float* out32, bf16* pre, int relu, cudaStream_t st) {
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return cudaErrorNotSupported;
    const int n = 27 * cin * cout;
    tc::k_pack_halo_weights<<<nblk(n), 256, 0, st>>>(wt, cin, cout, u->wh);
    const cudaError_t pe = cudaGetLastError();
    if (pe != cudaSuccess) return pe;
    tc::HaloArgs a;
    std::memset(&a, 0, sizeof(a));
    // input channel group g: (8 channels, W, H, D) at in + 8 g; strides in bytes include the channel padding
    const cuuint64_t dims[4] = {8, (cuuint64_t)L.W, (cuuint64_t)L.H, (cuuint64_t)L.D};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)L.W * cin * 2, (cuuint64_t)L.H * L.W * cin * 2};
    const cuuint32_t boxd[4] = {8, (cuuint32_t)tc::kHaloX, (cuuint32_t)tc::kHaloBoxY, (cuuint32_t)tc::kHaloBoxZ};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    for (int g = 0; g < cin / 8; g++) {
        const CUresult r = encode(&a.map[g], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)(in + 8 * g), dims, strides, boxd,
                                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    }
    a.wh = u->wh;
    a.bias = bias; a.skip = skip; a.out = out; a.out32 = out32; a.pre = pre;
    a.D = L.D; a.H = L.H; a.W = L.W; a.cin = cin; a.relu = relu; a.err = u->err;
    int sm_count = 0;
    cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, 0);
    if (cout == 16) return launch_halo<16>(a, L.W, L.H, L.D, sm_count, st);
    if (cout == 32) return launch_halo<32>(a, L.W, L.H, L.D, sm_count, st);
    return launch_halo<64>(a, L.W, L.H, L.D, sm_count, st);
}

// k_conv3_slab's shared memory ceiling: the device's opt-in maximum per block, set once for every instantiation
// (outside any stream capture)
cudaError_t slab_setup(UNetState* u) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(tc::k_conv3_slab<16, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(tc::k_conv3_slab<32, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(tc::k_conv3_slab<64, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(tc::k_conv3_slab<16, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(tc::k_conv3_slab<32, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e == cudaSuccess) u->slab_smem = optin;
    return e;
}

// k_conv3_slab's tensor maps of `in` (channels-last, cin channels on level L): plane g covers channels 8 g ..
// 8 g + 7; the box is one slab's brick.  Left empty (maps->n = 0, the kernel then gathers by cp.async) when the
// driver's encoder is unavailable or refuses a map.
void slab_maps(const bf16* in, int cin, const Level& L, int zs, tc::SlabMaps* maps) {
    maps->n = 0;
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode || cin / 8 > 8) return;
    const cuuint64_t dims[4] = {8, (cuuint64_t)L.W, (cuuint64_t)L.H, (cuuint64_t)L.D};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)L.W * cin * 2, (cuuint64_t)L.H * L.W * cin * 2};
    const cuuint32_t boxd[4] = {8, (cuuint32_t)tc::kSlabHX, (cuuint32_t)tc::kSlabHY, (cuuint32_t)(zs + 2)};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    for (int g = 0; g < cin / 8; g++) {
        const CUresult r = encode(&maps->map[g], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void*)(in + 8 * g), dims, strides,
                                  boxd, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return;
    }
    maps->n = cin / 8;
}

// whether the level's convolution of cin input channels runs below the halo-tile kernel (the slab kernel, or
// the implicit-GEMM one where the slab does not fit).  Wide levels take the halo-tile kernel for 32 and 64 input
// channels; with 16 the slab kernel is faster there too (at 256^3 layer 0 0.60 against 0.89 ms, at 192^3 0.26
// against 0.50 ms), with 32 and 64 slower (one to three CTAs an SM).
bool conv_im2col(const UNetState* u, int level, int cin) {
    const Level& L = u->L[level];
    return !(L.W >= kHaloMinWidth && cin % 16 == 0 && cin <= 64 && cin > 16);
}

// up: `in` is the next coarser level's tensor, read as its nearest up-sampling (not on halo-tile levels).
// pool: also the 2x2x2 mean of `out` on the next coarser level (fused into the slab kernel where it serves).
cudaError_t conv(UNetState* u, int layer, const bf16* in, const bf16* wt, int cin, int cout, int level, const float* bias,
                 const bf16* skip, bf16* out, float* out32, bf16* pre, int relu, cudaStream_t st, bool up = false,
                 bf16* pool = nullptr) {
    const Level& L = u->L[level];
    auto pool_after = [&](cudaError_t e) -> cudaError_t {
        if (e != cudaSuccess || !pool) return e;
        const Level& P = u->L[level + 1];
        k_pool<<<nblk(P.V * (cout / 8)), 256, 0, st>>>(out, L, pool, P, cout);
        return cudaGetLastError();
    };
    if (!conv_im2col(u, level, cin)) {
        if (up) return cudaErrorInvalidValue;
        return pool_after(conv_halo(u, in, wt, cin, cout, L, bias, skip, out, out32, pre, relu, st));
    }
    tc::ConvArgs a{in, wt, bias, skip, out, out32, pre, L.D, L.H, L.W, cin, relu, u->err, nullptr, 0, up ? 1 : 0};
    // narrow grids: one CTA per 8 x 16 slab (two z slabs where the pooling is fused), its input brick and
    // weights in shared memory; the layer's weights come packed in that order where `wt` is one of its copies
    a.wslab = wt == u->wf[layer] ? u->wsf[layer] : wt == u->wb[layer] ? u->wsb[layer] : nullptr;
    const size_t slab1 = tc::slab_smem_bytes(cin, cout, 1), slab2 = tc::slab_smem_bytes(cin, cout, 2);
    tc::SlabMaps maps;
    std::memset(&maps, 0, sizeof(maps));
    if (tc::slab_fits(cin) && pool && cout <= 32 && slab2 <= (size_t)u->slab_smem) {
        a.pool = pool;
        if (!up) slab_maps(in, cin, L, 2, &maps);
        const unsigned gs = (unsigned)tc::slab_count(L.W, L.H, L.D, 2);
        if (cout == 16) tc::k_conv3_slab<16, 2><<<gs, tc::kConvThreads, slab2, st>>>(a, maps);
        else tc::k_conv3_slab<32, 2><<<gs, tc::kConvThreads, slab2, st>>>(a, maps);
        return cudaGetLastError();
    }
    if (tc::slab_fits(cin) && slab1 <= (size_t)u->slab_smem) {
        if (!up) slab_maps(in, cin, L, 1, &maps);
        const unsigned gs = (unsigned)tc::slab_count(L.W, L.H, L.D, 1);
        if (cout == 16) tc::k_conv3_slab<16, 1><<<gs, tc::kConvThreads, slab1, st>>>(a, maps);
        else if (cout == 32) tc::k_conv3_slab<32, 1><<<gs, tc::kConvThreads, slab1, st>>>(a, maps);
        else tc::k_conv3_slab<64, 1><<<gs, tc::kConvThreads, slab1, st>>>(a, maps);
        return pool_after(cudaGetLastError());
    }
    const unsigned grid = (unsigned)((L.V + 127) / 128);
    // Small grids (the coarse levels of the network, and the whole network on FCG's bottom grid) give too few
    // CTAs, each running all 27 x cin/16 MMA steps in sequence: split the steps over more CTAs, then sum.
    const int s_all = 27 * (cin / 16);
    int ks = 1, per = s_all;
    // as many splits as fill one wave of resident CTAs (7 per SM: kConvSmem and the TMEM columns): a second,
    // mostly empty wave costs a whole CTA lifetime
    const int slots = 7 * u->sm;
    if (!pre && u->split && (int)grid < slots) {
        ks = std::min(s_all, slots / (int)grid);
        per = (s_all + ks - 1) / ks;
        ks = (s_all + per - 1) / per;   // every split gets at least one step
        if ((long long)ks * L.V * cout > u->split_cap) ks = 1;
    }
    if (ks > 1) {
        a.partial = u->split;
        a.split_per = per;
        const dim3 g2(grid, (unsigned)ks);
        if (cout == 16) tc::k_conv3_tc<16><<<g2, tc::kConvThreads, tc::kConvSmem, st>>>(a);
        else if (cout == 32) tc::k_conv3_tc<32><<<g2, tc::kConvThreads, tc::kConvSmem, st>>>(a);
        else tc::k_conv3_tc<64><<<g2, tc::kConvThreads, tc::kConvSmem, st>>>(a);
        {
            const cudaError_t ce = cudaGetLastError();
            if (ce != cudaSuccess) return ce;
        }
        const int lanes = tc::split_lanes(ks);
        const unsigned rg = nblk(L.V * (cout / 4) * lanes);
#define EFS_SPLIT_REDUCE(CO, LN) tc::k_conv_split_reduce<CO, LN><<<rg, 256, 0, st>>>(u->split, ks, (int)L.V, bias, skip, out, out32, relu)
        if (lanes == 8) {
            if (cout == 16) EFS_SPLIT_REDUCE(16, 8);
            else if (cout == 32) EFS_SPLIT_REDUCE(32, 8);
            else EFS_SPLIT_REDUCE(64, 8);
        } else {
            if (cout == 16) EFS_SPLIT_REDUCE(16, 1);
            else if (cout == 32) EFS_SPLIT_REDUCE(32, 1);
            else EFS_SPLIT_REDUCE(64, 1);
        }
#undef EFS_SPLIT_REDUCE
        return pool_after(cudaGetLastError());
    }
    if (cout == 16) tc::k_conv3_tc<16><<<grid, tc::kConvThreads, tc::kConvSmem, st>>>(a);
    else if (cout == 32) tc::k_conv3_tc<32><<<grid, tc::kConvThreads, tc::kConvSmem, st>>>(a);
    else tc::k_conv3_tc<64><<<grid, tc::kConvThreads, tc::kConvSmem, st>>>(a);
    return pool_after(cudaGetLastError());
}

cudaError_t wgrad(UNetState* u, const bf16* in, const bf16* g, int cin, int cout, int level, float* dw, int sm_count,
                  cudaStream_t st) {
    const Level& L = u->L[level];
    const int mt = (27 * cin + 127) / 128;
    const long long want = std::max(1LL, (long long)(4 * sm_count + mt - 1) / mt);
    const long long splits = std::min(want, (L.V + 15) / 16);
    long long per = (L.V + splits - 1) / splits;
    per = (per + 15) / 16 * 16;
    const unsigned ny = (unsigned)((L.V + per - 1) / per);
    tc::WgradArgs a{in, g, dw, L.D, L.H, L.W, cin, (int)per, u->err};
    const dim3 grid((unsigned)mt, ny);
    if (cout == 16) tc::k_wgrad3_tc<16><<<grid, tc::kConvThreads, tc::kConvSmem, st>>>(a);
    else if (cout == 32) tc::k_wgrad3_tc<32><<<grid, tc::kConvThreads, tc::kConvSmem, st>>>(a);
    else tc::k_wgrad3_tc<64><<<grid, tc::kConvThreads, tc::kConvSmem, st>>>(a);
    return cudaGetLastError();
}

#define UCK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return e_; } while (0)

cudaError_t refresh_bf16(UNetState* u, cudaStream_t st) {
    for (int k = 0; k < kLayers; k++) {
        const int n = 27 * kSpec[k].cin * kSpec[k].cout;
        k_w_to_bf16<<<nblk(n), 256, 0, st>>>(u->w32 + u->woff[k], kSpec[k].cin, kSpec[k].cout, u->wf[k], u->wb[k],
                                              u->wsf[k], u->wsb[k]);
        UCK(cudaGetLastError());
    }
    return cudaSuccess;
}

// rms scale of x over rows into scal[0..2]
cudaError_t scale_rows(UNetState* u, const float* x, const uint16_t* rowinfo, long long n, double* scal, cudaStream_t st) {
    k_sumsq_rows<<<kRedBlocks, 256, 0, st>>>(x, rowinfo, n, u->dpart);
    UCK(cudaGetLastError());
    k_finish_scale<<<1, 256, 0, st>>>(u->dpart, kRedBlocks, scal);
    return cudaGetLastError();
}

// forward pass on the input field `r` (FP32, reference layout) with matrix rows `rowinfo`; y32 holds the output.
// train: keep the pre-activations for the backward pass.
// prescaled: u->dscal[0..2] already hold the input's sum of squares, row count and 1 / rms (FCG's restriction
// kernel computes them on the way down).
cudaError_t forward(UNetState* u, const float* r, const LvView& M, bool train, cudaStream_t st,
                    cudaEvent_t* ev = nullptr, bool prescaled = false) {
    const Level *L = u->L;
    const uint16_t* rowinfo = M.info;
    // ev (optional): 12 events recorded before and after each of the six convolutions (layers 0 and 1 with their
    // pooling)
    auto mark = [&](int k) { if (ev) cudaEventRecord(ev[k], st); };
    if (!prescaled) UCK(scale_rows(u, r, rowinfo, L[0].V, u->dscal, st));
    k_pack<<<nblk(L[0].V), 256, 0, st>>>(r, rowinfo, u->dscal, L[0].V, u->x0, M.w, M.diag,
                                          1.f / (float)(1 << (2 * u->level)));
    UCK(cudaGetLastError());
    const float* B[kLayers];
    for (int k = 0; k < kLayers; k++) B[k] = u->w32 + u->boff[k];
    mark(0);
    // layers 0 and 1 with the 2x2x2 mean pooling of their outputs (p0, p1)
    UCK(conv(u, 0, u->x0, u->wf[0], 16, 16, 0, B[0], nullptr, u->e0, nullptr, train ? u->a0 : nullptr, 1, st, false,
             u->p0));
    mark(1);
    mark(2);
    UCK(conv(u, 1, u->p0, u->wf[1], 16, 32, 1, B[1], nullptr, u->e1, nullptr, train ? u->a1 : nullptr, 1, st, false,
             u->p1));
    mark(3);
    mark(4);
    UCK(conv(u, 2, u->p1, u->wf[2], 32, 64, 2, B[2], nullptr, u->e2, nullptr, train ? u->a2 : nullptr, 1, st));
    mark(5);
    // the up-samplings: read in place by the next convolution where it is the implicit-GEMM kernel and nothing
    // keeps the up-sampled tensor (training's weight gradients read it)
    // (wide levels materialise the up-sampling: a gather of it per brick there is slower than the copy)
    const bool up3 = !train && conv_im2col(u, 1, 64) && u->L[1].W < kHaloMinWidth,
               up4 = !train && conv_im2col(u, 0, 32) && u->L[0].W < kHaloMinWidth;
    if (!up3) {
        k_up<<<nblk(L[1].V * 8), 256, 0, st>>>(u->e2, L[2], u->u2, L[1], 64);
        UCK(cudaGetLastError());
    }
    mark(6);
    UCK(conv(u, 3, up3 ? u->e2 : u->u2, u->wf[3], 64, 32, 1, B[3], u->e1, u->d1, nullptr, train ? u->a3 : nullptr, 1, st,
             up3));
    mark(7);
    if (!up4) {
        k_up<<<nblk(L[0].V * 4), 256, 0, st>>>(u->d1, L[1], u->u1, L[0], 32);
        UCK(cudaGetLastError());
    }
    mark(8);
    UCK(conv(u, 4, up4 ? u->d1 : u->u1, u->wf[4], 32, 16, 0, B[4], u->e0, u->d0, nullptr, train ? u->a4 : nullptr, 1, st,
             up4));
    mark(9);
    mark(10);
    UCK(conv(u, 5, u->d0, u->wf[5], 16, 16, 0, B[5], nullptr, nullptr, u->y32, nullptr, 0, st));
    mark(11);
    return cudaSuccess;
}

// The training losses (kind 0: mean squared error against the target field p normalised by its rms over
// rows; kind 1: energy-norm alignment with the error p for input r, see k_energy_grad) and the gradients of
// every parameter, accumulated into u->grad.  Requires a forward(train = true) on input r just before.
cudaError_t backward(UNetState* u, const float* r, const float* p, const LvView& M, int kind, int sm_count,
                     cudaStream_t st) {
    const uint16_t* rowinfo = M.info;
    const Level* L = u->L;
    float* G = u->grad;
    const unsigned nb = nblk(L[0].V);
    if (kind == 0) {
        UCK(scale_rows(u, p, rowinfo, L[0].V, u->dscal + 3, st));
        k_loss<<<nb, 256, 0, st>>>(u->y32, p, rowinfo, u->dscal + 3, L[0].V, u->g5, u->dpart);
        UCK(cudaGetLastError());
        k_sum_partials<<<1, 256, 0, st>>>(u->dpart, (int)nb, u->dscal + 3, u->dloss);
        UCK(cudaGetLastError());
    } else {
        k_unpack<<<nb, 256, 0, st>>>(u->y32, rowinfo, L[0].V, u->tz);
        UCK(cudaGetLastError());
        UCK(ml_matvec(M, u->tz, u->tq, st));
        k_dots3<<<kRedBlocks, 256, 0, st>>>(u->tz, r, u->tz, u->tq, p, r, L[0].V, u->dpart);
        UCK(cudaGetLastError());
        k_dots3_finish<<<1, 256, 0, st>>>(u->dpart, kRedBlocks, u->dscal + 8);
        UCK(cudaGetLastError());
        k_energy_grad<<<nb, 256, 0, st>>>(r, u->tq, rowinfo, u->dscal + 8, L[0].V, u->g5);
        UCK(cudaGetLastError());
        k_energy_loss<<<1, 1, 0, st>>>(u->dscal + 8, u->dloss);
        UCK(cudaGetLastError());
    }
    auto bgrad = [&](const bf16* g, long long V, int C, int layer) {
        k_bias_grad<<<256, 256, 0, st>>>(g, V, C, G + u->boff[layer]);
        return cudaGetLastError();
    };
    // layer 5
    UCK(wgrad(u, u->d0, u->g5, 16, 16, 0, G + u->woff[5], sm_count, st));
    UCK(bgrad(u->g5, L[0].V, 16, 5));
    UCK(conv(u, 5, u->g5, u->wb[5], 16, 16, 0, nullptr, nullptr, u->gd0, nullptr, nullptr, 0, st));
    // layer 4: d0 = relu(a4) + e0
    k_relu_bwd<<<nblk(L[0].V * 2), 256, 0, st>>>(u->gd0, u->a4, L[0].V * 2, u->ga4);
    UCK(cudaGetLastError());
    UCK(wgrad(u, u->u1, u->ga4, 32, 16, 0, G + u->woff[4], sm_count, st));
    UCK(bgrad(u->ga4, L[0].V, 16, 4));
    UCK(conv(u, 4, u->ga4, u->wb[4], 16, 32, 0, nullptr, nullptr, u->gu1, nullptr, nullptr, 0, st));
    k_up_bwd<<<nblk(L[1].V * 4), 256, 0, st>>>(u->gu1, L[0], u->gd1, L[1], 32);
    UCK(cudaGetLastError());
    // layer 3: d1 = relu(a3) + e1
    k_relu_bwd<<<nblk(L[1].V * 4), 256, 0, st>>>(u->gd1, u->a3, L[1].V * 4, u->ga3);
    UCK(cudaGetLastError());
    UCK(wgrad(u, u->u2, u->ga3, 64, 32, 1, G + u->woff[3], sm_count, st));
    UCK(bgrad(u->ga3, L[1].V, 32, 3));
    UCK(conv(u, 3, u->ga3, u->wb[3], 32, 64, 1, nullptr, nullptr, u->gu2, nullptr, nullptr, 0, st));
    k_up_bwd<<<nblk(L[2].V * 8), 256, 0, st>>>(u->gu2, L[1], u->ge2, L[2], 64);
    UCK(cudaGetLastError());
    // layer 2
    k_relu_bwd<<<nblk(L[2].V * 8), 256, 0, st>>>(u->ge2, u->a2, L[2].V * 8, u->ga2);
    UCK(cudaGetLastError());
    UCK(wgrad(u, u->p1, u->ga2, 32, 64, 2, G + u->woff[2], sm_count, st));
    UCK(bgrad(u->ga2, L[2].V, 64, 2));
    UCK(conv(u, 2, u->ga2, u->wb[2], 64, 32, 2, nullptr, nullptr, u->gp1, nullptr, nullptr, 0, st));
    k_pool_bwd<<<nblk(L[1].V * 4), 256, 0, st>>>(u->gp1, L[2], u->ge1, L[1], 32, u->gd1);
    UCK(cudaGetLastError());
    // layer 1
    k_relu_bwd<<<nblk(L[1].V * 4), 256, 0, st>>>(u->ge1, u->a1, L[1].V * 4, u->ga1);
    UCK(cudaGetLastError());
    UCK(wgrad(u, u->p0, u->ga1, 16, 32, 1, G + u->woff[1], sm_count, st));
    UCK(bgrad(u->ga1, L[1].V, 32, 1));
    UCK(conv(u, 1, u->ga1, u->wb[1], 32, 16, 1, nullptr, nullptr, u->gp0, nullptr, nullptr, 0, st));
    k_pool_bwd<<<nblk(L[0].V * 2), 256, 0, st>>>(u->gp0, L[1], u->ge0, L[0], 16, u->gd0);
    UCK(cudaGetLastError());
    // layer 0
    k_relu_bwd<<<nblk(L[0].V * 2), 256, 0, st>>>(u->ge0, u->a0, L[0].V * 2, u->ga0);
    UCK(cudaGetLastError());
    UCK(wgrad(u, u->x0, u->ga0, 16, 16, 0, G + u->woff[0], sm_count, st));
    UCK(bgrad(u->ga0, L[0].V, 16, 0));
    return cudaSuccess;
}

cudaError_t alloc_train(UNetState* u) {
    if (u->train_ready) return cudaSuccess;
    const Level* L = u->L;
    UCK(ualloc(u, &u->a0, L[0].V * 16));
    UCK(ualloc(u, &u->a1, L[1].V * 32));
    UCK(ualloc(u, &u->a2, L[2].V * 64));
    UCK(ualloc(u, &u->a3, L[1].V * 32));
    UCK(ualloc(u, &u->a4, L[0].V * 16));
    UCK(ualloc(u, &u->g5, L[0].V * 16));
    UCK(ualloc(u, &u->gd0, L[0].V * 16));
    UCK(ualloc(u, &u->ga4, L[0].V * 16));
    UCK(ualloc(u, &u->gu1, L[0].V * 32));
    UCK(ualloc(u, &u->gd1, L[1].V * 32));
    UCK(ualloc(u, &u->ga3, L[1].V * 32));
    UCK(ualloc(u, &u->gu2, L[1].V * 64));
    UCK(ualloc(u, &u->ge2, L[2].V * 64));
    UCK(ualloc(u, &u->ga2, L[2].V * 64));
    UCK(ualloc(u, &u->gp1, L[2].V * 32));
    UCK(ualloc(u, &u->ge1, L[1].V * 32));
    UCK(ualloc(u, &u->ga1, L[1].V * 32));
    UCK(ualloc(u, &u->gp0, L[1].V * 16));
    UCK(ualloc(u, &u->ge0, L[0].V * 16));
    UCK(ualloc(u, &u->ga0, L[0].V * 16));
    UCK(ualloc(u, &u->tz, L[0].V));
    UCK(ualloc(u, &u->tq, L[0].V));
    UCK(ualloc(u, &u->grad, u->nparam));
    UCK(ualloc(u, &u->am, u->nparam));
    UCK(ualloc(u, &u->av, u->nparam));
    UCK(cudaMemset(u->am, 0, u->nparam * sizeof(float)));
    UCK(cudaMemset(u->av, 0, u->nparam * sizeof(float)));
    u->adam_t = 0;
    u->train_ready = true;
    return cudaSuccess;
}

cudaError_t alloc_net(efs_ctx* c, UNetState** out) {
    UNetState* u = new UNetState();
    *out = u;
    u->level = ml_resolve_levels(c);
    for (int l = 0; l < 3; l++) u->L[l] = level_of(c, u->level, l);
    long long off = 0;
    for (int k = 0; k < kLayers; k++) {
        u->woff[k] = off;
        off += 27LL * kSpec[k].cin * kSpec[k].cout;
        u->boff[k] = off;
        off += kSpec[k].cout;
    }
    u->nparam = off;
    const Level* L = u->L;
    UCK(ualloc(u, &u->w32, u->nparam));
    for (int k = 0; k < kLayers; k++) {
        UCK(ualloc(u, &u->wf[k], 27LL * kSpec[k].cin * kSpec[k].cout));
        UCK(ualloc(u, &u->wb[k], 27LL * kSpec[k].cin * kSpec[k].cout));
        UCK(ualloc(u, &u->wsf[k], 27LL * kSpec[k].cin * kSpec[k].cout));
        UCK(ualloc(u, &u->wsb[k], 27LL * kSpec[k].cin * kSpec[k].cout));
    }
    UCK(ualloc(u, &u->wh, 27LL * 64 * 64));
    // split convolutions run on grids of fewer than 8 x SMs CTAs of 128 voxels, into at most 8 x SMs + CTAs more
    // partial tiles: (8 x SMs + 8 x SMs) x 128 voxels x 64 channels bounds every layer (the launch also checks)
    u->sm = c->sm_count > 0 ? c->sm_count : 152;
    UCK(slab_setup(u));
    u->split_cap = 16LL * u->sm * 128 * 64;
    UCK(ualloc(u, &u->split, u->split_cap));
    UCK(ualloc(u, &u->x0, L[0].V * 16));
    UCK(ualloc(u, &u->e0, L[0].V * 16));
    UCK(ualloc(u, &u->p0, L[1].V * 16));
    UCK(ualloc(u, &u->e1, L[1].V * 32));
    UCK(ualloc(u, &u->p1, L[2].V * 32));
    UCK(ualloc(u, &u->e2, L[2].V * 64));
    UCK(ualloc(u, &u->u2, L[1].V * 64));
    UCK(ualloc(u, &u->d1, L[1].V * 32));
    UCK(ualloc(u, &u->u1, L[0].V * 32));
    UCK(ualloc(u, &u->d0, L[0].V * 16));
    UCK(ualloc(u, &u->y32, L[0].V));
    UCK(ualloc(u, &u->dscal, 12));
    UCK(ualloc(u, &u->dpart, 3LL * std::max<long long>(kRedBlocks, nblk(L[0].V))));
    UCK(ualloc(u, &u->dloss, 1));
    UCK(ualloc(u, &u->err, 1));
    UCK(ualloc(u, &u->tmp_in, L[0].V));
    UCK(ualloc(u, &u->tmp_t, L[0].V));
    UCK(cudaMemset(u->err, 0, sizeof(int)));
    return cudaSuccess;
}

int check_err(efs_ctx* c, UNetState* u) {
    int e = 0;
    if (cudaMemcpy(&e, u->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return EFS_ERR_CUDA;
    if (e) {
        c->err = "tensor-core kernel: an mbarrier wait timed out";
        return EFS_ERR_DEVICE_FAULT;
    }
    return EFS_OK;
}

int ufail(efs_ctx* c, int status, const std::string& msg) {
    if (c) c->err = msg;
    return status;
}
int ucuda(efs_ctx* c, cudaError_t e, const char* what) {
    return ufail(c, EFS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define ACK(call, what) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return efs::ucuda(c, e_, what); } while (0)

}  // namespace

void unet_free(efs_ctx* c) {
    if (!c || !c->unet) return;
    for (void* p : c->unet->allocs) cudaFree(p);
    delete c->unet;
    c->unet = nullptr;
}

// The network's correction for residual r on the bottom level B, left in unet_output(c) (channel 0 of the last
// convolution, to be read on B's rows).  The input scale (1 / rms of r over the rows) must already be in
// unet_scale_slot(c)[2], as FCG's restriction kernel leaves it.
cudaError_t unet_forward_prescaled(efs_ctx* c, const LvView& B, const float* r, cudaStream_t st) {
    UNetState* u = c->unet;
    if (!u || u->L[0].V != B.V) return cudaErrorInvalidValue;
    return forward(u, r, B, false, st, nullptr, true);
}
double* unet_scale_slot(efs_ctx* c) { return c->unet ? c->unet->dscal : nullptr; }
cudaError_t unet_scale_rows(efs_ctx* c, const LvView& B, const float* r, cudaStream_t st) {
    return scale_rows(c->unet, r, B.info, B.V, c->unet->dscal, st);
}
const float* unet_output(efs_ctx* c) { return c->unet ? c->unet->y32 : nullptr; }

bool unet_matches(const efs_ctx* c) { return c->unet && c->unet->level == ml_resolve_levels(c); }

// The matrix the network works on: the context's grid (level 0) or the FCG hierarchy's bottom level, built
// from the current rowinfo (launch_solver_prep first).
cudaError_t net_matrix(efs_ctx* c, LvView* M) {
    UNetState* u = c->unet;
    if (u->level == 0) {
        *M = ml_view(c, 0);
        return cudaSuccess;
    }
    if (ml_resolve_levels(c) != u->level) return cudaErrorInvalidValue;
    UCK(ml_alloc(c));
    UCK(ml_build(c, c->stream));
    *M = ml_view(c, u->level);
    return cudaSuccess;
}

}  // namespace efs

using efs::UNetState;

extern "C" {

int efs_unet_param_count(int64_t* n) {
    if (!n) return EFS_ERR_ARG;
    *n = efs::param_count_host();
    return EFS_OK;
}

int efs_unet_init(efs_ctx* c, uint64_t seed, int sample_capacity) {
    if (!c) return EFS_ERR_ARG;
    if (c->dim != 3) return efs::ufail(c, EFS_ERR_ARG, "the U-Net preconditioner is 3D only");
    if (sample_capacity < 0) return efs::ufail(c, EFS_ERR_ARG, "sample_capacity < 0");
    ACK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    efs::drop_all_graphs(c);      // captured solves address the old network's buffers
    efs::unet_free(c);
    UNetState* u = nullptr;
    cudaError_t e = efs::alloc_net(c, &u);
    c->unet = u;
    if (e != cudaSuccess) { efs::unet_free(c); return efs::ucuda(c, e, "U-Net allocation"); }
    for (int k = 0; k < efs::kLayers; k++) {
        const long long nw = 27LL * efs::kSpec[k].cin * efs::kSpec[k].cout;
        const long long nk = nw + efs::kSpec[k].cout;
        const float stdv = (float)std::sqrt(2.0 / (27.0 * efs::kSpec[k].cin));
        efs::k_init<<<efs::nblk(nk), 256, 0, c->stream>>>(u->w32 + u->woff[k], nk, nw, stdv, seed, (unsigned long long)k);
        ACK(cudaGetLastError(), "U-Net init");
    }
    ACK(efs::refresh_bf16(u, c->stream), "U-Net weights");
    if (sample_capacity > 0) {
        const long long V = u->L[0].V;
        ACK(efs::ualloc(u, &u->sb, V * sample_capacity), "sample buffer");
        ACK(efs::ualloc(u, &u->sp, V * sample_capacity), "sample buffer");
        ACK(efs::ualloc(u, &u->srow, V * sample_capacity), "sample buffer");
        if (u->level > 0) {
            ACK(efs::ualloc(u, &u->sw, 6 * V * sample_capacity), "sample buffer");
            ACK(efs::ualloc(u, &u->sdiag, V * sample_capacity), "sample buffer");
        }
        u->cap = sample_capacity;
    }
    ACK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

int efs_unet_get_weights(efs_ctx* c, float* host, int64_t n) {
    if (!c) return EFS_ERR_ARG;
    if (!c->unet) return efs::ufail(c, EFS_ERR_STATE, "no U-Net: call efs_unet_init first");
    if (!host || n != c->unet->nparam) return efs::ufail(c, EFS_ERR_ARG, "host buffer must hold efs_unet_param_count floats");
    ACK(cudaMemcpyAsync(host, c->unet->w32, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "download weights");
    ACK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

int efs_unet_set_weights(efs_ctx* c, const float* host, int64_t n) {
    if (!c) return EFS_ERR_ARG;
    if (!c->unet) return efs::ufail(c, EFS_ERR_STATE, "no U-Net: call efs_unet_init first");
    if (!host || n != c->unet->nparam) return efs::ufail(c, EFS_ERR_ARG, "host buffer must hold efs_unet_param_count floats");
    for (int64_t i = 0; i < n; i++)
        if (!std::isfinite(host[i])) return efs::ufail(c, EFS_ERR_ARG, "weights must be finite");
    ACK(cudaMemcpyAsync(c->unet->w32, host, n * sizeof(float), cudaMemcpyHostToDevice, c->stream), "upload weights");
    ACK(efs::refresh_bf16(c->unet, c->stream), "U-Net weights");
    if (c->unet->train_ready) {   // new weights: fresh optimiser state
        ACK(cudaMemsetAsync(c->unet->am, 0, n * sizeof(float), c->stream), "memset");
        ACK(cudaMemsetAsync(c->unet->av, 0, n * sizeof(float), c->stream), "memset");
        c->unet->adam_t = 0;
    }
    ACK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return EFS_OK;
}

int efs_unet_apply(efs_ctx* c, const float* r_host, float* z_host) {
    if (!c) return EFS_ERR_ARG;
    UNetState* u = c->unet;
    if (!u) return efs::ufail(c, EFS_ERR_STATE, "no U-Net: call efs_unet_init first");
    if (!r_host || !z_host) return efs::ufail(c, EFS_ERR_ARG, "NULL field");
    const long long N = u->L[0].V;
    ACK(efs::launch_solver_prep(c), "solver prep");
    efs::LvView M;
    ACK(efs::net_matrix(c, &M), "hierarchy (efs_unet_init again after changing fcg_levels)");
    ACK(cudaMemcpyAsync(u->tmp_in, r_host, N * sizeof(float), cudaMemcpyHostToDevice, c->stream), "upload");
    ACK(efs::forward(u, u->tmp_in, M, false, c->stream), "U-Net forward");
    efs::k_unpack<<<efs::nblk(N), 256, 0, c->stream>>>(u->y32, M.info, N, u->tmp_t);
    ACK(cudaGetLastError(), "unpack");
    ACK(cudaMemcpyAsync(z_host, u->tmp_t, N * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "download");
    ACK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return efs::check_err(c, u);
}

int efs_unet_loss_grad(efs_ctx* c, int loss_kind, const float* b_host, const float* p_host, float* loss, float* grads_host) {
    if (!c) return EFS_ERR_ARG;
    UNetState* u = c->unet;
    if (!u) return efs::ufail(c, EFS_ERR_STATE, "no U-Net: call efs_unet_init first");
    if (!b_host || !p_host) return efs::ufail(c, EFS_ERR_ARG, "NULL field");
    if (loss_kind != 0 && loss_kind != 1) return efs::ufail(c, EFS_ERR_ARG, "loss_kind: 0 (pressure MSE) or 1 (energy)");
    const long long N = u->L[0].V;
    cudaStream_t st = c->stream;
    ACK(efs::alloc_train(u), "U-Net training buffers");
    ACK(efs::launch_solver_prep(c), "solver prep");
    efs::LvView M;
    ACK(efs::net_matrix(c, &M), "hierarchy (efs_unet_init again after changing fcg_levels)");
    ACK(cudaMemcpyAsync(u->tmp_in, b_host, N * sizeof(float), cudaMemcpyHostToDevice, st), "upload");
    ACK(cudaMemcpyAsync(u->tmp_t, p_host, N * sizeof(float), cudaMemcpyHostToDevice, st), "upload");
    ACK(cudaMemsetAsync(u->grad, 0, u->nparam * sizeof(float), st), "memset");
    ACK(cudaMemsetAsync(u->dloss, 0, sizeof(double), st), "memset");
    ACK(efs::forward(u, u->tmp_in, M, true, st), "U-Net forward");
    ACK(efs::backward(u, u->tmp_in, u->tmp_t, M, loss_kind, c->sm_count, st), "U-Net backward");
    double l = 0;
    ACK(cudaMemcpyAsync(&l, u->dloss, sizeof(double), cudaMemcpyDeviceToHost, st), "download");
    if (grads_host) ACK(cudaMemcpyAsync(grads_host, u->grad, u->nparam * sizeof(float), cudaMemcpyDeviceToHost, st), "download");
    ACK(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (loss) *loss = (float)l;
    return efs::check_err(c, u);
}

int efs_unet_time_forward(efs_ctx* c, int reps, float* ms_forward, float* ms_layers) {
    if (!c) return EFS_ERR_ARG;
    UNetState* u = c->unet;
    if (!u) return efs::ufail(c, EFS_ERR_STATE, "no U-Net: call efs_unet_init first");
    if (reps < 1) return efs::ufail(c, EFS_ERR_ARG, "reps >= 1");
    cudaStream_t st = c->stream;
    cudaEvent_t ev[12], e0, e1;
    for (auto& e : ev) ACK(cudaEventCreate(&e), "cudaEventCreate");
    ACK(cudaEventCreate(&e0), "cudaEventCreate");
    ACK(cudaEventCreate(&e1), "cudaEventCreate");
    ACK(efs::launch_solver_prep(c), "solver prep");
    efs::LvView M;
    ACK(efs::net_matrix(c, &M), "hierarchy (efs_unet_init again after changing fcg_levels)");
    // the input: the divergence itself, or carried down to the network's level as the V-cycle carries it
    const float* in = c->div;
    if (u->level > 0) ACK(efs::ml_descend(c, c->div, st, &in), "descend");
    ACK(efs::forward(u, in, M, false, st), "U-Net forward");   // warm-up
    double lay[6] = {0, 0, 0, 0, 0, 0};
    float total = 0.f;
    cudaError_t err = cudaSuccess;
    for (int k = 0; k < reps && err == cudaSuccess; k++) {
        cudaEventRecord(e0, st);
        err = efs::forward(u, in, M, false, st, ev);
        cudaEventRecord(e1, st);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (err == cudaSuccess) { cudaEventElapsedTime(&ms, e0, e1); total += ms; }
        for (int l = 0; l < 6 && err == cudaSuccess; l++) {
            float m = 0.f;
            cudaEventElapsedTime(&m, ev[2 * l], ev[2 * l + 1]);
            lay[l] += m;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ACK(err, "U-Net timing");
    if (ms_forward) *ms_forward = total / reps;
    if (ms_layers)
        for (int l = 0; l < 6; l++) ms_layers[l] = (float)(lay[l] / reps);
    return efs::check_err(c, u);
}

int efs_unet_add_sample(efs_ctx* c) {
    if (!c) return EFS_ERR_ARG;
    UNetState* u = c->unet;
    if (!u || u->cap == 0) return efs::ufail(c, EFS_ERR_STATE, "no sample buffer: efs_unet_init with sample_capacity > 0");
    const long long V = u->L[0].V;
    const int slot = u->next;
    cudaStream_t st = c->stream;
    if (u->level == 0) {
        ACK(cudaMemcpyAsync(u->sb + (size_t)slot * V, c->div, V * sizeof(float), cudaMemcpyDeviceToDevice, st), "sample");
        ACK(cudaMemcpyAsync(u->sp + (size_t)slot * V, c->p, V * sizeof(float), cudaMemcpyDeviceToDevice, st), "sample");
        ACK(cudaMemcpyAsync(u->srow + (size_t)slot * V, c->rowinfo, V * sizeof(uint16_t), cudaMemcpyDeviceToDevice, st),
            "sample");
    } else {
        // the divergence as the first V-cycle carries it to the network's level, and its exact correction there
        efs::LvView M;
        ACK(efs::launch_solver_prep(c), "solver prep");
        ACK(efs::net_matrix(c, &M), "hierarchy (efs_unet_init again after changing fcg_levels)");
        const float* rb = nullptr;
        ACK(efs::ml_descend(c, c->div, st, &rb), "descend");
        if (!u->c1) {
            ACK(efs::ualloc(u, &u->c1, V), "sample CG");
            ACK(efs::ualloc(u, &u->c2, V), "sample CG");
            ACK(efs::ualloc(u, &u->c3, V), "sample CG");
        }
        float* sb = u->sb + (size_t)slot * V;
        float* sp = u->sp + (size_t)slot * V;
        ACK(cudaMemcpyAsync(sb, rb, V * sizeof(float), cudaMemcpyDeviceToDevice, st), "sample");
        if (efs::ml_level_cg(c, M, sb, sp, u->c1, u->c2, u->c3, 1e-8, 20000, st) < 0)
            return efs::ufail(c, EFS_ERR_CUDA, "bottom-level CG of a training sample failed");
        ACK(cudaMemcpyAsync(u->srow + (size_t)slot * V, M.info, V * sizeof(uint16_t), cudaMemcpyDeviceToDevice, st), "sample");
        ACK(cudaMemcpyAsync(u->sw + (size_t)slot * 6 * V, M.w, 6 * V, cudaMemcpyDeviceToDevice, st), "sample");
        ACK(cudaMemcpyAsync(u->sdiag + (size_t)slot * V, M.diag, V * sizeof(float), cudaMemcpyDeviceToDevice, st), "sample");
    }
    u->next = (u->next + 1) % u->cap;
    u->count = std::min(u->count + 1, u->cap);
    return EFS_OK;
}

int efs_unet_grid(efs_ctx* c, int* width, int* height, int* depth, int* level) {
    if (!c) return EFS_ERR_ARG;
    if (!c->unet) return efs::ufail(c, EFS_ERR_STATE, "no U-Net: call efs_unet_init first");
    if (width) *width = c->unet->L[0].W;
    if (height) *height = c->unet->L[0].H;
    if (depth) *depth = c->unet->L[0].D;
    if (level) *level = c->unet->level;
    return EFS_OK;
}

int efs_unet_sample_count(efs_ctx* c, int* count) {
    if (!c || !count) return EFS_ERR_ARG;
    *count = c->unet ? c->unet->count : 0;
    return EFS_OK;
}

int efs_unet_train(efs_ctx* c, int loss_kind, int iterations, int batch, float lr, float synthetic, uint64_t seed,
                   float* last_loss) {
    if (!c) return EFS_ERR_ARG;
    UNetState* u = c->unet;
    if (!u) return efs::ufail(c, EFS_ERR_STATE, "no U-Net: call efs_unet_init first");
    if (u->count == 0) return efs::ufail(c, EFS_ERR_STATE, "no training samples: efs_unet_add_sample after a projection");
    if (iterations < 0 || batch < 1 || !(lr > 0) || !(synthetic >= 0.f && synthetic <= 1.f) ||
        (loss_kind != 0 && loss_kind != 1))
        return efs::ufail(c, EFS_ERR_ARG, "loss_kind 0/1, iterations >= 0, batch >= 1, lr > 0, 0 <= synthetic <= 1");
    cudaStream_t st = c->stream;
    const long long N = u->L[0].V;
    ACK(efs::alloc_train(u), "U-Net training buffers");
    unsigned long long rng = seed * 6364136223846793005ull + 1442695040888963407ull;
    double l = 0;
    for (int it = 0; it < iterations; it++) {
        ACK(cudaMemsetAsync(u->grad, 0, u->nparam * sizeof(float), st), "memset");
        ACK(cudaMemsetAsync(u->dloss, 0, sizeof(double), st), "memset");
        for (int b = 0; b < batch; b++) {
            rng = rng * 6364136223846793005ull + 1442695040888963407ull;
            const int s = (int)((rng >> 33) % (unsigned long long)u->count);
            const float* sb = u->sb + (size_t)s * N;
            const float* sp = u->sp + (size_t)s * N;
            const uint16_t* sr = u->srow + (size_t)s * N;
            efs::LvView M{u->L[0].W, u->L[0].H, u->L[0].D, N, sr, u->sw ? u->sw + (size_t)s * 6 * N : nullptr,
                          u->sdiag ? u->sdiag + (size_t)s * N : nullptr};
            rng = rng * 6364136223846793005ull + 1442695040888963407ull;
            if ((float)((rng >> 40) * (1.0 / 16777216.0)) < synthetic) {
                // synthetic pair on this sample's geometry: e random and multi-scale, input L e, target e
                efs::SynthAmp amp;
                rng = rng * 6364136223846793005ull + 1442695040888963407ull;
                const float gam = (float)((rng >> 40) * (2.0 / 16777216.0));
                for (int k = 0; k < 5; k++) {
                    rng = rng * 6364136223846793005ull + 1442695040888963407ull;
                    amp.a[k] = std::pow((float)(1 << k), gam) * (0.25f + 0.75f * (float)((rng >> 40) * (1.0 / 16777216.0)));
                }
                efs::k_synth_error<<<efs::nblk(N), 256, 0, st>>>(u->L[0], sr, rng, amp, u->tmp_t);
                ACK(cudaGetLastError(), "synthetic error");
                ACK(efs::ml_matvec(M, u->tmp_t, u->tmp_in, st), "synthetic residual");
                sb = u->tmp_in;
                sp = u->tmp_t;
            }
            ACK(efs::forward(u, sb, M, true, st), "U-Net forward");
            ACK(efs::backward(u, sb, sp, M, loss_kind, c->sm_count, st), "U-Net backward");
        }
        u->adam_t += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        const float bc1 = 1.f - std::pow(b1, (float)u->adam_t), bc2 = 1.f - std::pow(b2, (float)u->adam_t);
        efs::k_adam<<<efs::nblk(u->nparam), 256, 0, st>>>(u->nparam, u->w32, u->grad, u->am, u->av, lr, b1, b2, 1e-8f, bc1,
                                                          bc2, 1.f / (float)batch);
        ACK(cudaGetLastError(), "adam");
        ACK(efs::refresh_bf16(u, st), "U-Net weights");
        if (it == iterations - 1) {
            ACK(cudaMemcpyAsync(&l, u->dloss, sizeof(double), cudaMemcpyDeviceToHost, st), "download");
        }
    }
    ACK(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (last_loss) *last_loss = (float)(l / batch);
    return efs::check_err(c, u);
}

}  // extern "C"
