// efs_fields.cu — conversions between the reference's host layout and the device field store.
//
// Velocity and forces arrive as interleaved glm::vec3 / glm::vec2 floats (VecField3D / VecField2D storage,
// include/simulation/data/VecField3D.h:93) and are split into one array per component; the boundary field
// (float 0/1, ScalField3D) becomes one byte per cell.  Scalar fields share the reference layout and are
// copied as they are.
#include <algorithm>
#include <cstdint>

#include "efs_internal.h"

namespace efs {

namespace {

__global__ void k_split(int n, int dim, const float* __restrict__ src, float* __restrict__ a, float* __restrict__ b,
                        float* __restrict__ c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = src[(size_t)dim * i];
    b[i] = src[(size_t)dim * i + 1];
    if (dim == 3) c[i] = src[(size_t)dim * i + 2];
}

__global__ void k_interleave(int n, int dim, float* __restrict__ dst, const float* __restrict__ a,
                             const float* __restrict__ b, const float* __restrict__ c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[(size_t)dim * i] = a[i];
    dst[(size_t)dim * i + 1] = b[i];
    if (dim == 3) dst[(size_t)dim * i + 2] = c[i];
}

__global__ void k_bnd_to_solid(int n, const float* __restrict__ src, uint8_t* __restrict__ solid, DevCtl* ctl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float bv = src[i];
    if (!(bv == 0.0f || bv == 1.0f)) atomicOr(&ctl->error, DEV_ERR_BAD_BOUNDARY);
    solid[i] = (bv == 1.0f) ? 1 : 0;
}

__global__ void k_solid_to_bnd(int n, const uint8_t* __restrict__ solid, float* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = solid[i] ? 1.0f : 0.0f;
}

// Grid3D / Grid2D constructor state (src/simulation/data/Grid3D.cpp:10-48): gamma = 1, solid border, rho 0
// on it; every other field zero.
__global__ void k_reset(Geo g, int dim, float* __restrict__ gamma, float* __restrict__ rho, uint8_t* __restrict__ solid) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    const int x = i % g.W, y = (i / g.W) % g.H, z = i / g.WH;
    bool border = x == 0 || y == 0 || x == g.W - 1 || y == g.H - 1;
    if (dim == 3) border = border || z == 0 || z == g.D - 1;
    gamma[i] = 1.0f;
    rho[i] = 0.0f;
    solid[i] = border ? 1 : 0;
}

__global__ void k_mass(int n, const float* __restrict__ rho, double* __restrict__ out) {
    __shared__ double s[256];
    double acc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += (double)rho[i];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = s[0];
}

inline int nblk(int n) { return (n + 255) / 256; }

// dst[i] = src[i]; 16 bytes per thread where both pointers allow it.  Either side may be page-locked host
// memory that the GPU addresses directly.
__global__ void k_copy(long long n, const float* __restrict__ src, float* __restrict__ dst, int vec4) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    if (vec4) {
        const long long n4 = n >> 2;
        const float4* s4 = reinterpret_cast<const float4*>(src);
        float4* d4 = reinterpret_cast<float4*>(dst);
        for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n4; k += stride) d4[k] = s4[k];
        for (long long k = (n4 << 2) + blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += stride) dst[k] = src[k];
    } else {
        for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += stride) dst[k] = src[k];
    }
}

}  // namespace

cudaError_t launch_copy(efs_ctx* c, const float* src, float* dst, long long n) {
    const int vec4 = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
    const long long work = vec4 ? (n + 3) / 4 : n;
    const int blocks = (int)std::min<long long>(std::max<long long>(1, (work + 255) / 256), (long long)c->sm_count * 8);
    k_copy<<<blocks, 256, 0, c->stream>>>(n, src, dst, vec4);
    return cudaGetLastError();
}

cudaError_t launch_upload_vec(efs_ctx* c, const float* staged, float* a, float* b, float* cc, cudaStream_t st) {
    k_split<<<nblk(c->g.N), 256, 0, st ? st : c->stream>>>(c->g.N, c->dim, staged, a, b, cc);
    return cudaGetLastError();
}

cudaError_t launch_download_vec(efs_ctx* c, float* staged, const float* a, const float* b, const float* cc,
                                cudaStream_t st) {
    k_interleave<<<nblk(c->g.N), 256, 0, st ? st : c->stream>>>(c->g.N, c->dim, staged, a, b, cc);
    return cudaGetLastError();
}

cudaError_t launch_boundary_to_solid(efs_ctx* c, const float* staged) {
    k_bnd_to_solid<<<nblk(c->g.N), 256, 0, c->stream>>>(c->g.N, staged, c->solid, c->ctl);
    return cudaGetLastError();
}

cudaError_t launch_solid_to_boundary(efs_ctx* c, float* staged) {
    k_solid_to_bnd<<<nblk(c->g.N), 256, 0, c->stream>>>(c->g.N, c->solid, staged);
    return cudaGetLastError();
}

cudaError_t launch_reset_fields(efs_ctx* c) {
    const size_t bytes = (size_t)c->g.N * sizeof(float);
    float* zero[] = {c->u, c->v, c->w, c->beta, c->div, c->p, c->fx, c->fy, c->fz, c->tvel};
    for (float* z : zero) {
        cudaError_t e = cudaMemsetAsync(z, 0, z == c->tvel ? 3 * bytes : bytes, c->stream);
        if (e != cudaSuccess) return e;
    }
    k_reset<<<nblk(c->g.N), 256, 0, c->stream>>>(c->g, c->dim, c->gamma, c->rho, c->solid);
    return cudaGetLastError();
}

// FP64 sum of rho: 256 block partials written to out_dev[0..255]; the caller adds them in order.
cudaError_t launch_mass(efs_ctx* c, double* out_dev) {
    k_mass<<<256, 256, 0, c->stream>>>(c->g.N, c->rho, out_dev);
    return cudaGetLastError();
}

}  // namespace efs
