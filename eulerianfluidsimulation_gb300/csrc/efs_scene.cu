// efs_scene.cu — building a scene in the device field store and measuring it: the editor and scene-node
// side of the reference that writes or reads the grid between steps.
//
// - efs_mesh_label: the inside/outside label of every cell centre against a triangle soup, as the SDF
//   compute shader computes it (assets/shaders/sdf.comp:29-114; used by Editor::initFluid and
//   Editor::initBoundaries, src/core/Editor.cpp:99-137, :186-218).
// - efs_mesh_cells: the ordered list of inside cells (assets/shaders/forcefield_cells.comp:90-111; used by
//   Editor::updateForceFields, Editor.cpp:260-332).
// - efs_fill_box: a constant over a box of cells (the box fluid spawn, Editor.cpp:155-161; the initial fill,
//   baseFluidFill.comp:24-35; DeletionNode::update, DeletionNode.cpp:27-33; clearing a field).
// - efs_set_cells: a constant at listed cells (Scene2D::loadScene index lists, Scene2D.cpp:59-62; the force
//   field cells, Editor.cpp:325-330).
// - efs_seal_boundary: the solid border and rho = 0 in solids (Editor.cpp:220-229).
// - efs_query_box: QueryNode::update's metrics over a box (QueryNode.cpp:47-84).
//
// All of it runs on the context's stream.  The mesh label is compiled like the step (no fused multiply-add)
// and evaluates the shader's expressions in the shader's order, so it equals the CPU restatement of the
// shader except through atan2 (the winding number), whose library implementations differ in the last bits.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "efs_internal.h"

namespace efs {

namespace {

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float dot2(V3 a) { return dot(a, a); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float sgn(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
__device__ __forceinline__ V3 normalize(V3 a) {
    const float l = sqrtf(dot(a, a));
    return v3(a.x / l, a.y / l, a.z / l);
}

// The squared distance of p from triangle (a, b, c) before its square root (sdf.comp:29-51, the
// published unsigned triangle distance of I. Quilez).  Only whether it is zero matters to the label: the
// signed distance is -best inside and +best outside, and a cell is labelled outside when it is > 0, so a cell
// whose nearest triangle passes through its centre is inside whatever its winding number.
__device__ __forceinline__ float tri_dist2(V3 p, V3 a, V3 b, V3 c) {
    const V3 v21 = b - a, v32 = c - b, v13 = a - c;
    const V3 p1 = p - a, p2 = p - b, p3 = p - c;
    const V3 nor = cross(v21, v13);
    if (sgn(dot(cross(v21, nor), p1)) + sgn(dot(cross(v32, nor), p2)) + sgn(dot(cross(v13, nor), p3)) < 2.0f) {
        return fminf(fminf(dot2(v21 * clamp01(dot(v21, p1) / dot2(v21)) - p1),
                           dot2(v32 * clamp01(dot(v32, p2) / dot2(v32)) - p2)),
                     dot2(v13 * clamp01(dot(v13, p3) / dot2(v13)) - p3));
    }
    return dot(nor, p1) * dot(nor, p1) / dot2(nor);
}

// The solid angle of triangle (a, b, c) seen from p (sdf.comp:53-68, the formula of Van Oosterom and
// Strackee).
__device__ __forceinline__ float solid_angle(V3 p, V3 a, V3 b, V3 c) {
    const V3 na = normalize(a - p), nb = normalize(b - p), nc = normalize(c - p);
    const float num = dot(na, cross(nb, nc));
    const float den = 1.0f + dot(na, nb) + dot(nb, nc) + dot(nc, na);
    return 2.0f * atan2f(num, den);
}

constexpr int kTileTris = 128;
constexpr int kLabelThreads = 256;

enum LabelOut { LABEL_FLOAT = 0, LABEL_SOLID = 1, LABEL_MASK = 2 };

struct LabelArgs {
    Geo g;
    const float4* tris;     // 3 float4 per triangle: v0, v1, v2 (w unused), the reference Triangle layout
    int ntri;
    float cx, cy, cz, sx, sy, sz;   // domain centre and size
    float vin, vout;
    int out_kind;
    float* fout;
    uint8_t* bout;
};

// One thread per cell of [0, W-1) x [0, H-1) x [0, D-1) (sdf.comp:95-97); triangles pass through shared
// memory in tiles that every thread of the block loads together.
__global__ void __launch_bounds__(kLabelThreads) k_mesh_label(LabelArgs a) {
    __shared__ float4 s_tri[kTileTris * 3];
    const Geo& g = a.g;
    const int Wi = g.W - 1, Hi = g.H - 1, Di = g.D - 1;
    const long long ncell = (long long)Wi * Hi * Di;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = k < ncell;
    int x = 0, y = 0, z = 0;
    if (live) {
        x = (int)(k % Wi);
        y = (int)((k / Wi) % Hi);
        z = (int)(k / ((long long)Wi * Hi));
    }
    // sdf.comp:101-105: cellSize = uDomainSize / cellCount; domainMin = uDomainCenter - 0.5 * uDomainSize;
    // queryPosition = domainMin + cellSize * vec3(x, y, z) + cellSize * 0.5
    const float csx = a.sx / (float)g.W, csy = a.sy / (float)g.H, csz = a.sz / (float)g.D;
    const float mx = a.cx - 0.5f * a.sx, my = a.cy - 0.5f * a.sy, mz = a.cz - 0.5f * a.sz;
    const V3 p = v3(mx + csx * (float)x + csx * 0.5f, my + csy * (float)y + csy * 0.5f, mz + csz * (float)z + csz * 0.5f);

    bool on_surface = false;
    float wind = 0.0f;
    for (int pass = 0; pass < 2; pass++) {
        // pass 0: is any triangle at distance exactly 0; pass 1 (skipped when one is): the winding number
        const int need = __syncthreads_or(live && (pass == 0 || !on_surface));
        if (!need) break;
        for (int t0 = 0; t0 < a.ntri; t0 += kTileTris) {
            const int nt = min(kTileTris, a.ntri - t0);
            __syncthreads();
            for (int q = threadIdx.x; q < nt * 3; q += blockDim.x) s_tri[q] = a.tris[(size_t)t0 * 3 + q];
            __syncthreads();
            if (!live) continue;
            if (pass == 0) {
                if (on_surface) continue;
                for (int t = 0; t < nt; t++) {
                    const float4 A = s_tri[3 * t], B = s_tri[3 * t + 1], C = s_tri[3 * t + 2];
                    if (tri_dist2(p, v3(A.x, A.y, A.z), v3(B.x, B.y, B.z), v3(C.x, C.y, C.z)) == 0.0f) {
                        on_surface = true;
                        break;
                    }
                }
            } else if (!on_surface) {
                for (int t = 0; t < nt; t++) {
                    const float4 A = s_tri[3 * t], B = s_tri[3 * t + 1], C = s_tri[3 * t + 2];
                    wind += solid_angle(p, v3(A.x, A.y, A.z), v3(B.x, B.y, B.z), v3(C.x, C.y, C.z));
                }
            }
        }
    }
    if (!live) return;
    // sdf.comp:91: abs(winding) > 3.1415926 -> -best (inside), else best; the cell is outside when that is > 0
    const bool inside = on_surface || fabsf(wind) > 3.1415926f;
    const long long i = (long long)z * g.WH + (long long)y * g.W + x;
    if (a.out_kind == LABEL_FLOAT) a.fout[i] = inside ? a.vin : a.vout;
    else if (a.out_kind == LABEL_SOLID) a.bout[i] = inside ? (a.vin != 0.0f) : (a.vout != 0.0f);
    else a.bout[i] = inside ? 1 : 0;
}

// ---- ordered compaction of a byte mask into cell indices (tiles of 1024 cells) ---------------------------
constexpr int kTile = 1024;

__global__ void k_mask_count(const uint8_t* __restrict__ mask, long long n, int* __restrict__ counts) {
    __shared__ int s_w[32];
    const long long i = (long long)blockIdx.x * kTile + threadIdx.x;
    const int f = (i < n && mask[i]) ? 1 : 0;
    const int c = __popc(__ballot_sync(0xffffffffu, f));
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < kTile / 32; w++) s += s_w[w];
        counts[blockIdx.x] = s;
    }
}

// Exclusive scan of the tile counts by one block, in order; total written to counts[ntiles].
__global__ void k_scan_counts(int* __restrict__ counts, int ntiles, long long* __restrict__ offsets) {
    __shared__ long long s_part[1024];
    const int per = (ntiles + blockDim.x - 1) / blockDim.x;
    const int lo = threadIdx.x * per, hi = min(ntiles, lo + per);
    long long s = 0;
    for (int t = lo; t < hi; t++) s += counts[t];
    s_part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long run = 0;
        for (int q = 0; q < (int)blockDim.x; q++) { const long long v = s_part[q]; s_part[q] = run; run += v; }
        offsets[ntiles] = run;
    }
    __syncthreads();
    long long run = s_part[threadIdx.x];
    for (int t = lo; t < hi; t++) { offsets[t] = run; run += counts[t]; }
}

__global__ void k_mask_write(const uint8_t* __restrict__ mask, long long n, const long long* __restrict__ offsets,
                             int* __restrict__ out, long long cap) {
    __shared__ int s_w[32];
    const long long i = (long long)blockIdx.x * kTile + threadIdx.x;
    const int f = (i < n && mask[i]) ? 1 : 0;
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_w[warp] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int w = 0; w < kTile / 32; w++) { const int v = s_w[w]; s_w[w] = run; run += v; }
    }
    __syncthreads();
    if (f) {
        const long long pos = offsets[blockIdx.x] + s_w[warp] + __popc(bal & ((1u << lane) - 1u));
        if (pos < cap) out[pos] = (int)i;
    }
}

// ---- constants over boxes and lists ------------------------------------------------------------------------
struct FieldPtrs {
    float* f[3];            // scalar: f[0]; vector: one array per component
    uint8_t* solid;         // boundary
    int ncomp;
};

__global__ void k_fill_box(Geo g, FieldPtrs F, int x0, int y0, int z0, int nx, int ny, int nz, float v0, float v1,
                           float v2) {
    const long long n = (long long)nx * ny * nz;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int x = x0 + (int)(k % nx), y = y0 + (int)((k / nx) % ny), z = z0 + (int)(k / ((long long)nx * ny));
        const long long i = (long long)z * g.WH + (long long)y * g.W + x;
        if (F.solid) { F.solid[i] = v0 != 0.0f; continue; }
        F.f[0][i] = v0;
        if (F.ncomp > 1) F.f[1][i] = v1;
        if (F.ncomp > 2) F.f[2][i] = v2;
    }
}

__global__ void k_set_cells(long long N, const int* __restrict__ cells, long long n, FieldPtrs F, float v0, float v1,
                            float v2, DevCtl* ctl) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const long long i = cells[k];
        if (i < 0 || i >= N) { atomicOr(&ctl->error, DEV_ERR_BAD_INDEX); continue; }
        if (F.solid) { F.solid[i] = v0 != 0.0f; continue; }
        F.f[0][i] = v0;
        if (F.ncomp > 1) F.f[1][i] = v1;
        if (F.ncomp > 2) F.f[2][i] = v2;
    }
}

// Editor::initBoundaries' last loop: the outer layer of cells is solid, and rho is 0 in every solid cell.
__global__ void k_seal(Geo g, int dim, uint8_t* __restrict__ solid, float* __restrict__ rho) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g.N; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.W), y = (int)((i / g.W) % g.H), z = (int)(i / g.WH);
        bool border = x == 0 || y == 0 || x == g.W - 1 || y == g.H - 1;
        if (dim == 3) border = border || z == 0 || z == g.D - 1;
        if (border) solid[i] = 1;
        if (solid[i]) rho[i] = 0.0f;
    }
}

// ---- QueryNode metrics ------------------------------------------------------------------------------------
// Per block: cell count, min and max of x, y, z, exact integer sums of x, y, z, and FP64 sums of u, v, w, p;
// the second kernel adds the block partials in block order, so the result does not depend on timing.
struct QPart {
    long long cnt, sx, sy, sz;
    int mnx, mny, mnz, mxx, mxy, mxz;
    double su, sv, sw, sp;
};
constexpr int kQueryBlocks = 304;
constexpr int kQueryThreads = 256;

struct QueryArgs {
    Geo g;
    int x0, y0, z0, nx, ny, nz;
    int only_fluid;
    const float *rho, *u, *v, *w, *p;
    QPart* part;
};

__device__ __forceinline__ void q_merge(QPart& a, const QPart& b) {
    a.cnt += b.cnt; a.sx += b.sx; a.sy += b.sy; a.sz += b.sz;
    a.mnx = min(a.mnx, b.mnx); a.mny = min(a.mny, b.mny); a.mnz = min(a.mnz, b.mnz);
    a.mxx = max(a.mxx, b.mxx); a.mxy = max(a.mxy, b.mxy); a.mxz = max(a.mxz, b.mxz);
    a.su += b.su; a.sv += b.sv; a.sw += b.sw; a.sp += b.sp;
}
__device__ __forceinline__ QPart q_empty() {
    QPart q;
    q.cnt = q.sx = q.sy = q.sz = 0;
    q.mnx = q.mny = q.mnz = INT_MAX;
    q.mxx = q.mxy = q.mxz = INT_MIN;
    q.su = q.sv = q.sw = q.sp = 0.0;
    return q;
}

__device__ void q_block_reduce(QPart& q, QPart* s) {
    s[threadIdx.x] = q;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) q_merge(s[threadIdx.x], s[threadIdx.x + h]);
        __syncthreads();
    }
    q = s[0];
}

__global__ void __launch_bounds__(kQueryThreads) k_query(QueryArgs a) {
    __shared__ QPart s[kQueryThreads];
    QPart q = q_empty();
    const long long n = (long long)a.nx * a.ny * a.nz;
    // block b takes the contiguous range [b*n/B, (b+1)*n/B) so the order of its sums is fixed
    const long long lo = n * blockIdx.x / gridDim.x, hi = n * (blockIdx.x + 1) / gridDim.x;
    for (long long k = lo + threadIdx.x; k < hi; k += blockDim.x) {
        const int x = a.x0 + (int)(k % a.nx), y = a.y0 + (int)((k / a.nx) % a.ny), z = a.z0 + (int)(k / ((long long)a.nx * a.ny));
        const long long i = (long long)z * a.g.WH + (long long)y * a.g.W + x;
        if (a.only_fluid && a.rho[i] < 0.5f) continue;
        q.cnt += 1; q.sx += x; q.sy += y; q.sz += z;
        q.mnx = min(q.mnx, x); q.mny = min(q.mny, y); q.mnz = min(q.mnz, z);
        q.mxx = max(q.mxx, x); q.mxy = max(q.mxy, y); q.mxz = max(q.mxz, z);
        q.su += a.u[i]; q.sv += a.v[i]; if (a.w) q.sw += a.w[i]; q.sp += a.p[i];
    }
    q_block_reduce(q, s);
    if (threadIdx.x == 0) a.part[blockIdx.x] = q;
}

__global__ void __launch_bounds__(kQueryThreads) k_query_final(const QPart* __restrict__ part, int nparts, efs_query_metrics* out) {
    __shared__ QPart s[kQueryThreads];
    QPart q = q_empty();
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) q_merge(q, part[b]);
    q_block_reduce(q, s);
    if (threadIdx.x != 0) return;
    efs_query_metrics m;
    m.count = q.cnt;
    if (q.cnt > 0) {
        const double c = (double)q.cnt;
        m.max_position[0] = (float)q.mxx; m.max_position[1] = (float)q.mxy; m.max_position[2] = (float)q.mxz;
        m.min_position[0] = (float)q.mnx; m.min_position[1] = (float)q.mny; m.min_position[2] = (float)q.mnz;
        m.avg_position[0] = (float)(q.sx / c); m.avg_position[1] = (float)(q.sy / c); m.avg_position[2] = (float)(q.sz / c);
        m.velocity[0] = (float)(q.su / c); m.velocity[1] = (float)(q.sv / c); m.velocity[2] = (float)(q.sw / c);
        m.pressure = (float)(q.sp / c);
    } else {
        for (int d = 0; d < 3; d++) {
            m.max_position[d] = m.min_position[d] = m.avg_position[d] = m.velocity[d] = 0.0f;
        }
        m.pressure = 0.0f;
    }
    m.pad = 0;
    *out = m;
}

int blocks_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    return (int)std::max(1LL, std::min(b, 152LL * 16));
}

}  // namespace

// ---- launchers called by the C ABI (efs_api.cu) -------------------------------------------------------------
bool scene_field_ptrs(efs_ctx* c, int field, FieldPtrsOut& out) {
    out = FieldPtrsOut{};
    switch (field) {
        case EFS_FIELD_VEL: out.f[0] = c->u; out.f[1] = c->v; out.f[2] = c->w; out.ncomp = c->dim; return true;
        case EFS_FIELD_FORCES: out.f[0] = c->fx; out.f[1] = c->fy; out.f[2] = c->fz; out.ncomp = c->dim; return true;
        case EFS_FIELD_RHO: out.f[0] = c->rho; out.ncomp = 1; return true;
        case EFS_FIELD_GAMMA: out.f[0] = c->gamma; out.ncomp = 1; return true;
        case EFS_FIELD_BETA: out.f[0] = c->beta; out.ncomp = 1; return true;
        case EFS_FIELD_DIVERGENCE: out.f[0] = c->div; out.ncomp = 1; return true;
        case EFS_FIELD_PRESSURE: out.f[0] = c->p; out.ncomp = 1; return true;
        case EFS_FIELD_BOUNDARY: out.solid = c->solid; out.ncomp = 1; return true;
        default: return false;
    }
}

static FieldPtrs to_ptrs(const FieldPtrsOut& o) {
    FieldPtrs F;
    for (int d = 0; d < 3; d++) F.f[d] = o.f[d];
    F.solid = o.solid;
    F.ncomp = o.ncomp;
    return F;
}

cudaError_t launch_mesh_label(efs_ctx* c, const float* d_tris, int ntri, const float center[3], const float size[3],
                              float vin, float vout, int field, uint8_t* mask) {
    LabelArgs a;
    a.g = c->g;
    a.tris = reinterpret_cast<const float4*>(d_tris);
    a.ntri = ntri;
    a.cx = center[0]; a.cy = center[1]; a.cz = center[2];
    a.sx = size[0]; a.sy = size[1]; a.sz = size[2];
    a.vin = vin; a.vout = vout;
    a.fout = nullptr; a.bout = nullptr;
    if (mask) { a.out_kind = LABEL_MASK; a.bout = mask; }
    else if (field == EFS_FIELD_BOUNDARY) { a.out_kind = LABEL_SOLID; a.bout = c->solid; }
    else {
        FieldPtrsOut o;
        if (!scene_field_ptrs(c, field, o) || o.ncomp != 1) return cudaErrorInvalidValue;
        a.out_kind = LABEL_FLOAT;
        a.fout = o.f[0];
    }
    const long long ncell = (long long)(c->g.W - 1) * (c->g.H - 1) * (c->g.D - 1);
    if (ncell <= 0) return cudaSuccess;
    const long long blocks = (ncell + kLabelThreads - 1) / kLabelThreads;
    k_mesh_label<<<(unsigned)blocks, kLabelThreads, 0, c->stream>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mask_compact(efs_ctx* c, const uint8_t* mask, int* d_out, long long cap, int* d_counts,
                                long long* d_offsets) {
    const long long n = c->g.N;
    const int ntiles = (int)((n + kTile - 1) / kTile);
    k_mask_count<<<ntiles, kTile, 0, c->stream>>>(mask, n, d_counts);
    k_scan_counts<<<1, 1024, 0, c->stream>>>(d_counts, ntiles, d_offsets);
    k_mask_write<<<ntiles, kTile, 0, c->stream>>>(mask, n, d_offsets, d_out, cap);
    return cudaGetLastError();
}

long long mask_tiles(const efs_ctx* c) { return (c->g.N + kTile - 1) / kTile; }

cudaError_t launch_fill_box(efs_ctx* c, int field, const int lo[3], const int hi[3], const float* value) {
    FieldPtrsOut o;
    if (!scene_field_ptrs(c, field, o)) return cudaErrorInvalidValue;
    const int nx = hi[0] - lo[0], ny = hi[1] - lo[1], nz = hi[2] - lo[2];
    if (nx <= 0 || ny <= 0 || nz <= 0) return cudaSuccess;
    const float v1 = o.ncomp > 1 ? value[1] : 0.0f, v2 = o.ncomp > 2 ? value[2] : 0.0f;
    k_fill_box<<<blocks_for((long long)nx * ny * nz, 256), 256, 0, c->stream>>>(c->g, to_ptrs(o), lo[0], lo[1], lo[2],
                                                                                nx, ny, nz, value[0], v1, v2);
    return cudaGetLastError();
}

cudaError_t launch_set_cells(efs_ctx* c, int field, const int* d_cells, long long n, const float* value) {
    FieldPtrsOut o;
    if (!scene_field_ptrs(c, field, o)) return cudaErrorInvalidValue;
    if (n <= 0) return cudaSuccess;
    const float v1 = o.ncomp > 1 ? value[1] : 0.0f, v2 = o.ncomp > 2 ? value[2] : 0.0f;
    k_set_cells<<<blocks_for(n, 256), 256, 0, c->stream>>>(c->g.N, d_cells, n, to_ptrs(o), value[0], v1, v2, c->ctl);
    return cudaGetLastError();
}

cudaError_t launch_seal_boundary(efs_ctx* c) {
    k_seal<<<blocks_for(c->g.N, 256), 256, 0, c->stream>>>(c->g, c->dim, c->solid, c->rho);
    return cudaGetLastError();
}

size_t query_scratch_bytes() { return sizeof(QPart) * kQueryBlocks + sizeof(efs_query_metrics) + 64; }

cudaError_t launch_query_box(efs_ctx* c, const int lo[3], const int hi[3], int only_fluid, void* scratch,
                             efs_query_metrics* d_out) {
    QueryArgs a;
    a.g = c->g;
    a.x0 = lo[0]; a.y0 = lo[1]; a.z0 = lo[2];
    a.nx = std::max(0, hi[0] - lo[0]); a.ny = std::max(0, hi[1] - lo[1]); a.nz = std::max(0, hi[2] - lo[2]);
    a.only_fluid = only_fluid;
    a.rho = c->rho; a.u = c->u; a.v = c->v; a.w = c->dim == 3 ? c->w : nullptr; a.p = c->p;
    a.part = reinterpret_cast<QPart*>(scratch);
    k_query<<<kQueryBlocks, kQueryThreads, 0, c->stream>>>(a);
    k_query_final<<<1, kQueryThreads, 0, c->stream>>>(a.part, kQueryBlocks, d_out);
    return cudaGetLastError();
}

}  // namespace efs
