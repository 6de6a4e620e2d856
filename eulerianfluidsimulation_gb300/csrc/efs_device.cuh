// efs_device.cuh — device-side building blocks of the liquid step (sm_103a).
//
// Field store: structure-of-arrays in HBM, one float array per scalar and per velocity component, indexed
// like the reference (x fastest; i = z*W*H + y*W + x, the one-cell wall border included).  Solid cells are
// one byte each (1 = boundary 1.0).  The interpolation and tracing helpers below restate the reference's
// CPU functions operation by operation; the simulation translation units are compiled with --fmad=false so
// that every product and sum rounds separately, as in the reference's x86-64 build.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace efs {

// Grid geometry passed by value to every kernel.
struct Geo {
    int W, H, D;      // cells per axis including the border (D == 1 in 2D)
    int WH;           // W * H
    int N;            // W * H * D
};

// a / b in FP64 without the FP64 division sequence (about 550 cycles of dependent latency on GB300): a
// float reciprocal refined by two Newton steps in FP64, relative error near 1e-16.  Falls back to the
// division when b is outside the range where the float reciprocal is finite and normal.
__device__ __forceinline__ double div_fast(double a, double b) {
    const float bf = (float)b;
    float r0 = 1.0f / bf;
    if (!(fabsf(r0) < 1e37f && fabsf(r0) > 1e-37f)) return a / b;
    double r = (double)r0;
    r = fma(r, fma(-b, r, 1.0), r);
    r = fma(r, fma(-b, r, 1.0), r);
    return a * r;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (hi < v ? hi : v); }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }
__device__ __forceinline__ float maxf(float a, float b) { return (a < b) ? b : a; }   // std::max
__device__ __forceinline__ float minf(float a, float b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ double maxd(double a, double b) { return (a < b) ? b : a; }

// ---------------------------------------------------------------------------------------------------
// 3D
// ---------------------------------------------------------------------------------------------------

// VecField3D::trilinear_interpolation (src/simulation/data/VecField3D.cpp:21-50) for one component whose
// staggering offset is (ox, oy, oz).
__device__ __forceinline__ float vtrilin3(const float* __restrict__ f, const Geo& g, float px, float py, float pz,
                                          int lx, int ly, int lz, float ox, float oy, float oz) {
    const float x0 = (float)lx + ox, y0 = (float)ly + oy, z0 = (float)lz + oz;
    const float tx = px - x0, ty = py - y0, tz = pz - z0;
    const int i = lz * g.WH + ly * g.W + lx;
    const float v000 = __ldg(f + i), v001 = __ldg(f + i + g.WH);
    const float v010 = __ldg(f + i + g.W), v011 = __ldg(f + i + g.W + g.WH);
    const float v100 = __ldg(f + i + 1), v101 = __ldg(f + i + 1 + g.WH);
    const float v110 = __ldg(f + i + 1 + g.W), v111 = __ldg(f + i + 1 + g.W + g.WH);
    const float v00 = v000 * (1.0f - tz) + v001 * tz;
    const float v01 = v010 * (1.0f - tz) + v011 * tz;
    const float v10 = v100 * (1.0f - tz) + v101 * tz;
    const float v11 = v110 * (1.0f - tz) + v111 * tz;
    const float vLow = v00 * (1.0f - ty) + v01 * ty;
    const float vHigh = v10 * (1.0f - ty) + v11 * ty;
    return vLow * (1.0f - tx) + vHigh * tx;
}

// VecField3D::interpolate (VecField3D.cpp:54-78): lowIndex = (int)(floor(coord - offset) + 1e-10f),
// offsets (-1,-.5,-.5), (-.5,-1,-.5), (-.5,-.5,-1) (StaggeredOffset3D, :12-19).  The + 1e-10f is left out:
// floor gives an integer-valued float F, and F + 1e-10f rounds back to F when |F| >= 1 (1e-10 is below half an
// ulp of 1) and truncates to 0 when F is +-0, so the index is (int)F either way (fidx below).  The traces are
// bound by instruction issue, and this is 9 additions per velocity sample.
__device__ __forceinline__ int fidx(float v) { return (int)floorf(v); }
__device__ __forceinline__ void vinterp3(const float* __restrict__ u, const float* __restrict__ v,
                                         const float* __restrict__ w, const Geo& g, float px, float py, float pz,
                                         float& ou, float& ov, float& ow) {
    {
        const int lx = fidx(px + 1.0f), ly = fidx(py + 0.5f),
                  lz = fidx(pz + 0.5f);
        ou = vtrilin3(u, g, px, py, pz, lx, ly, lz, -1.0f, -0.5f, -0.5f);
    }
    {
        const int lx = fidx(px + 0.5f), ly = fidx(py + 1.0f),
                  lz = fidx(pz + 0.5f);
        ov = vtrilin3(v, g, px, py, pz, lx, ly, lz, -0.5f, -1.0f, -0.5f);
    }
    {
        const int lx = fidx(px + 0.5f), ly = fidx(py + 0.5f),
                  lz = fidx(pz + 1.0f);
        ow = vtrilin3(w, g, px, py, pz, lx, ly, lz, -0.5f, -0.5f, -1.0f);
    }
}

// a / d for d the distance of two (clamped) cell centres, which is exactly 1 or 0: a / 1 is a exactly, so only
// other values divide (IEEE division is a long instruction sequence and the scalar samples run once per cell).
__device__ __forceinline__ float div_spacing(float a, float d) { return d == 1.0f ? a : a / d; }

// ScalField3D::interpolate (src/simulation/data/ScalField3D.cpp:18-107): samples at i + 0.5, clamped.
__device__ __forceinline__ float sinterp3(const float* __restrict__ f, const Geo& g, float px, float py, float pz) {
    const int x = (int)px, y = (int)py, z = (int)pz;
    int ix1 = x, ix2 = x + 1;
    if (px - (float)x < 0.5f) { ix1 = x - 1; ix2 = x; }
    int iy1 = y, iy2 = y + 1;
    if (py - (float)y < 0.5f) { iy1 = y - 1; iy2 = y; }
    int iz1 = z, iz2 = z + 1;
    if (pz - (float)z < 0.5f) { iz1 = z - 1; iz2 = z; }
    ix1 = clampi(ix1, 0, g.W - 1); ix2 = clampi(ix2, 0, g.W - 1);
    iy1 = clampi(iy1, 0, g.H - 1); iy2 = clampi(iy2, 0, g.H - 1);
    iz1 = clampi(iz1, 0, g.D - 1); iz2 = clampi(iz2, 0, g.D - 1);
    const float v0 = f[iz1 * g.WH + iy1 * g.W + ix1], v1 = f[iz2 * g.WH + iy1 * g.W + ix1];
    const float v2 = f[iz1 * g.WH + iy2 * g.W + ix1], v3 = f[iz2 * g.WH + iy2 * g.W + ix1];
    const float v4 = f[iz1 * g.WH + iy1 * g.W + ix2], v5 = f[iz2 * g.WH + iy1 * g.W + ix2];
    const float v6 = f[iz1 * g.WH + iy2 * g.W + ix2], v7 = f[iz2 * g.WH + iy2 * g.W + ix2];
    const float x1 = (float)ix1 + 0.5f, x2 = (float)ix2 + 0.5f;
    const float y1 = (float)iy1 + 0.5f, y2 = (float)iy2 + 0.5f;
    const float z1 = (float)iz1 + 0.5f, z2 = (float)iz2 + 0.5f;
    const float dz2z1 = z2 - z1;
    float f00, f01, f10, f11;
    if (dz2z1 < 1e-9f) { f00 = v1; f01 = v3; f10 = v5; f11 = v7; }
    else {
        const float wz1 = div_spacing(z2 - pz, dz2z1), wz2 = div_spacing(pz - z1, dz2z1);
        f00 = wz1 * v0 + wz2 * v1; f01 = wz1 * v2 + wz2 * v3;
        f10 = wz1 * v4 + wz2 * v5; f11 = wz1 * v6 + wz2 * v7;
    }
    const float dy2y1 = y2 - y1;
    float fx1, fx2;
    if (dy2y1 < 1e-9f) { fx1 = f01; fx2 = f11; }
    else {
        const float wy1 = div_spacing(y2 - py, dy2y1), wy2 = div_spacing(py - y1, dy2y1);
        fx1 = wy1 * f00 + wy2 * f01; fx2 = wy1 * f10 + wy2 * f11;
    }
    const float dx2x1 = x2 - x1;
    if (dx2x1 < 1e-9f) return fx2;
    const float wx1 = div_spacing(x2 - px, dx2x1), wx2 = div_spacing(px - x1, dx2x1);
    return wx1 * fx1 + wx2 * fx2;
}

// Grid3D::traceParticle inWall (src/simulation/data/Grid3D.cpp:73-80)
__device__ __forceinline__ bool inwall3(const uint8_t* __restrict__ solid, const Geo& g, float px, float py, float pz) {
    const float W = (float)g.W, H = (float)g.H, D = (float)g.D;
    if (px < 1.f || px > W - 2.f || py < 1.f || py > H - 2.f || pz < 1.f || pz > D - 2.f) return true;
    const int ix = clampi((int)px, 0, g.W - 1), iy = clampi((int)py, 0, g.H - 1), iz = clampi((int)pz, 0, g.D - 1);
    return __ldg(solid + iz * g.WH + iy * g.W + ix) != 0;
}

// Grid3D::traceParticle (Grid3D.cpp:66-122): RK2 midpoint with the midpoint clamped, 8-step bisection when a
// substep ends in a wall, start returned unchanged when it is inside a wall.
__device__ __forceinline__ void trace3(const float* __restrict__ u, const float* __restrict__ v,
                                       const float* __restrict__ w, const uint8_t* __restrict__ solid, const Geo& g,
                                       float sx, float sy, float sz, float dt, int substeps,
                                       float& ox, float& oy, float& oz) {
    ox = sx; oy = sy; oz = sz;
    if (inwall3(solid, g, sx, sy, sz)) return;
    const float W = (float)g.W, H = (float)g.H, D = (float)g.D;
    const float subDt = dt / (float)substeps;
    const float h = subDt * 0.5f;
    float px = sx, py = sy, pz = sz;
    for (int s = 0; s < substeps; s++) {
        float k1x, k1y, k1z, k2x, k2y, k2z;
        vinterp3(u, v, w, g, px - 0.5f, py - 0.5f, pz - 0.5f, k1x, k1y, k1z);
        const float mx = clampf(px + k1x * h, 1.f, W - 2.f);
        const float my = clampf(py + k1y * h, 1.f, H - 2.f);
        const float mz = clampf(pz + k1z * h, 1.f, D - 2.f);
        vinterp3(u, v, w, g, mx - 0.5f, my - 0.5f, mz - 0.5f, k2x, k2y, k2z);
        const float nx = px + k2x * subDt, ny = py + k2y * subDt, nz = pz + k2z * subDt;
        if (inwall3(solid, g, nx, ny, nz)) {
            float sfx = px, sfy = py, sfz = pz, ux = nx, uy = ny, uz = nz;
            for (int b = 0; b < 8; b++) {
                const float hx = (sfx + ux) * 0.5f, hy = (sfy + uy) * 0.5f, hz = (sfz + uz) * 0.5f;
                if (inwall3(solid, g, hx, hy, hz)) { ux = hx; uy = hy; uz = hz; }
                else { sfx = hx; sfy = hy; sfz = hz; }
            }
            ox = sfx; oy = sfy; oz = sfz;
            return;
        }
        px = nx; py = ny; pz = nz;
    }
    ox = px; oy = py; oz = pz;
}

// Integer-centred trilinear corner weights of CPUSimulator3D::rho_advect (CPUSimulator3D.cpp:140-161,
// :195-216): corner k = (k & 1, k >> 1 & 1, k >> 2 & 1) from floor(pos); zero at solid corners; returns the
// sum in the reference's order and the base index.
__device__ __forceinline__ float corner_weights3(const uint8_t* __restrict__ solid, const Geo& g, float px, float py,
                                                 float pz, int& base, float m[8]) {
    const int p0x = (int)floorf(px), p0y = (int)floorf(py), p0z = (int)floorf(pz);
    const float dx0 = 1 - (px - (float)p0x), dy0 = 1 - (py - (float)p0y), dz0 = 1 - (pz - (float)p0z);
    const float dx1 = 1 - ((float)(p0x + 1) - px), dy1 = 1 - ((float)(p0y + 1) - py), dz1 = 1 - ((float)(p0z + 1) - pz);
    base = p0z * g.WH + p0y * g.W + p0x;
    const float wx[2] = {dx0, dx1}, wy[2] = {dy0, dy1}, wz[2] = {dz0, dz1};
    float sum = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
        m[k] = 0;
        if (__ldg(solid + base + ox + oy * g.W + oz * g.WH) == 0) m[k] = wx[ox] * wy[oy] * wz[oz];
    }
#pragma unroll
    for (int k = 0; k < 8; k++) sum += m[k];
    return sum;
}

__device__ __forceinline__ int corner_offset3(const Geo& g, int k) {
    return (k & 1) + ((k >> 1) & 1) * g.W + ((k >> 2) & 1) * g.WH;
}

// ---------------------------------------------------------------------------------------------------
// 2D
// ---------------------------------------------------------------------------------------------------

// VecField2D::bilinear_interpolation / interpolate (src/simulation/data/VecField2D.cpp:26-63)
__device__ __forceinline__ float vbilin2(const float* __restrict__ f, const Geo& g, float px, float py, int lx, int ly,
                                         float ox, float oy) {
    const float x0 = (float)lx + ox, y0 = (float)ly + oy;
    const float tx = px - x0, ty = py - y0;
    const int i = ly * g.W + lx;
    const float v00 = __ldg(f + i), v01 = __ldg(f + i + g.W), v10 = __ldg(f + i + 1), v11 = __ldg(f + i + 1 + g.W);
    const float vLow = v00 * (1.0f - ty) + v01 * ty;
    const float vHigh = v10 * (1.0f - ty) + v11 * ty;
    return vLow * (1.0f - tx) + vHigh * tx;
}

__device__ __forceinline__ void vinterp2(const float* __restrict__ u, const float* __restrict__ v, const Geo& g,
                                         float px, float py, float& ou, float& ov) {
    ou = vbilin2(u, g, px, py, fidx(px + 1.0f), fidx(py + 0.5f), -1.0f, -0.5f);
    ov = vbilin2(v, g, px, py, fidx(px + 0.5f), fidx(py + 1.0f), -0.5f, -1.0f);
}

// ScalField2D::interpolate (src/simulation/data/ScalField2D.cpp:20-69), including its pos += 1 shift.
__device__ __forceinline__ float sinterp2(const float* __restrict__ f, const Geo& g, float px, float py) {
    px += 1.f; py += 1.f;
    const int x = (int)px, y = (int)py;
    int ix1 = x, ix2 = x + 1;
    if (px - (float)x < 0.5f) { ix1 = x - 1; ix2 = x; }
    int iy1 = y, iy2 = y + 1;
    if (py - (float)y < 0.5f) { iy1 = y - 1; iy2 = y; }
    ix1 = clampi(ix1, 0, g.W - 1); ix2 = clampi(ix2, 0, g.W - 1);
    iy1 = clampi(iy1, 0, g.H - 1); iy2 = clampi(iy2, 0, g.H - 1);
    const float v0 = f[iy1 * g.W + ix1], v1 = f[iy2 * g.W + ix1], v2 = f[iy1 * g.W + ix2], v3 = f[iy2 * g.W + ix2];
    const float x1 = (float)ix1 + 0.5f, x2 = (float)ix2 + 0.5f, y1 = (float)iy1 + 0.5f, y2 = (float)iy2 + 0.5f;
    const float dx2x1 = x2 - x1;
    float fxy1 = (div_spacing(x2 - px, dx2x1)) * v0 + (div_spacing(px - x1, dx2x1)) * v2;
    float fxy2 = (div_spacing(x2 - px, dx2x1)) * v1 + (div_spacing(px - x1, dx2x1)) * v3;
    if ((double)dx2x1 < 1e-9) { fxy1 = v1; fxy2 = v3; }
    const float dy2y1 = y2 - y1;
    float fxy = (div_spacing(y2 - py, dy2y1)) * fxy1 + (div_spacing(py - y1, dy2y1)) * fxy2;
    if ((double)dy2y1 < 1e-9) fxy = fxy1;
    return fxy;
}

// Grid2D::traceParticle (src/simulation/data/Grid2D.cpp:84-137)
__device__ __forceinline__ bool inwall2(const uint8_t* __restrict__ solid, const Geo& g, float px, float py) {
    const float W = (float)g.W, H = (float)g.H;
    if (px < 1.f || px > W - 2.f || py < 1.f || py > H - 2.f) return true;
    const int ix = clampi((int)px, 0, g.W - 1), iy = clampi((int)py, 0, g.H - 1);
    return __ldg(solid + iy * g.W + ix) != 0;
}

__device__ __forceinline__ void trace2(const float* __restrict__ u, const float* __restrict__ v,
                                       const uint8_t* __restrict__ solid, const Geo& g, float sx, float sy, float dt,
                                       int substeps, float& ox, float& oy) {
    ox = sx; oy = sy;
    if (inwall2(solid, g, sx, sy)) return;
    const float W = (float)g.W, H = (float)g.H;
    const float subDt = dt / (float)substeps;
    const float h = subDt * 0.5f;
    float px = sx, py = sy;
    for (int s = 0; s < substeps; s++) {
        float k1x, k1y, k2x, k2y;
        vinterp2(u, v, g, px - 0.5f, py - 0.5f, k1x, k1y);
        const float mx = clampf(px + k1x * h, 1.f, W - 2.f), my = clampf(py + k1y * h, 1.f, H - 2.f);
        vinterp2(u, v, g, mx - 0.5f, my - 0.5f, k2x, k2y);
        const float nx = px + k2x * subDt, ny = py + k2y * subDt;
        if (inwall2(solid, g, nx, ny)) {
            float sfx = px, sfy = py, ux = nx, uy = ny;
            for (int b = 0; b < 8; b++) {
                const float hx = (sfx + ux) * 0.5f, hy = (sfy + uy) * 0.5f;
                if (inwall2(solid, g, hx, hy)) { ux = hx; uy = hy; } else { sfx = hx; sfy = hy; }
            }
            ox = sfx; oy = sfy;
            return;
        }
        px = nx; py = ny;
    }
    ox = px; oy = py;
}

// Corner weights of CPUSimulator2D::rho_advect (src/simulation/simulator/CPUSimulator2D.cpp:149-163)
__device__ __forceinline__ float corner_weights2(const uint8_t* __restrict__ solid, const Geo& g, float px, float py,
                                                 int& base, float m[4]) {
    const int p0x = (int)floorf(px), p0y = (int)floorf(py);
    const float dx0 = 1 - (px - (float)p0x), dy0 = 1 - (py - (float)p0y);
    const float dx1 = 1 - ((float)(p0x + 1) - px), dy1 = 1 - ((float)(p0y + 1) - py);
    base = p0y * g.W + p0x;
    m[0] = m[1] = m[2] = m[3] = 0;
    if (__ldg(solid + base) == 0) m[0] = dx0 * dy0;
    if (__ldg(solid + base + 1) == 0) m[1] = dx1 * dy0;
    if (__ldg(solid + base + g.W) == 0) m[2] = dx0 * dy1;
    if (__ldg(solid + base + g.W + 1) == 0) m[3] = dx1 * dy1;
    return m[0] + m[1] + m[2] + m[3];
}

__device__ __forceinline__ int corner_offset2(const Geo& g, int k) { return (k & 1) + ((k >> 1) & 1) * g.W; }

// per-axis term of max_inc / max_dec (CPUSimulator3D.cpp:390-418): std::pow(float, int) is evaluated in double
__device__ __forceinline__ double sq_d(float v) { return (double)v * (double)v; }

// (r - 0.5)^3 of the sharpening weight (CPUSimulator3D.cpp:431, std::pow(float, 3.f)): cube in double,
// rounded once to float.
__device__ __forceinline__ float cube_f(float x) {
    const double d = (double)x;
    return (float)(d * d * d);
}

}  // namespace efs
