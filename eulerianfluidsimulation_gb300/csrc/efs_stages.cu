// efs_stages.cu — the seven stages of the liquid step as sm_103a kernels (3D and 2D).
//
// Each kernel restates one loop of the reference CPU backend (src/simulation/simulator/CPUSimulator3D.cpp,
// CPUSimulator2D.cpp); the comments give the lines.  Where the reference loop is order dependent the kernels
// keep its result:
//   - density diffusion sweeps are in place along one axis; rows along that axis are independent, so one
//     thread walks one row sequentially (CPUSimulator3D.cpp:276-363);
//   - the Chentanez-Mueller matrix A is stored as 8 backward weights per row plus 8 forward weights per
//     column (no hash map); row and column sums that the reference forms by iterating over A become passes
//     over those weights with atomic adds for the scattered part.
// Density sharpening applies every cell's change, then traces every changed cell on that field, then
// scatters (EFS_SHARPEN_PARALLEL); the reference interleaves the three per cell, which
// EFS_SHARPEN_SEQUENTIAL reproduces on one thread for parity.
#include <mutex>

#include "efs_batch.h"
#include "efs_internal.h"

namespace efs {

namespace {

constexpr int BX = 32, BY = 8;

__device__ __forceinline__ bool cell3(const Geo& g, int bx, int by, int bz, int& x, int& y, int& z, int& i) {
    x = 1 + bx * blockDim.x + threadIdx.x;
    y = 1 + by * blockDim.y + threadIdx.y;
    z = 1 + bz;
    if (x > g.W - 2 || y > g.H - 2) return false;
    i = z * g.WH + y * g.W + x;
    return true;
}
__device__ __forceinline__ bool cell2(const Geo& g, int bx, int by, int& x, int& y, int& i) {
    x = 1 + bx * blockDim.x + threadIdx.x;
    y = 1 + by * blockDim.y + threadIdx.y;
    if (x > g.W - 2 || y > g.H - 2) return false;
    i = y * g.W + x;
    return true;
}

// ------------------------------------------------------------------------------------------------
// stage 0: vel_decay (CPUSimulator3D.cpp:54-59, CPUSimulator2D.cpp:65-70)
// ------------------------------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void d_vel_decay(const Geo& g, int bx, int by, int bz, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, const float* __restrict__ rho, float k) {
    int x, y, z = 0, i;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, i)) return; } else { if (!cell2(g, bx, by, x, y, i)) return; }
    if ((double)rho[i] < 0.5) {
        u[i] *= k; v[i] *= k;
        if (DIM == 3) w[i] *= k;
    }
}
template <int DIM>
__global__ void k_vel_decay(Geo g, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                            const float* __restrict__ rho, float k) {
    d_vel_decay<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, u, v, w, rho, k);
}

// ------------------------------------------------------------------------------------------------
// stage 1: vel_extrapolate (CPUSimulator3D.cpp:61-111, CPUSimulator2D.cpp:72-120)
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void d_extrap_init(const Geo& g, int bx, int by, int bz, int dim, const float* __restrict__ rho, const uint8_t* __restrict__ solid, uint8_t* __restrict__ valid) {
    const int i = bx * blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    const int x = i % g.W, y = (i / g.W) % g.H, z = i / g.WH;
    bool interior = x >= 1 && x <= g.W - 2 && y >= 1 && y <= g.H - 2;
    if (dim == 3) interior = interior && z >= 1 && z <= g.D - 2;
    valid[i] = (interior && rho[i] >= 0.5f && solid[i] == 0) ? 1 : 0;
}
__global__ void k_extrap_init(Geo g, int dim, const float* __restrict__ rho, const uint8_t* __restrict__ solid,
                              uint8_t* __restrict__ valid) {
    d_extrap_init(g, blockIdx.x, blockIdx.y, blockIdx.z, dim, rho, solid, valid);
}

template <int DIM>
// From the second pass on (`settled`), the destination of a pass is the source of the pass before, so it
// already holds every cell that pass copied: solid cells, cells that stayed invalid, and cells that were
// valid in that pass's source mask, which is what dV holds before this pass writes it.  Those cells are
// skipped; only cells that became valid in the last two passes are written.  Valid cells stay valid.
__device__ __forceinline__ void d_extrap_pass(const Geo& g, int bx, int by, int bz, const float* __restrict__ su, const float* __restrict__ sv, const float* __restrict__ sw, const uint8_t* __restrict__ sV, float* __restrict__ du, float* __restrict__ dv, float* __restrict__ dw, uint8_t* __restrict__ dV, const uint8_t* __restrict__ solid, bool settled = false) {
    int x, y, z = 0, i;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, i)) return; } else { if (!cell2(g, bx, by, x, y, i)) return; }
    if (solid[i]) {
        if (settled) return;
        du[i] = su[i]; dv[i] = sv[i]; if (DIM == 3) dw[i] = sw[i];
        dV[i] = 0;
        return;
    }
    if (sV[i]) {
        if (settled && dV[i]) return;
        du[i] = su[i]; dv[i] = sv[i]; if (DIM == 3) dw[i] = sw[i];
        dV[i] = 1;
        return;
    }
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, n = 0;
    const int nb[6] = {i - 1, i + 1, i - g.W, i + g.W, i - g.WH, i + g.WH};
#pragma unroll
    for (int k = 0; k < 2 * DIM; k++) {
        const int j = nb[k];
        if (sV[j]) {
            s0 += su[j]; s1 += sv[j];
            if (DIM == 3) s2 += sw[j];
            n++;
        }
    }
    if (n > 0) {
        du[i] = s0 / n; dv[i] = s1 / n; if (DIM == 3) dw[i] = s2 / n;
    } else {
        if (settled) return;
        du[i] = su[i]; dv[i] = sv[i]; if (DIM == 3) dw[i] = sw[i];
    }
    dV[i] = (n > 0) ? 1 : 0;
}
template <int DIM>
__global__ void k_extrap_pass(Geo g, const float* __restrict__ su, const float* __restrict__ sv,
                              const float* __restrict__ sw, const uint8_t* __restrict__ sV, float* __restrict__ du,
                              float* __restrict__ dv, float* __restrict__ dw, uint8_t* __restrict__ dV,
                              const uint8_t* __restrict__ solid, int settled) {
    d_extrap_pass<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, su, sv, sw, sV, du, dv, dw, dV, solid, settled != 0);
}

// ------------------------------------------------------------------------------------------------
// stage 2: rho_sharpen (CPUSimulator3D.cpp:366-456 with trace_along_field :568-607 and scatter_values
// :609-655; 2D CPUSimulator2D.cpp:320-402, :526-595)
// ------------------------------------------------------------------------------------------------
template <int DIM>
// (batched scenes: the list holds packed cell indices i + ibase and, in sid, the scene of each entry)
__device__ __forceinline__ void d_sharpen_calc(const Geo& g, int bx, int by, int bz, const float* __restrict__ rho,
                                               float delT, int* __restrict__ idx, float* __restrict__ val, DevCtl* ctl,
                                               int cap, int ibase = 0, int scene = 0, int* __restrict__ sid = nullptr) {
    int x, y, z = 0, i;
    bool ok;
    if (DIM == 3) ok = cell3(g, bx, by, bz, x, y, z, i); else ok = cell2(g, bx, by, x, y, i);
    float dr = 0.f;
    // Cells whose result is decided without the slope terms: rho < 1e-5 gives dr = -rho, and rho > 0.5 gives
    // dr = 0 (there the weight is >= 0, so rho + dr >= rho > 0 and the reference's second branch applies).
    // Only the interface band 1e-5 <= rho <= 0.5 (or NaN) evaluates the FP64 slope terms below.
    const float r0 = ok ? rho[i] : 0.f;
    const bool settled = ok && ((double)r0 < 1e-5 || r0 > 0.5f);
    if (settled) dr = ((double)r0 < 1e-5) ? -r0 : 0.f;
    if (ok && !settled) {
        const float r = r0;
        const float rxm = rho[i - 1], rxp = rho[i + 1], rym = rho[i - g.W], ryp = rho[i + g.W];
        const float dpx = -(r - rxm) * delT, dmx = -(rxp - r) * delT;
        const float dpy = -(r - rym) * delT, dmy = -(ryp - r) * delT;
        double inc = maxd(sq_d(maxf(dpx, 0.f)), sq_d(minf(dmx, 0.f))) + maxd(sq_d(maxf(dpy, 0.f)), sq_d(minf(dmy, 0.f)));
        double dec = maxd(sq_d(minf(dpx, 0.f)), sq_d(maxf(dmx, 0.f))) + maxd(sq_d(minf(dpy, 0.f)), sq_d(maxf(dmy, 0.f)));
        float mx = -INFINITY;
        mx = maxf(mx, fabsf(r - rxm)); mx = maxf(mx, fabsf(r - rxp));
        mx = maxf(mx, fabsf(r - rym)); mx = maxf(mx, fabsf(r - ryp));
        if (DIM == 3) {
            const float rzm = rho[i - g.WH], rzp = rho[i + g.WH];
            const float dpz = -(r - rzm) * delT, dmz = -(rzp - r) * delT;
            inc = inc + maxd(sq_d(maxf(dpz, 0.f)), sq_d(minf(dmz, 0.f)));
            dec = dec + maxd(sq_d(minf(dpz, 0.f)), sq_d(maxf(dmz, 0.f)));
            mx = maxf(mx, fabsf(r - rzm)); mx = maxf(mx, fabsf(r - rzp));
        }
        const float max_inc = (float)sqrt(inc), max_dec = (float)sqrt(dec);
        const float wgt = cube_f(r - 0.5f) * (1 - minf(1.f, mx / 0.2f));
        dr = (wgt >= 0) ? wgt * max_inc : wgt * max_dec;
        if (r + dr < 0 || (double)r < 1e-5) dr = -r;
        else if (r > 0.5f) dr = 0;
    }
    const bool active = ok && !(fabsf(dr) < 1e-6f);
    // warp-aggregated append
    const unsigned mask = __ballot_sync(0xffffffffu, active);
    if (mask == 0) return;
    // the lane within the warp: blocks are 2D (tile_x x tile_y) and tile_x may be below 32, so threadIdx.x is not it
    unsigned lane;
    asm("mov.u32 %0, %%laneid;" : "=r"(lane));
    int base = 0;
    if ((int)lane == __ffs(mask) - 1) base = atomicAdd(&ctl->sh_count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
    if (active) {
        const int slot = base + __popc(mask & ((1u << lane) - 1u));
        if (slot < cap) {
            idx[slot] = i + ibase;
            val[slot] = dr;
            if (sid) sid[slot] = scene;
        }
        else atomicOr(&ctl->error, DEV_ERR_LIST_OVERFLOW);
    }
}
template <int DIM>
__global__ void k_sharpen_calc(Geo g, const float* __restrict__ rho, float delT, int* __restrict__ idx,
                               float* __restrict__ val, DevCtl* ctl, int cap) {
    d_sharpen_calc<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, rho, delT, idx, val, ctl, cap);
}

__global__ void k_sharpen_apply(float* __restrict__ rho, const int* __restrict__ idx, const float* __restrict__ val,
                                const DevCtl* ctl, int cap) {
    const int n = min(ctl->sh_count, cap);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const int i = idx[s];
        float r = rho[i] + val[s];
        rho[i] = maxf(r, 0.f);
    }
}

// Trace of one changed cell up the density gradient (trace_along_field, CPUSimulator3D.cpp:568-607).
template <int DIM>
__device__ __forceinline__ void sharpen_trace_one(const Geo& g, const float* __restrict__ rho, const uint8_t* __restrict__ solid,
                                                  int i, float Dist, float& px, float& py, float& pz) {
    const float stepSize = Dist / (float)10;
    px = (float)(i % g.W); py = (float)((i / g.W) % g.H); pz = (float)(i / g.WH);
    for (int st = 0; st < 10; st++) {
        const float sv = (DIM == 3) ? sinterp3(rho, g, px, py, pz) : sinterp2(rho, g, px, py);
        if (sv >= 0.5f) break;
        const int ix = clampi((int)px, 1, g.W - 2), iy = clampi((int)py, 1, g.H - 2);
        const int iz = (DIM == 3) ? clampi((int)pz, 1, g.D - 2) : 0;
        const int c = iz * g.WH + iy * g.W + ix;
        const float gx = rho[c + 1] - rho[c - 1];
        const float gy = rho[c + g.W] - rho[c - g.W];
        const float gz = (DIM == 3) ? rho[c + g.WH] - rho[c - g.WH] : 0.f;
        const float len = (DIM == 3) ? sqrtf(gx * gx + gy * gy + gz * gz) : sqrtf(gx * gx + gy * gy);
        if (len < 1e-6f) break;
        float nx = px + (gx / len) * stepSize, ny = py + (gy / len) * stepSize;
        nx = clampf(nx, 1.f, (float)g.W - 2.f);
        ny = clampf(ny, 1.f, (float)g.H - 2.f);
        float nz = pz;
        if (DIM == 3) { nz = pz + (gz / len) * stepSize; nz = clampf(nz, 1.f, (float)g.D - 2.f); }
        const int ci = (DIM == 3 ? (int)nz * g.WH : 0) + (int)ny * g.W + (int)nx;
        if (solid[ci]) break;
        px = nx; py = ny; pz = nz;
    }
}

// Trilinear scatter of `value` at (px, py, pz) onto the non-solid corners (scatter_values,
// CPUSimulator3D.cpp:609-655).  ATOMIC: many threads scatter at once (parallel mode); otherwise one thread
// owns rho (sequential mode) and adds in the reference's corner order.
template <int DIM, bool ATOMIC = true>
__device__ __forceinline__ void sharpen_scatter_one(const Geo& g, float* __restrict__ rho, const uint8_t* __restrict__ solid,
                                                    float px, float py, float pz, float value) {
    const int x0 = clampi((int)px, 0, g.W - 1), y0 = clampi((int)py, 0, g.H - 1);
    const int x1 = clampi((int)px + 1, 0, g.W - 1), y1 = clampi((int)py + 1, 0, g.H - 1);
    const float fx = px - (float)(int)px, fy = py - (float)(int)py;
    if (DIM == 3) {
        const int z0 = clampi((int)pz, 0, g.D - 1), z1 = clampi((int)pz + 1, 0, g.D - 1);
        const float fz = pz - (float)(int)pz;
        float w[8];
        w[0] = (1.f - fx) * (1.f - fy) * (1.f - fz);
        w[1] = fx * (1.f - fy) * (1.f - fz);
        w[2] = (1.f - fx) * fy * (1.f - fz);
        w[3] = fx * fy * (1.f - fz);
        w[4] = (1.f - fx) * (1.f - fy) * fz;
        w[5] = fx * (1.f - fy) * fz;
        w[6] = (1.f - fx) * fy * fz;
        w[7] = fx * fy * fz;
        int c[8];
        c[0] = z0 * g.WH + y0 * g.W + x0; c[1] = z0 * g.WH + y0 * g.W + x1;
        c[2] = z0 * g.WH + y1 * g.W + x0; c[3] = z0 * g.WH + y1 * g.W + x1;
        c[4] = z1 * g.WH + y0 * g.W + x0; c[5] = z1 * g.WH + y0 * g.W + x1;
        c[6] = z1 * g.WH + y1 * g.W + x0; c[7] = z1 * g.WH + y1 * g.W + x1;
#pragma unroll
        for (int k = 0; k < 8; k++) if (solid[c[k]]) w[k] = 0.f;
        const float total = w[0] + w[1] + w[2] + w[3] + w[4] + w[5] + w[6] + w[7];
        if (total < 1e-6f) return;
        const float inv = 1.f / total;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            if (ATOMIC) atomicAdd(&rho[c[k]], value * w[k] * inv);
            else rho[c[k]] += value * w[k] * inv;
        }
    } else {
        float w[4];
        w[0] = (1.f - fx) * (1.f - fy); w[1] = fx * (1.f - fy); w[2] = (1.f - fx) * fy; w[3] = fx * fy;
        const int c[4] = {y0 * g.W + x0, y0 * g.W + x1, y1 * g.W + x0, y1 * g.W + x1};
#pragma unroll
        for (int k = 0; k < 4; k++) if (solid[c[k]]) w[k] = 0.f;
        const float total = w[0] + w[1] + w[2] + w[3];
        if (total < 1e-6f) return;
        const float inv = 1.f / total;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (ATOMIC) atomicAdd(&rho[c[k]], value * w[k] * inv);
            else rho[c[k]] += value * w[k] * inv;
        }
    }
}

template <int DIM>
__global__ void k_sharpen_trace(Geo g, const float* __restrict__ rho, const uint8_t* __restrict__ solid,
                                const int* __restrict__ idx, float* __restrict__ ends, float Dist,
                                const DevCtl* ctl, int cap) {
    const int n = min(ctl->sh_count, cap);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        float px, py, pz;
        sharpen_trace_one<DIM>(g, rho, solid, idx[s], Dist, px, py, pz);
        ends[3 * s] = px; ends[3 * s + 1] = py; ends[3 * s + 2] = pz;
    }
}

template <int DIM>
__global__ void k_sharpen_scatter(Geo g, float* __restrict__ rho, const uint8_t* __restrict__ solid,
                                  const float* __restrict__ val, const float* __restrict__ ends, const DevCtl* ctl,
                                  int cap) {
    const int n = min(ctl->sh_count, cap);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        sharpen_scatter_one<DIM>(g, rho, solid, ends[3 * s], ends[3 * s + 1], ends[3 * s + 2], -val[s]);
}

// EFS_SHARPEN_SEQUENTIAL: the reference's loop (CPUSimulator3D.cpp:446-455, CPUSimulator2D.cpp:388-401) in its
// own order.  The changes of every cell were computed from the density before the loop (k_sharpen_calc) and
// spread into the dense array `del` (zero where a cell does not change).  One block walks the cells in index
// order, 1024 at a time: its threads compact that slice's changed cells in order into shared memory, and thread
// 0 then applies, traces and scatters each of them before the next, so every trace sees the density that the
// cells before it left, as in the reference.  rho is written here, so it is read through plain loads.
__global__ void k_sharpen_densify(float* __restrict__ del, const int* __restrict__ idx, const float* __restrict__ val,
                                  const DevCtl* ctl, int cap) {
    const int n = min(ctl->sh_count, cap);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) del[idx[s]] = val[s];
}

constexpr int kSeqThreads = 1024;

template <int DIM>
__global__ void __launch_bounds__(kSeqThreads) k_sharpen_sequential(Geo g, float* rho, const uint8_t* __restrict__ solid,
                                                                   const float* __restrict__ del, float Dist) {
    __shared__ int s_list[kSeqThreads];
    __shared__ int s_off[kSeqThreads / 32];
    __shared__ int s_n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int base = 0; base < g.N; base += kSeqThreads) {
        const int i = base + tid;
        // cells outside the interior were never listed, so their del is 0; a NaN change counts as changed,
        // as in the reference's `std::abs(dr) < 1e-6f` test
        const bool act = i < g.N && !(fabsf(del[i]) < 1e-6f);
        const unsigned m = __ballot_sync(0xffffffffu, act);
        if (lane == 0) s_off[warp] = __popc(m);
        __syncthreads();
        if (warp == 0) {
            const int v = s_off[lane];
            int incl = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            s_off[lane] = incl - v;
            if (lane == 31) s_n = incl;
        }
        __syncthreads();
        if (act) s_list[s_off[warp] + __popc(m & ((1u << lane) - 1u))] = i;
        __syncthreads();
        if (tid == 0) {
            for (int k = 0; k < s_n; k++) {
                const int c = s_list[k];
                const float dr = del[c];
                rho[c] = maxf(rho[c] + dr, 0.f);
                float px, py, pz;
                sharpen_trace_one<DIM>(g, rho, solid, c, Dist, px, py, pz);
                sharpen_scatter_one<DIM, false>(g, rho, solid, px, py, pz, -dr);
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------------------------------------
// stage 3: rho_advect (CPUSimulator3D.cpp:113-364, CPUSimulator2D.cpp:122-318)
// ------------------------------------------------------------------------------------------------

// Steps 1-4: back-trace (shared by steps 1 and 2, which trace the same point), gamma' at the trace end,
// backward weights m_k / sum / gamma', column sums beta1.
template <int DIM>
// tex, tey, tez (optional): the trace end of every interior cell, kept for vel_advect, whose back-trace
// from the cell (CPUSimulator3D.cpp:478-504) is this one: same start, velocity, dt and substeps, and the
// velocity does not change in between (a trace from a solid cell ends at its start).
__device__ __forceinline__ void d_adv_backward(const Geo& g, int bx, int by, int bz, const float* __restrict__ u, const float* __restrict__ v, const float* __restrict__ w, const uint8_t* __restrict__ solid, const float* __restrict__ gamma, float dt, float* __restrict__ wb, int* __restrict__ bb, float* __restrict__ bsum, float* __restrict__ tex = nullptr, float* __restrict__ tey = nullptr, float* __restrict__ tez = nullptr) {
    constexpr int K = (DIM == 3) ? 8 : 4;
    int x, y, z = 0, i;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, i)) return; } else { if (!cell2(g, bx, by, x, y, i)) return; }
    if (solid[i]) {                           // step 1 skips solids; step 2 finds no free corner for them
        bb[i] = -1;
        if (tex) { tex[i] = (float)x; tey[i] = (float)y; if (DIM == 3) tez[i] = (float)z; }
        return;
    }
    float px, py, pz = 0.f, gp;
    float m[K];
    int base;
    float sum;
    if (DIM == 3) {
        trace3(u, v, w, solid, g, (float)x, (float)y, (float)z, -dt, 4, px, py, pz);
        if (tex) { tex[i] = px; tey[i] = py; tez[i] = pz; }
        gp = sinterp3(gamma, g, px, py, pz);
        sum = corner_weights3(solid, g, px, py, pz, base, m);
    } else {
        trace2(u, v, solid, g, (float)x, (float)y, -dt, 4, px, py);
        if (tex) { tex[i] = px; tey[i] = py; }
        gp = sinterp2(gamma, g, px, py);
        sum = corner_weights2(solid, g, px, py, base, m);
    }
    if (sum == 0) { bb[i] = -1; return; }
    bb[i] = base;
#pragma unroll
    for (int k = 0; k < K; k++) {
        float val = m[k] / sum;
        if (gp > 1.e-5f) val /= gp;
        wb[k * g.N + i] = val;
        const int c = base + (DIM == 3 ? corner_offset3(g, k) : corner_offset2(g, k));
        atomicAdd(&bsum[c], val);
    }
}
template <int DIM>
__global__ void k_adv_backward(Geo g, const float* __restrict__ u, const float* __restrict__ v,
                               const float* __restrict__ w, const uint8_t* __restrict__ solid,
                               const float* __restrict__ gamma, float dt, float* __restrict__ wb,
                               int* __restrict__ bb, float* __restrict__ bsum, float* __restrict__ tend) {
    d_adv_backward<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, u, v, w, solid, gamma, dt, wb, bb, bsum, tend,
                        tend ? tend + g.N : nullptr, tend ? tend + 2 * (size_t)g.N : nullptr);
}

// Step 5: forward trace for beta_j < 1; forward weights (1 - beta_j) m_k / sum; their row sums into gsum.
template <int DIM>
__device__ __forceinline__ void d_adv_forward(const Geo& g, int bx, int by, int bz, const float* __restrict__ u, const float* __restrict__ v, const float* __restrict__ w, const uint8_t* __restrict__ solid, const float* __restrict__ bsum, float dt, float* __restrict__ wf, int* __restrict__ fb, float* __restrict__ gsum) {
    constexpr int K = (DIM == 3) ? 8 : 4;
    int x, y, z = 0, j;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, j)) return; } else { if (!cell2(g, bx, by, x, y, j)) return; }
    const float beta = bsum[j];
    if (beta >= 1) { fb[j] = -1; return; }
    float px, py, pz = 0.f;
    float m[K];
    int base;
    float sum;
    if (DIM == 3) {
        trace3(u, v, w, solid, g, (float)x, (float)y, (float)z, +dt, 4, px, py, pz);
        sum = corner_weights3(solid, g, px, py, pz, base, m);
    } else {
        trace2(u, v, solid, g, (float)x, (float)y, +dt, 4, px, py);
        sum = corner_weights2(solid, g, px, py, base, m);
    }
    if (sum == 0) { fb[j] = -1; return; }
    fb[j] = base;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const float val = (1 - beta) * (m[k] / sum);
        wf[k * g.N + j] = val;
        atomicAdd(&gsum[base + (DIM == 3 ? corner_offset3(g, k) : corner_offset2(g, k))], val);
    }
}
template <int DIM>
__global__ void k_adv_forward(Geo g, const float* __restrict__ u, const float* __restrict__ v,
                              const float* __restrict__ w, const uint8_t* __restrict__ solid,
                              const float* __restrict__ bsum, float dt, float* __restrict__ wf, int* __restrict__ fb,
                              float* __restrict__ gsum) {
    d_adv_forward<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, u, v, w, solid, bsum, dt, wf, fb, gsum);
}

// Steps 6-8 for the backward rows: gamma2 = row sum, A /= gamma2, column sums beta2 (into beta).
template <int DIM>
__device__ __forceinline__ void d_adv_rows(const Geo& g, int bx, int by, int bz, float* __restrict__ wb, const int* __restrict__ bb, float* __restrict__ gsum, float* __restrict__ beta) {
    constexpr int K = (DIM == 3) ? 8 : 4;
    int x, y, z = 0, i;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, i)) return; } else { if (!cell2(g, bx, by, x, y, i)) return; }
    const int base = bb[i];
    float vals[K];
    float local = 0;
    if (base >= 0) {
#pragma unroll
        for (int k = 0; k < K; k++) { vals[k] = wb[k * g.N + i]; local += vals[k]; }
    }
    const float g2 = local + gsum[i];
    gsum[i] = g2;
    if (base < 0) return;
#pragma unroll
    for (int k = 0; k < K; k++) {
        float val = vals[k];
        if (g2 > 1.e-5f) val /= g2;
        wb[k * g.N + i] = val;
        atomicAdd(&beta[base + (DIM == 3 ? corner_offset3(g, k) : corner_offset2(g, k))], val);
    }
}
template <int DIM>
__global__ void k_adv_rows(Geo g, float* __restrict__ wb, const int* __restrict__ bb, float* __restrict__ gsum,
                           float* __restrict__ beta) {
    d_adv_rows<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, wb, bb, gsum, beta);
}

// Steps 7-8 for the forward entries: A /= gamma2 of their row, column sums into beta.
template <int DIM>
__device__ __forceinline__ void d_adv_cols(const Geo& g, int bx, int by, int bz, float* __restrict__ wf, const int* __restrict__ fb, const float* __restrict__ gsum, float* __restrict__ beta) {
    constexpr int K = (DIM == 3) ? 8 : 4;
    int x, y, z = 0, j;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, j)) return; } else { if (!cell2(g, bx, by, x, y, j)) return; }
    const int base = fb[j];
    if (base < 0) return;
    float local = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
        float val = wf[k * g.N + j];
        const float g2 = gsum[base + (DIM == 3 ? corner_offset3(g, k) : corner_offset2(g, k))];
        if (g2 > 1.e-5f) val /= g2;
        wf[k * g.N + j] = val;
        local += val;
    }
    atomicAdd(&beta[j], local);
}
template <int DIM>
__global__ void k_adv_cols(Geo g, float* __restrict__ wf, const int* __restrict__ fb, const float* __restrict__ gsum,
                           float* __restrict__ beta) {
    d_adv_cols<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, wf, fb, gsum, beta);
}

// Steps 9-11 for the backward rows, every cell: A /= beta2 of the column, gamma3 = row sum, rho' = A rho.
// Cells without a backward row (border, solids) get 0, which the forward pass then adds to.
template <int DIM>
__device__ __forceinline__ void d_adv_apply_rows(const Geo& g, int bx, int by, int bz, const float* __restrict__ wb, const int* __restrict__ bb, const float* __restrict__ beta, const float* __restrict__ rho, float* __restrict__ gamma_out, float* __restrict__ rho_out) {
    constexpr int K = (DIM == 3) ? 8 : 4;
    const int i = bx * blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    const int x = i % g.W, y = (i / g.W) % g.H, z = i / g.WH;
    bool interior = x >= 1 && x <= g.W - 2 && y >= 1 && y <= g.H - 2;
    if (DIM == 3) interior = interior && z >= 1 && z <= g.D - 2;
    float gs = 0, rs = 0;
    const int base = interior ? bb[i] : -1;
    if (base >= 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int c = base + (DIM == 3 ? corner_offset3(g, k) : corner_offset2(g, k));
            float val = wb[k * g.N + i];
            const float b2 = beta[c];
            if (b2 > 1.e-5f) val /= b2;
            gs += val;
            rs += val * rho[c];
        }
    }
    gamma_out[i] = gs;
    rho_out[i] = rs;
}
template <int DIM>
__global__ void k_adv_apply_rows(Geo g, const float* __restrict__ wb, const int* __restrict__ bb,
                                 const float* __restrict__ beta, const float* __restrict__ rho,
                                 float* __restrict__ gamma_out, float* __restrict__ rho_out) {
    d_adv_apply_rows<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, wb, bb, beta, rho, gamma_out, rho_out);
}

// Steps 9-11 for the forward entries: A /= beta2_j, scattered into gamma3 and rho'.
template <int DIM>
__device__ __forceinline__ void d_adv_apply_cols(const Geo& g, int bx, int by, int bz, const float* __restrict__ wf, const int* __restrict__ fb, const float* __restrict__ beta, const float* __restrict__ rho, float* __restrict__ gamma_out, float* __restrict__ rho_out) {
    constexpr int K = (DIM == 3) ? 8 : 4;
    int x, y, z = 0, j;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, j)) return; } else { if (!cell2(g, bx, by, x, y, j)) return; }
    const int base = fb[j];
    if (base < 0) return;
    const float b2 = beta[j];
    const float rj = rho[j];
#pragma unroll
    for (int k = 0; k < K; k++) {
        float val = wf[k * g.N + j];
        if (b2 > 1.e-5f) val /= b2;
        const int c = base + (DIM == 3 ? corner_offset3(g, k) : corner_offset2(g, k));
        atomicAdd(&gamma_out[c], val);
        atomicAdd(&rho_out[c], val * rj);
    }
}
template <int DIM>
__global__ void k_adv_apply_cols(Geo g, const float* __restrict__ wf, const int* __restrict__ fb,
                                 const float* __restrict__ beta, const float* __restrict__ rho,
                                 float* __restrict__ gamma_out, float* __restrict__ rho_out) {
    d_adv_apply_cols<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, wf, fb, beta, rho, gamma_out, rho_out);
}

// Step 12: one in-place sweep of pairwise gamma-equalising transfers along one axis
// (CPUSimulator3D.cpp:277-362).  One thread walks one line sequentially; `stride` is the axis stride,
// `n` the line length (cells), line start = `first`.  Only the carried pair (rho, gamma) of the previous cell
// depends on earlier steps: every cell is read from memory before this thread writes it, and lines are
// disjoint, so the loads of the next kPf cells are issued while the current kPf cells are processed.
constexpr int kPf = 16;
// One pairwise transfer between the carried cell j and the next cell i along the line.  The sweep is a
// sequential chain per line, so its speed is this function's latency: both directions share one division,
// formed from selected operands (the same operations in the same order as either branch), and the result is
// applied by selects, so no lane of a warp waits on another lane's branch.
__device__ __forceinline__ void diffuse_pair(float& rj, float& gj, bool sj, float& ri, float& gi, bool si) {
    const bool act = !(si || sj) && !(gj < 1e-5f || gi < 1e-5f) && !(gj == gi);
    const bool down = gj > gi;   // mass moves from j to i
    const float avg = (gj + gi) / 2.f;
    const float num = down ? rj * (gj - gi) : ri * (gi - gj);
    const float den = 2.f * (down ? gj : gi);
    const float dif = num / den;
    const float rjn = down ? rj - dif : rj + dif;
    const float rin = down ? ri + dif : ri - dif;
    rj = act ? rjn : rj;
    ri = act ? rin : ri;
    gj = act ? avg : gj;
    gi = act ? avg : gi;
}
struct LineBlock {
    float r[kPf], g[kPf];
    unsigned solid;   // bit k: cell k of the block is solid
};
__device__ __forceinline__ void load_block(LineBlock& b, const float* __restrict__ rsrc, const float* __restrict__ gsrc,
                                           const uint8_t* __restrict__ solid, int first, int stride, int c0, int last) {
    b.solid = 0;
#pragma unroll
    for (int k = 0; k < kPf; k++) {
        if (c0 + k <= last) {
            const int i = first + stride * (c0 + k);
            b.r[k] = rsrc[i];
            b.g[k] = gsrc[i];
            b.solid |= (unsigned)(solid[i] != 0) << k;
        }
    }
}
__device__ __forceinline__ void diffuse_line(const float* __restrict__ rsrc, const float* __restrict__ gsrc,
                                             float* __restrict__ rdst, float* __restrict__ gdst,
                                             const uint8_t* __restrict__ solid, int first, int stride, int n) {
    // cells first + stride * c for c = 1 .. n-2; pairs (c-1, c) for c = 2 .. n-2
    const int last = n - 2;
    int jj = first + stride;
    float rj = rsrc[jj], gj = gsrc[jj];
    bool sj = solid[jj] != 0;
    LineBlock cur, nxt;
    load_block(cur, rsrc, gsrc, solid, first, stride, 2, last);
    for (int c0 = 2; c0 <= last; c0 += kPf) {
        load_block(nxt, rsrc, gsrc, solid, first, stride, c0 + kPf, last);
#pragma unroll
        for (int k = 0; k < kPf; k++) {
            if (c0 + k > last) break;
            const int ii = jj + stride;
            float ri = cur.r[k], gi = cur.g[k];
            const bool si = (cur.solid >> k) & 1u;
            diffuse_pair(rj, gj, sj, ri, gi, si);
            rdst[jj] = rj; gdst[jj] = gj;
            jj = ii; rj = ri; gj = gi; sj = si;
        }
        cur = nxt;
    }
    if (n >= 3) { rdst[jj] = rj; gdst[jj] = gj; }
}

// X sweep: one thread per (y, z) line.
__device__ __forceinline__ void d_diffuse_x(const Geo& g, int bx, int by, int bz, int dim, const float* rsrc, const float* gsrc, float* rdst, float* gdst, const uint8_t* __restrict__ solid) {
    const int y = 1 + bx * blockDim.x + threadIdx.x;
    const int z = (dim == 3) ? 1 + by : 0;
    if (y > g.H - 2) return;
    diffuse_line(rsrc, gsrc, rdst, gdst, solid, z * g.WH + y * g.W, 1, g.W);
}
// All of step 12 for a 2D grid small enough for one SM's shared memory (rho, gamma and the solid bytes of the
// whole grid, rows padded to W + 1 so that neither a row walk nor a column walk has bank conflicts): one block
// loads the grid (rho from rho_acc on the interior, folding step 11's copy), runs the `iters` x and y sweeps
// with a block barrier between sweeps, and writes the interior back.  A 2D grid has only H - 2 (W - 2) lines
// a sweep, each a sequential chain, so a sweep is bound by the chain's latency: from shared memory that is a
// few cycles a load instead of an L2 round trip per step, and 14 launches become one.  Same order and
// arithmetic as diffuse_line; only interior cells are read or written, as there.
constexpr int kD2Threads = 256;
__global__ void __launch_bounds__(kD2Threads) k_diffuse_2d_smem(Geo g, const float* __restrict__ rho_acc, float* rho,
                                                                 float* gamma, const uint8_t* __restrict__ solid,
                                                                 int iters) {
    extern __shared__ float sm[];
    const int W = g.W, H = g.H, P = W + 1;
    float* sr = sm;
    float* sg = sm + (size_t)H * P;
    uint8_t* ss = reinterpret_cast<uint8_t*>(sg + (size_t)H * P);
    for (int k = threadIdx.x; k < W * H; k += blockDim.x) {
        const int y = k / W, x = k - y * W;
        const bool in = x >= 1 && x <= W - 2 && y >= 1 && y <= H - 2;
        sr[y * P + x] = in ? rho_acc[k] : rho[k];
        sg[y * P + x] = gamma[k];
        ss[y * P + x] = solid[k];
    }
    __syncthreads();
    for (int it = 0; it < iters; it++) {
        for (int axis = 0; axis < 2; axis++) {
            // axis 0: x sweep, line y = 1 + t (stride 1, n = W); axis 1: y sweep, line x = 1 + t (stride P, n = H)
            const int lines = axis == 0 ? H - 2 : W - 2;
            const int n = axis == 0 ? W : H;
            const int stride = axis == 0 ? 1 : P;
            for (int t = threadIdx.x; t < lines; t += blockDim.x) {
                const int first = axis == 0 ? (1 + t) * P : 1 + t;
                int jj = first + stride;
                float rj = sr[jj], gj = sg[jj];
                bool sj = ss[jj] != 0;
                for (int c = 2; c <= n - 2; c++) {
                    const int ii = jj + stride;
                    float ri = sr[ii], gi = sg[ii];
                    const bool si = ss[ii] != 0;
                    diffuse_pair(rj, gj, sj, ri, gi, si);
                    sr[jj] = rj; sg[jj] = gj;
                    jj = ii; rj = ri; gj = gi; sj = si;
                }
                if (n >= 3) { sr[jj] = rj; sg[jj] = gj; }
            }
            __syncthreads();
        }
    }
    for (int k = threadIdx.x; k < W * H; k += blockDim.x) {
        const int y = k / W, x = k - y * W;
        if (x >= 1 && x <= W - 2 && y >= 1 && y <= H - 2) { rho[k] = sr[y * P + x]; gamma[k] = sg[y * P + x]; }
    }
}
// Shared memory of k_diffuse_2d_smem for a W x H grid, and the largest it takes.
inline size_t diffuse_2d_smem_bytes(const Geo& g) { return (size_t)g.H * (g.W + 1) * (2 * sizeof(float) + 1); }
constexpr size_t kD2MaxSmem = 200 * 1024;

// X sweep of a 2D grid: one thread per line.  A 2D grid has too few lines (H - 2) for the tiled kernel below,
// whose load and store phases then stand between the sequential steps of one block's lines (measured at 128^2:
// 92 against 45 us per sweep); its few lines stay in L1.
__global__ void k_diffuse_x_lines(Geo g, int dim, const float* rsrc, const float* gsrc, float* rdst, float* gdst,
                                  const uint8_t* __restrict__ solid) {
    d_diffuse_x(g, blockIdx.x, blockIdx.y, blockIdx.z, dim, rsrc, gsrc, rdst, gdst, solid);
}

// X sweep of a single grid through shared memory.  Along x a thread's line is contiguous, so one thread per
// line reads 32 different lines per warp instruction.  Here a warp owns 32 lines (consecutive y, one plane)
// and walks them in 32-cell tiles: each tile comes in row by row (one 128-byte row per instruction) into a
// padded shared tile, lane l runs the sequential transfers of line l out of shared memory, and the tile goes
// back row by row.  Cell x0 - 1, which becomes final at the first pair of a tile after its own tile was
// stored, and the last cell of the line are written by the lane directly.  Same arithmetic and order as
// diffuse_line.
constexpr int kDxWarps = 4;
__global__ void __launch_bounds__(kDxWarps * 32) k_diffuse_x(Geo g, int dim, const float* rsrc, const float* gsrc,
                                                               float* rdst, float* gdst, const uint8_t* __restrict__ solid) {
    __shared__ float s_r[kDxWarps][32][33], s_g[kDxWarps][32][33];
    __shared__ unsigned s_m[kDxWarps][32];   // per line: bit p = cell x0 + p is solid
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y0 = 1 + (blockIdx.x * kDxWarps + warp) * 32;
    const int z = (dim == 3) ? 1 + blockIdx.y : 0;
    const int nlines = min(32, g.H - 1 - y0);   // lines y0 .. y0 + nlines - 1 (y <= H - 2)
    if (nlines <= 0) return;                    // warp-uniform
    const int n = g.W;
    const size_t plane = (size_t)z * g.WH;
    float (*tr)[33] = s_r[warp];
    float (*tg)[33] = s_g[warp];
    unsigned* tm = s_m[warp];
    const size_t mine = plane + (size_t)(y0 + lane) * n;   // start of lane's own line (valid for lane < nlines)
    float rj = 0.f, gj = 0.f;
    bool sj = false;
    for (int x0 = 0; x0 <= n - 2; x0 += 32) {
        const int x = x0 + lane;
        for (int j = 0; j < nlines; j++) {
            const size_t i = plane + (size_t)(y0 + j) * n + x;
            bool sol = false;
            if (x <= n - 2) {
                tr[j][lane] = rsrc[i];
                tg[j][lane] = gsrc[i];
                sol = solid[i] != 0;
            }
            const unsigned m = __ballot_sync(0xffffffffu, sol);
            if (lane == 0) tm[j] = m;
        }
        __syncwarp();
        if (lane < nlines) {
            const unsigned m = tm[lane];
            int p = 0;
            if (x0 == 0) { rj = tr[lane][1]; gj = tg[lane][1]; sj = (m >> 1) & 1u; p = 2; }
            const int pend = min(31, n - 2 - x0);   // last cell of this tile that is processed
            for (; p <= pend; p++) {
                float ri = tr[lane][p], gi = tg[lane][p];
                const bool si = (m >> p) & 1u;
                diffuse_pair(rj, gj, sj, ri, gi, si);
                if (p == 0) { rdst[mine + x0 - 1] = rj; gdst[mine + x0 - 1] = gj; }
                else { tr[lane][p - 1] = rj; tg[lane][p - 1] = gj; }
                rj = ri; gj = gi; sj = si;
            }
            if (x0 + 31 >= n - 2 && n >= 3) { rdst[mine + n - 2] = rj; gdst[mine + n - 2] = gj; }
        }
        __syncwarp();
        // cells finalised in this tile: x in [max(1, x0), min(n - 3, x0 + 30)]
        if (lane <= 30 && x >= 1 && x <= n - 3) {
            for (int j = 0; j < nlines; j++) {
                const size_t i = plane + (size_t)(y0 + j) * n + x;
                rdst[i] = tr[j][lane];
                gdst[i] = tg[j][lane];
            }
        }
        __syncwarp();
    }
}
// Y sweep: one thread per (x, z) line (consecutive threads = consecutive x: coalesced).
__device__ __forceinline__ void d_diffuse_y(const Geo& g, int bx, int by, int bz, int dim, float* rho, float* gamma, const uint8_t* __restrict__ solid) {
    const int x = 1 + bx * blockDim.x + threadIdx.x;
    const int z = (dim == 3) ? 1 + by : 0;
    if (x > g.W - 2) return;
    diffuse_line(rho, gamma, rho, gamma, solid, z * g.WH + x, g.W, g.H);
}
__global__ void k_diffuse_y(Geo g, int dim, float* rho, float* gamma, const uint8_t* __restrict__ solid) {
    d_diffuse_y(g, blockIdx.x, blockIdx.y, blockIdx.z, dim, rho, gamma, solid);
}
// Z sweep: one thread per (x, y) line.
__global__ void k_diffuse_z(Geo g, float* rho, float* gamma, const uint8_t* __restrict__ solid) {
    const int x = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int y = 1 + blockIdx.y;
    if (x > g.W - 2) return;
    diffuse_line(rho, gamma, rho, gamma, solid, y * g.W + x, g.WH, g.D);
}

// ------------------------------------------------------------------------------------------------
// stage 4: vel_advect (CPUSimulator3D.cpp:478-504, CPUSimulator2D.cpp:427-448), optionally followed by
// stage 5 add_force in the same pass.
// ------------------------------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void d_vadv_trace(const Geo& g, int bx, int by, int bz, const float* __restrict__ u, const float* __restrict__ v, const float* __restrict__ w, const uint8_t* __restrict__ solid, float dt, float* __restrict__ tu, float* __restrict__ tv, float* __restrict__ tw) {
    int x, y, z = 0, i;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, i)) return; } else { if (!cell2(g, bx, by, x, y, i)) return; }
    if (DIM == 3) {
        float px, py, pz, a, b, c;
        trace3(u, v, w, solid, g, (float)x, (float)y, (float)z, -dt, 4, px, py, pz);
        vinterp3(u, v, w, g, px - 0.5f, py - 0.5f, pz - 0.5f, a, b, c);
        tu[i] = a; tv[i] = b; tw[i] = c;
    } else {
        float px, py, a, b;
        trace2(u, v, solid, g, (float)x, (float)y, -dt, 4, px, py);
        vinterp2(u, v, g, px - 0.5f, py - 0.5f, a, b);
        tu[i] = a; tv[i] = b;
    }
}
template <int DIM>
__global__ void k_vadv_trace(Geo g, const float* __restrict__ u, const float* __restrict__ v,
                             const float* __restrict__ w, const uint8_t* __restrict__ solid, float dt,
                             float* __restrict__ tu, float* __restrict__ tv, float* __restrict__ tw) {
    d_vadv_trace<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, u, v, w, solid, dt, tu, tv, tw);
}

// vel_advect's sample at a trace end kept by rho_advect (k_adv_backward's `tend`, in tu/tv/tw, read and
// overwritten per cell).
template <int DIM>
__global__ void k_vadv_sample(Geo g, const float* __restrict__ u, const float* __restrict__ v,
                              const float* __restrict__ w, float* tu, float* tv, float* tw) {
    int x, y, z = 0, i;
    if (DIM == 3) { if (!cell3(g, blockIdx.x, blockIdx.y, blockIdx.z, x, y, z, i)) return; }
    else { if (!cell2(g, blockIdx.x, blockIdx.y, x, y, i)) return; }
    if (DIM == 3) {
        const float px = tu[i], py = tv[i], pz = tw[i];
        float a, b, c;
        vinterp3(u, v, w, g, px - 0.5f, py - 0.5f, pz - 0.5f, a, b, c);
        tu[i] = a; tv[i] = b; tw[i] = c;
    } else {
        const float px = tu[i], py = tv[i];
        float a, b;
        vinterp2(u, v, g, px - 0.5f, py - 0.5f, a, b);
        tu[i] = a; tv[i] = b;
    }
}

struct ForceArgs {
    int enabled;          // fuse add_force after the averaging
    int has_forces;       // forces field is not all zero
    int gravity;
    float dt, gforce;
    const float *fx, *fy, *fz;
};

// 3D add_force on one cell (CPUSimulator3D.cpp:458-476)
__device__ __forceinline__ void add_force_cell3(const ForceArgs& f, int i, bool solid_i, float& a, float& b, float& c) {
    if (solid_i) return;
    if (f.has_forces) { a += f.fx[i] * f.dt; b += f.fy[i] * f.dt; c += f.fz[i] * f.dt; }
    if (f.gravity) b -= f.gforce * f.dt;
}
// 2D add_force on one cell, face based (CPUSimulator2D.cpp:404-425)
__device__ __forceinline__ void add_force_cell2(const ForceArgs& f, int i, bool s_i, bool s_xm, bool s_ym, float& a,
                                                float& b) {
    if (!s_i || !s_xm) a += f.fx[i] * f.dt; else a = 0.f;
    if (!s_i || !s_ym) {
        b += f.fy[i] * f.dt;
        if (f.gravity) b -= f.gforce * f.dt;
    } else b = 0.f;
}

template <int DIM>
__device__ __forceinline__ void d_vadv_average(const Geo& g, int bx, int by, int bz, const float* __restrict__ tu, const float* __restrict__ tv, const float* __restrict__ tw, const uint8_t* __restrict__ solid, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, ForceArgs f) {
    int x, y, z = 0, i;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, i)) return; } else { if (!cell2(g, bx, by, x, y, i)) return; }
    const bool si = solid[i], sx = solid[i - 1], sy = solid[i - g.W];
    float a = (x == 1 || si || sx) ? tu[i] : 0.5f * (tu[i] + tu[i - 1]);
    float b = (y == 1 || si || sy) ? tv[i] : 0.5f * (tv[i] + tv[i - g.W]);
    if (DIM == 3) {
        const bool sz = solid[i - g.WH];
        float c = (z == 1 || si || sz) ? tw[i] : 0.5f * (tw[i] + tw[i - g.WH]);
        if (f.enabled) add_force_cell3(f, i, si, a, b, c);
        w[i] = c;
    } else {
        if (f.enabled) add_force_cell2(f, i, si, sx, sy, a, b);
    }
    u[i] = a; v[i] = b;
}
template <int DIM>
__global__ void k_vadv_average(Geo g, const float* __restrict__ tu, const float* __restrict__ tv,
                               const float* __restrict__ tw, const uint8_t* __restrict__ solid, float* __restrict__ u,
                               float* __restrict__ v, float* __restrict__ w, ForceArgs f) {
    d_vadv_average<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, tu, tv, tw, solid, u, v, w, f);
}

template <int DIM>
__device__ __forceinline__ void d_add_force(const Geo& g, int bx, int by, int bz, const uint8_t* __restrict__ solid, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, ForceArgs f) {
    int x, y, z = 0, i;
    if (DIM == 3) { if (!cell3(g, bx, by, bz, x, y, z, i)) return; } else { if (!cell2(g, bx, by, x, y, i)) return; }
    float a = u[i], b = v[i];
    if (DIM == 3) {
        float c = w[i];
        add_force_cell3(f, i, solid[i] != 0, a, b, c);
        w[i] = c;
    } else {
        add_force_cell2(f, i, solid[i] != 0, solid[i - 1] != 0, solid[i - g.W] != 0, a, b);
    }
    u[i] = a; v[i] = b;
}
template <int DIM>
__global__ void k_add_force(Geo g, const uint8_t* __restrict__ solid, float* __restrict__ u, float* __restrict__ v,
                            float* __restrict__ w, ForceArgs f) {
    d_add_force<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, solid, u, v, w, f);
}

// ------------------------------------------------------------------------------------------------
// stage 6: project (CPUSimulator3D.cpp:506-566 with enforce_wall_boundaries :657-679;
// CPUSimulator2D.cpp:450-524, :597-607)
// ------------------------------------------------------------------------------------------------

// wall rule of one face (3D: sign dependent; 2D: zero when either side is solid)
template <int DIM>
__device__ __forceinline__ float wall_face(float val, bool solid_here, bool solid_below) {
    if (DIM == 3) {
        if (solid_here && val > 0) val = 0.f;
        if (solid_below && val < 0) val = 0.f;
        return val;
    } else {
        return (solid_here || solid_below) ? 0.f : val;
    }
}

struct ProjectArgs {
    float thrL, lp, lm, eta;
    int jacobi;          // p starts at 0 (Jacobi) or at b (CG)
};

// Walls on every face, divergence with the density correction, initial pressure, matrix-row description and
// active-chunk flags.  One thread per cell, 1D over the linear index (a warp is one aligned 32-cell chunk).
template <int DIM>
__device__ __forceinline__ void d_project_pre(const Geo& g, int bx, int by, int bz, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, const float* __restrict__ rho, const uint8_t* __restrict__ solid, float* __restrict__ div, float* __restrict__ p, uint16_t* __restrict__ rowinfo, uint8_t* __restrict__ chunk_flag, ProjectArgs a) {
    const int i = bx * blockDim.x + threadIdx.x;
    const bool in = i < g.N;
    bool active = false;
    if (in) {
        const int x = i % g.W, y = (i / g.W) % g.H, z = (DIM == 3) ? i / g.WH : 0;
        const bool si = solid[i];
        // enforce_wall_boundaries on this cell's faces
        float fu = u[i], fv = v[i], fw = 0.f;
        if (DIM == 3) {
            if (x >= 1 && y >= 1 && z >= 1) {
                fu = wall_face<3>(fu, si, solid[i - 1]);
                fv = wall_face<3>(fv, si, solid[i - g.W]);
                fw = wall_face<3>(w[i], si, solid[i - g.WH]);
                u[i] = fu; v[i] = fv; w[i] = fw;
            }
        } else {
            fu = wall_face<2>(fu, si, x > 0 && solid[i - (x > 0 ? 1 : 0)]);
            fv = wall_face<2>(fv, si, y > 0 && solid[i - (y > 0 ? g.W : 0)]);
            u[i] = fu; v[i] = fv;
        }
        bool interior = x >= 1 && x <= g.W - 2 && y >= 1 && y <= g.H - 2;
        if (DIM == 3) interior = interior && z >= 1 && z <= g.D - 2;
        float d = 0.f;
        const float r = rho[i];
        if (interior && !(r < a.thrL) && !si) {
            const float up = wall_face<DIM>(u[i + 1], solid[i + 1], si);
            const float vp = wall_face<DIM>(v[i + g.W], solid[i + g.W], si);
            const float dx = up - fu, dy = vp - fv;
            if (DIM == 3) {
                const float wp = wall_face<3>(w[i + g.WH], solid[i + g.WH], si);
                d = dx + dy + (wp - fw);
            } else {
                d = dx + dy;
            }
            if (r > 1.f) d -= minf(a.lm * (r - 1.f), a.eta);
            if (r < 1.f) d += minf(a.lp * (1.f - r), a.eta);
        }
        div[i] = d;
        p[i] = a.jacobi ? 0.f : d;
        // matrix row (CGSolver.cpp:467-497): rho > 0.5 and not solid; neighbours counted when inside, off the
        // border and not solid; summed when also rho > 0.5.  Bits: x-1, x+1, y-1, y+1, z-1, z+1.
        uint16_t info = 0;
        if (r > 0.5f && !si) {
            const int nx[6] = {x - 1, x + 1, x, x, x, x}, ny[6] = {y, y, y - 1, y + 1, y, y};
            const int nz[6] = {z, z, z, z, z - 1, z + 1};
            const int off[6] = {-1, 1, -g.W, g.W, -g.WH, g.WH};
            int cnt = 0;
#pragma unroll
            for (int k = 0; k < 2 * DIM; k++) {
                if (nx[k] <= 0 || nx[k] >= g.W - 1 || ny[k] <= 0 || ny[k] >= g.H - 1) continue;
                if (DIM == 3 && (nz[k] <= 0 || nz[k] >= g.D - 1)) continue;
                const int j = i + off[k];
                if (solid[j]) continue;
                cnt++;
                if (rho[j] > 0.5f) info |= (uint16_t)(1u << k);
            }
            info |= (uint16_t)(cnt << 8) | (uint16_t)0x8000u;
        }
        rowinfo[i] = info;
        active = (info & 0x8000u) || d != 0.f;
    }
    const unsigned any = __ballot_sync(0xffffffffu, active);
    if ((threadIdx.x & 31) == 0 && (i >> 5) < ((g.N + 31) >> 5)) chunk_flag[i >> 5] = any ? 1 : 0;
}
template <int DIM>
__global__ void k_project_pre(Geo g, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                              const float* __restrict__ rho, const uint8_t* __restrict__ solid,
                              float* __restrict__ div, float* __restrict__ p, uint16_t* __restrict__ rowinfo,
                              uint8_t* __restrict__ chunk_flag, ProjectArgs a) {
    d_project_pre<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, u, v, w, rho, solid, div, p, rowinfo, chunk_flag, a);
}

// v -= grad p on non-solid interior cells, then walls on every face; skipped (with PAUSED set) when the solve
// did not converge (CPUSimulator3D.cpp:541-566).
template <int DIM>
__device__ __forceinline__ void d_project_post(const Geo& g, int bx, int by, int bz, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w, const float* __restrict__ p, const uint8_t* __restrict__ solid, DevCtl* ctl, int do_walls) {
    if (!ctl->converged) {
        if (bx == 0 && by == 0 && bz == 0 && threadIdx.x == 0 && threadIdx.y == 0) ctl->paused = 1;
        return;
    }
    const int x = 1 + bx * blockDim.x + threadIdx.x;
    const int y = 1 + by * blockDim.y + threadIdx.y;
    const int z = (DIM == 3) ? 1 + bz : 0;
    if (x > g.W - 1 || y > g.H - 1) return;
    const int i = z * g.WH + y * g.W + x;
    const bool si = solid[i];
    const bool interior = x <= g.W - 2 && y <= g.H - 2 && (DIM == 2 || z <= g.D - 2);
    float fu = u[i], fv = v[i], fw = (DIM == 3) ? w[i] : 0.f;
    if (interior) {
        if (DIM == 3) {
            if (!si) {
                float gx = 0, gy = 0, gz = 0;
                if (x > 1) gx = p[i] - p[i - 1];
                if (y > 1) gy = p[i] - p[i - g.W];
                if (z > 1) gz = p[i] - p[i - g.WH];
                fu -= gx; fv -= gy; fw -= gz;
            }
        } else {
            if (!si && !solid[i - 1]) fu -= (p[i] - p[i - 1]); else fu = 0.f;
            if (!si && !solid[i - g.W]) fv -= (p[i] - p[i - g.W]); else fv = 0.f;
        }
    }
    if (do_walls) {
        fu = wall_face<DIM>(fu, si, solid[i - 1]);
        fv = wall_face<DIM>(fv, si, solid[i - g.W]);
        if (DIM == 3) fw = wall_face<3>(fw, si, solid[i - g.WH]);
    }
    u[i] = fu; v[i] = fv;
    if (DIM == 3) w[i] = fw;
}
template <int DIM>
__global__ void k_project_post(Geo g, float* __restrict__ u, float* __restrict__ v, float* __restrict__ w,
                               const float* __restrict__ p, const uint8_t* __restrict__ solid, DevCtl* ctl,
                               int do_walls) {
    d_project_post<DIM>(g, blockIdx.x, blockIdx.y, blockIdx.z, u, v, w, p, solid, ctl, do_walls);
}

// ISolver::solve on the current divergence: matrix-row description, active-chunk flags and the solver's
// initial pressure (CG: p = b, CGSolver.cpp:429; Jacobi: the current p, JacobiSolver.cpp:159).
template <int DIM>
__global__ void k_solver_prep(Geo g, const float* __restrict__ rho, const uint8_t* __restrict__ solid,
                              const float* __restrict__ div, float* __restrict__ p, uint16_t* __restrict__ rowinfo,
                              uint8_t* __restrict__ chunk_flag, int jacobi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool active = false;
    if (i < g.N) {
        const int x = i % g.W, y = (i / g.W) % g.H, z = (DIM == 3) ? i / g.WH : 0;
        const float d = div[i];
        if (!jacobi) p[i] = d;
        uint16_t info = 0;
        if (rho[i] > 0.5f && !solid[i]) {
            const int nx[6] = {x - 1, x + 1, x, x, x, x}, ny[6] = {y, y, y - 1, y + 1, y, y};
            const int nz[6] = {z, z, z, z, z - 1, z + 1};
            const int off[6] = {-1, 1, -g.W, g.W, -g.WH, g.WH};
            int cnt = 0;
#pragma unroll
            for (int k = 0; k < 2 * DIM; k++) {
                if (nx[k] <= 0 || nx[k] >= g.W - 1 || ny[k] <= 0 || ny[k] >= g.H - 1) continue;
                if (DIM == 3 && (nz[k] <= 0 || nz[k] >= g.D - 1)) continue;
                const int j = i + off[k];
                if (solid[j]) continue;
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

// 2D RE_CALC_DIV (CPUSimulator2D.cpp:503-521) and the closing walls when it is on.
__global__ void k_recalc_div2(Geo g, const float* __restrict__ u, const float* __restrict__ v,
                              const float* __restrict__ rho, const uint8_t* __restrict__ solid, float* __restrict__ div,
                              ProjectArgs a, const DevCtl* ctl) {
    if (!ctl->converged) return;
    int x, y, i;
    if (!cell2(g, blockIdx.x, blockIdx.y, x, y, i)) return;
    const float r = rho[i];
    if (r < a.thrL || solid[i]) return;
    float d = (u[i + 1] - u[i]) + (v[i + g.W] - v[i]);
    if (r > 1.f) d -= minf(a.lm * (r - 1.f), a.eta);
    if (r < 1.f) d += minf(a.lp * (1.f - r), a.eta);
    div[i] = d;
}
__global__ void k_walls2(Geo g, float* __restrict__ u, float* __restrict__ v, const uint8_t* __restrict__ solid,
                         const DevCtl* ctl) {
    if (!ctl->converged) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.N) return;
    const int x = i % g.W, y = i / g.W;
    const bool si = solid[i];
    if (si || (x > 0 && solid[i - 1])) u[i] = 0.f;
    if (si || (y > 0 && solid[i - g.W])) v[i] = 0.f;
}

inline dim3 grid_interior(const Geo& g, int dim) {
    return dim3((g.W - 2 + BX - 1) / BX, (g.H - 2 + BY - 1) / BY, dim == 3 ? g.D - 2 : 1);
}
inline dim3 grid_linear(int n, int threads) { return dim3((n + threads - 1) / threads); }

}  // namespace

#define EFS_LAUNCH_CHECK() do { cudaError_t e_ = cudaGetLastError(); if (e_ != cudaSuccess) return e_; } while (0)

static cudaError_t stage_decay(efs_ctx* c) {
    const dim3 b(BX, BY), gr = grid_interior(c->g, c->dim);
    if (c->dim == 3) k_vel_decay<3><<<gr, b, 0, c->stream>>>(c->g, c->u, c->v, c->w, c->rho, c->prm.vel_decay);
    else k_vel_decay<2><<<gr, b, 0, c->stream>>>(c->g, c->u, c->v, c->w, c->rho, c->prm.vel_decay);
    EFS_LAUNCH_CHECK();
    return cudaSuccess;
}

static cudaError_t stage_extrapolate(efs_ctx* c) {
    const Geo& g = c->g;
    float* tu = c->tvel; float* tv = c->tvel + g.N; float* tw = c->tvel + 2 * (size_t)g.N;
    k_extrap_init<<<grid_linear(g.N, 256), 256, 0, c->stream>>>(g, c->dim, c->rho, c->solid, c->validA);
    EFS_LAUNCH_CHECK();
    const dim3 b(BX, BY), gr = grid_interior(g, c->dim);
    for (int it = 0; it < 6; it++) {
        const bool odd = it & 1;
        const float* su = odd ? tu : c->u; const float* sv = odd ? tv : c->v; const float* sw = odd ? tw : c->w;
        float* du = odd ? c->u : tu; float* dv = odd ? c->v : tv; float* dw = odd ? c->w : tw;
        const uint8_t* sV = odd ? c->validB : c->validA;
        uint8_t* dV = odd ? c->validA : c->validB;
        if (c->dim == 3) k_extrap_pass<3><<<gr, b, 0, c->stream>>>(g, su, sv, sw, sV, du, dv, dw, dV, c->solid, it >= 1);
        else k_extrap_pass<2><<<gr, b, 0, c->stream>>>(g, su, sv, sw, sV, du, dv, dw, dV, c->solid, it >= 1);
        EFS_LAUNCH_CHECK();
    }
    return cudaSuccess;
}

static cudaError_t stage_sharpen(efs_ctx* c) {
    const Geo& g = c->g;
    cudaError_t e = cudaMemsetAsync(&c->ctl->sh_count, 0, sizeof(int), c->stream);
    if (e != cudaSuccess) return e;
    const dim3 b(BX, BY), gr = grid_interior(g, c->dim);
    const float delT = c->prm.dt * 3;
    const int cap = g.N;
    const int lg = c->sm_count * 4;
    if (c->dim == 3) k_sharpen_calc<3><<<gr, b, 0, c->stream>>>(g, c->rho, delT, c->sh_idx, c->sh_val, c->ctl, cap);
    else k_sharpen_calc<2><<<gr, b, 0, c->stream>>>(g, c->rho, delT, c->sh_idx, c->sh_val, c->ctl, cap);
    EFS_LAUNCH_CHECK();
    if (c->prm.sharpen_mode == EFS_SHARPEN_SEQUENTIAL) {
        // bsum is rho_advect's column-sum scratch, cleared by rho_advect before its first use
        if ((e = cudaMemsetAsync(c->bsum, 0, (size_t)g.N * sizeof(float), c->stream)) != cudaSuccess) return e;
        k_sharpen_densify<<<lg, 256, 0, c->stream>>>(c->bsum, c->sh_idx, c->sh_val, c->ctl, cap);
        EFS_LAUNCH_CHECK();
        if (c->dim == 3) k_sharpen_sequential<3><<<1, kSeqThreads, 0, c->stream>>>(g, c->rho, c->solid, c->bsum, c->prm.rho_d);
        else k_sharpen_sequential<2><<<1, kSeqThreads, 0, c->stream>>>(g, c->rho, c->solid, c->bsum, c->prm.rho_d);
        EFS_LAUNCH_CHECK();
        return cudaSuccess;
    }
    k_sharpen_apply<<<lg, 256, 0, c->stream>>>(c->rho, c->sh_idx, c->sh_val, c->ctl, cap);
    EFS_LAUNCH_CHECK();
    if (c->dim == 3) {
        k_sharpen_trace<3><<<lg, 256, 0, c->stream>>>(g, c->rho, c->solid, c->sh_idx, c->sh_end, c->prm.rho_d, c->ctl, cap);
        EFS_LAUNCH_CHECK();
        k_sharpen_scatter<3><<<lg, 256, 0, c->stream>>>(g, c->rho, c->solid, c->sh_val, c->sh_end, c->ctl, cap);
    } else {
        k_sharpen_trace<2><<<lg, 256, 0, c->stream>>>(g, c->rho, c->solid, c->sh_idx, c->sh_end, c->prm.rho_d, c->ctl, cap);
        EFS_LAUNCH_CHECK();
        k_sharpen_scatter<2><<<lg, 256, 0, c->stream>>>(g, c->rho, c->solid, c->sh_val, c->sh_end, c->ctl, cap);
    }
    EFS_LAUNCH_CHECK();
    return cudaSuccess;
}

template <int DIM>
static cudaError_t stage_advect_t(efs_ctx* c, bool keep_trace = false) {
    const Geo& g = c->g;
    const size_t bytes = (size_t)g.N * sizeof(float);
    const dim3 b(BX, BY), gr = grid_interior(g, DIM);
    cudaError_t e;
    if ((e = cudaMemsetAsync(c->bsum, 0, bytes, c->stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(c->gsum, 0, bytes, c->stream)) != cudaSuccess) return e;
    k_adv_backward<DIM><<<gr, b, 0, c->stream>>>(g, c->u, c->v, c->w, c->solid, c->gamma, c->prm.dt, c->wb, c->bb, c->bsum,
                                                  keep_trace ? c->tvel : nullptr);
    EFS_LAUNCH_CHECK();
    k_adv_forward<DIM><<<gr, b, 0, c->stream>>>(g, c->u, c->v, c->w, c->solid, c->bsum, c->prm.dt, c->wf, c->fb, c->gsum);
    EFS_LAUNCH_CHECK();
    if ((e = cudaMemsetAsync(c->beta, 0, bytes, c->stream)) != cudaSuccess) return e;
    k_adv_rows<DIM><<<gr, b, 0, c->stream>>>(g, c->wb, c->bb, c->gsum, c->beta);
    EFS_LAUNCH_CHECK();
    k_adv_cols<DIM><<<gr, b, 0, c->stream>>>(g, c->wf, c->fb, c->gsum, c->beta);
    EFS_LAUNCH_CHECK();
    k_adv_apply_rows<DIM><<<grid_linear(g.N, 256), 256, 0, c->stream>>>(g, c->wb, c->bb, c->beta, c->rho, c->gamma, c->rho_acc);
    EFS_LAUNCH_CHECK();
    k_adv_apply_cols<DIM><<<gr, b, 0, c->stream>>>(g, c->wf, c->fb, c->beta, c->rho, c->gamma, c->rho_acc);
    EFS_LAUNCH_CHECK();
    // step 11's copy of rho' into the interior is folded into the first x sweep (it reads rho_acc and writes
    // rho); step 12's sweeps follow
    const int iters = (DIM == 3) ? 3 : 7;
    if (DIM == 2 && diffuse_2d_smem_bytes(g) <= kD2MaxSmem) {
        static std::once_flag attr_once;
        static cudaError_t attr_err = cudaSuccess;
        std::call_once(attr_once, [] {
            attr_err = cudaFuncSetAttribute(k_diffuse_2d_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kD2MaxSmem);
        });
        if (attr_err != cudaSuccess) return attr_err;
        k_diffuse_2d_smem<<<1, kD2Threads, diffuse_2d_smem_bytes(g), c->stream>>>(g, c->rho_acc, c->rho, c->gamma, c->solid,
                                                                                 iters);
        EFS_LAUNCH_CHECK();
        return cudaSuccess;
    }
    for (int it = 0; it < iters; it++) {
        const float* rs = (it == 0) ? c->rho_acc : c->rho;
        if (DIM == 3) {
            k_diffuse_x<<<dim3((g.H - 2 + kDxWarps * 32 - 1) / (kDxWarps * 32), g.D - 2), kDxWarps * 32, 0, c->stream>>>(
                g, DIM, rs, c->gamma, c->rho, c->gamma, c->solid);
        } else {
            k_diffuse_x_lines<<<dim3((g.H - 2 + 127) / 128, 1), 128, 0, c->stream>>>(g, DIM, rs, c->gamma, c->rho, c->gamma,
                                                                                     c->solid);
        }
        EFS_LAUNCH_CHECK();
        k_diffuse_y<<<dim3((g.W - 2 + 127) / 128, DIM == 3 ? g.D - 2 : 1), 128, 0, c->stream>>>(g, DIM, c->rho, c->gamma, c->solid);
        EFS_LAUNCH_CHECK();
        if (DIM == 3) {
            k_diffuse_z<<<dim3((g.W - 2 + 127) / 128, g.H - 2), 128, 0, c->stream>>>(g, c->rho, c->gamma, c->solid);
            EFS_LAUNCH_CHECK();
        }
    }
    return cudaSuccess;
}

static ForceArgs force_args(efs_ctx* c, int enabled) {
    ForceArgs f;
    f.enabled = enabled;
    f.has_forces = c->has_forces ? 1 : 0;
    f.gravity = c->prm.gravity_enabled ? 1 : 0;
    f.dt = c->prm.dt;
    f.gforce = c->prm.gravity_force;
    f.fx = c->fx; f.fy = c->fy; f.fz = c->fz;
    return f;
}

// `traced`: rho_advect of the same step left every interior cell's trace end in tvel (the step runs the
// two stages back to back), so only the samples at the ends are taken.
static cudaError_t stage_vel_advect(efs_ctx* c, bool fuse_force, bool traced = false) {
    const Geo& g = c->g;
    float* tu = c->tvel; float* tv = c->tvel + g.N; float* tw = c->tvel + 2 * (size_t)g.N;
    const dim3 b(BX, BY), gr = grid_interior(g, c->dim);
    const ForceArgs f = force_args(c, fuse_force ? 1 : 0);
    if (c->dim == 3) {
        if (traced) k_vadv_sample<3><<<gr, b, 0, c->stream>>>(g, c->u, c->v, c->w, tu, tv, tw);
        else k_vadv_trace<3><<<gr, b, 0, c->stream>>>(g, c->u, c->v, c->w, c->solid, c->prm.dt, tu, tv, tw);
        EFS_LAUNCH_CHECK();
        k_vadv_average<3><<<gr, b, 0, c->stream>>>(g, tu, tv, tw, c->solid, c->u, c->v, c->w, f);
    } else {
        if (traced) k_vadv_sample<2><<<gr, b, 0, c->stream>>>(g, c->u, c->v, c->w, tu, tv, tw);
        else k_vadv_trace<2><<<gr, b, 0, c->stream>>>(g, c->u, c->v, c->w, c->solid, c->prm.dt, tu, tv, tw);
        EFS_LAUNCH_CHECK();
        k_vadv_average<2><<<gr, b, 0, c->stream>>>(g, tu, tv, tw, c->solid, c->u, c->v, c->w, f);
    }
    EFS_LAUNCH_CHECK();
    return cudaSuccess;
}

static cudaError_t stage_add_force(efs_ctx* c) {
    const dim3 b(BX, BY), gr = grid_interior(c->g, c->dim);
    const ForceArgs f = force_args(c, 1);
    if (c->dim == 3) k_add_force<3><<<gr, b, 0, c->stream>>>(c->g, c->solid, c->u, c->v, c->w, f);
    else k_add_force<2><<<gr, b, 0, c->stream>>>(c->g, c->solid, c->u, c->v, c->w, f);
    EFS_LAUNCH_CHECK();
    return cudaSuccess;
}

static ProjectArgs project_args(efs_ctx* c) {
    ProjectArgs a;
    a.thrL = c->prm.liquid_threshold; a.lp = c->prm.lambda_plus; a.lm = c->prm.lambda_minus; a.eta = c->prm.eta;
    a.jacobi = c->prm.solver == EFS_SOLVER_JACOBI;
    return a;
}

cudaError_t launch_project_pre(efs_ctx* c) {
    const Geo& g = c->g;
    const ProjectArgs a = project_args(c);
    const int nthreads = 256;
    const int nblk = (((g.N + 31) / 32) * 32 + nthreads - 1) / nthreads;
    if (c->dim == 3) k_project_pre<3><<<nblk, nthreads, 0, c->stream>>>(g, c->u, c->v, c->w, c->rho, c->solid, c->div, c->p, c->rowinfo, c->chunk_flag, a);
    else k_project_pre<2><<<nblk, nthreads, 0, c->stream>>>(g, c->u, c->v, c->w, c->rho, c->solid, c->div, c->p, c->rowinfo, c->chunk_flag, a);
    EFS_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t launch_project_post(efs_ctx* c) {
    const Geo& g = c->g;
    const dim3 b(BX, BY);
    const dim3 gr((g.W - 1 + BX - 1) / BX, (g.H - 1 + BY - 1) / BY, c->dim == 3 ? g.D - 1 : 1);
    if (c->dim == 3) {
        k_project_post<3><<<gr, b, 0, c->stream>>>(g, c->u, c->v, c->w, c->p, c->solid, c->ctl, 1);
        EFS_LAUNCH_CHECK();
    } else if (!c->prm.re_calc_div) {
        k_project_post<2><<<gr, b, 0, c->stream>>>(g, c->u, c->v, c->w, c->p, c->solid, c->ctl, 1);
        EFS_LAUNCH_CHECK();
    } else {
        k_project_post<2><<<gr, b, 0, c->stream>>>(g, c->u, c->v, c->w, c->p, c->solid, c->ctl, 0);
        EFS_LAUNCH_CHECK();
        k_recalc_div2<<<grid_interior(g, 2), b, 0, c->stream>>>(g, c->u, c->v, c->rho, c->solid, c->div, project_args(c), c->ctl);
        EFS_LAUNCH_CHECK();
        k_walls2<<<grid_linear(g.N, 256), 256, 0, c->stream>>>(g, c->u, c->v, c->solid, c->ctl);
        EFS_LAUNCH_CHECK();
    }
    return cudaSuccess;
}

cudaError_t launch_solver_prep(efs_ctx* c) {
    const Geo& g = c->g;
    const int nthreads = 256;
    const int nblk = (((g.N + 31) / 32) * 32 + nthreads - 1) / nthreads;
    const int jacobi = c->prm.solver == EFS_SOLVER_JACOBI;
    if (c->dim == 3) k_solver_prep<3><<<nblk, nthreads, 0, c->stream>>>(g, c->rho, c->solid, c->div, c->p, c->rowinfo, c->chunk_flag, jacobi);
    else k_solver_prep<2><<<nblk, nthreads, 0, c->stream>>>(g, c->rho, c->solid, c->div, c->p, c->rowinfo, c->chunk_flag, jacobi);
    EFS_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t launch_stage(efs_ctx* c, int stage, bool fuse_add_force, bool chain_traces) {
    switch (stage) {
        case EFS_STAGE_VEL_DECAY: return stage_decay(c);
        case EFS_STAGE_VEL_EXTRAPOLATE: return stage_extrapolate(c);
        case EFS_STAGE_RHO_SHARPEN: return stage_sharpen(c);
        case EFS_STAGE_RHO_ADVECT: return c->dim == 3 ? stage_advect_t<3>(c, chain_traces) : stage_advect_t<2>(c, chain_traces);
        case EFS_STAGE_VEL_ADVECT: return stage_vel_advect(c, fuse_add_force, chain_traces);
        case EFS_STAGE_ADD_FORCE: return stage_add_force(c);
        case EFS_STAGE_PROJECT: {
            cudaError_t e = launch_project_pre(c);
            if (e != cudaSuccess) return e;
            if ((e = launch_solver(c)) != cudaSuccess) return e;
            return launch_project_post(c);
        }
        default: return cudaErrorInvalidValue;
    }
}

// ================================================================================================
// Batched 2D scenes (efs_batch.h): the per-block code of the kernels above, run by persistent launches that
// walk a table of (scene, virtual block) entries, on each scene's geometry and packed field pointers.
// ================================================================================================
namespace {

template <class F>
__device__ __forceinline__ void for_entries(const BView& t, F f) {
    for (int k = blockIdx.x; k < t.n; k += gridDim.x) {
        const BEntry E = t.e[k];
        f(t.sc[E.scene], E);
    }
}

__global__ void kb_vel_decay(BView t, BFields F, float k) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_vel_decay<2>(S.g, E.bx, E.by, 0, F.u + o, F.v + o, nullptr, F.rho + o, k);
    });
}
__global__ void kb_extrap_init(BView t, BFields F) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_extrap_init(S.g, E.bx, 0, 0, 2, F.rho + o, F.solid + o, F.validA + o);
    });
}
__global__ void kb_extrap_pass(BView t, BFields F, int odd, int settled) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        const float* su = (odd ? F.tu : F.u) + o;
        const float* sv = (odd ? F.tv : F.v) + o;
        float* du = (odd ? F.u : F.tu) + o;
        float* dv = (odd ? F.v : F.tv) + o;
        const uint8_t* sV = (odd ? F.validB : F.validA) + o;
        uint8_t* dV = (odd ? F.validA : F.validB) + o;
        d_extrap_pass<2>(S.g, E.bx, E.by, 0, su, sv, nullptr, sV, du, dv, nullptr, dV, F.solid + o, settled != 0);
    });
}
__global__ void kb_sharpen_calc(BView t, BFields F, float delT) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        d_sharpen_calc<2>(S.g, E.bx, E.by, 0, F.rho + S.base, delT, F.sh_idx, F.sh_val, F.ctl, F.list_cap, (int)S.base,
                          E.scene, F.sh_sid);
    });
}
__global__ void kb_sharpen_apply(BFields F) {
    const int n = min(F.ctl->sh_count, F.list_cap);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const int i = F.sh_idx[s];
        F.rho[i] = maxf(F.rho[i] + F.sh_val[s], 0.f);
    }
}
__global__ void kb_sharpen_trace(BFields F, const BScene* __restrict__ sc, float Dist) {
    const int n = min(F.ctl->sh_count, F.list_cap);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const BScene S = sc[F.sh_sid[s]];
        float px, py, pz;
        sharpen_trace_one<2>(S.g, F.rho + S.base, F.solid + S.base, F.sh_idx[s] - (int)S.base, Dist, px, py, pz);
        F.sh_end[3 * s] = px; F.sh_end[3 * s + 1] = py; F.sh_end[3 * s + 2] = pz;
    }
}
__global__ void kb_sharpen_scatter(BFields F, const BScene* __restrict__ sc) {
    const int n = min(F.ctl->sh_count, F.list_cap);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const BScene S = sc[F.sh_sid[s]];
        sharpen_scatter_one<2>(S.g, F.rho + S.base, F.solid + S.base, F.sh_end[3 * s], F.sh_end[3 * s + 1],
                               F.sh_end[3 * s + 2], -F.sh_val[s]);
    }
}
__global__ void kb_adv_backward(BView t, BFields F, float dt, int keep_trace) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_adv_backward<2>(S.g, E.bx, E.by, 0, F.u + o, F.v + o, nullptr, F.solid + o, F.gamma + o, dt, F.wb + 4 * o,
                          F.bb + o, F.bsum + o, keep_trace ? F.tu + o : nullptr, keep_trace ? F.tv + o : nullptr);
    });
}
__global__ void kb_adv_forward(BView t, BFields F, float dt) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_adv_forward<2>(S.g, E.bx, E.by, 0, F.u + o, F.v + o, nullptr, F.solid + o, F.bsum + o, dt, F.wf + 4 * o,
                         F.fb + o, F.gsum + o);
    });
}
__global__ void kb_adv_rows(BView t, BFields F) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_adv_rows<2>(S.g, E.bx, E.by, 0, F.wb + 4 * o, F.bb + o, F.gsum + o, F.beta + o);
    });
}
__global__ void kb_adv_cols(BView t, BFields F) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_adv_cols<2>(S.g, E.bx, E.by, 0, F.wf + 4 * o, F.fb + o, F.gsum + o, F.beta + o);
    });
}
__global__ void kb_adv_apply_rows(BView t, BFields F) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_adv_apply_rows<2>(S.g, E.bx, 0, 0, F.wb + 4 * o, F.bb + o, F.beta + o, F.rho + o, F.gamma + o, F.rho_acc + o);
    });
}
__global__ void kb_adv_apply_cols(BView t, BFields F) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_adv_apply_cols<2>(S.g, E.bx, E.by, 0, F.wf + 4 * o, F.fb + o, F.beta + o, F.rho + o, F.gamma + o, F.rho_acc + o);
    });
}
__global__ void kb_diffuse_x(BView t, BFields F, int first) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_diffuse_x(S.g, E.bx, 0, 0, 2, (first ? F.rho_acc : F.rho) + o, F.gamma + o, F.rho + o, F.gamma + o, F.solid + o);
    });
}
__global__ void kb_diffuse_y(BView t, BFields F) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_diffuse_y(S.g, E.bx, 0, 0, 2, F.rho + o, F.gamma + o, F.solid + o);
    });
}
__global__ void kb_vadv_trace(BView t, BFields F, float dt) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_vadv_trace<2>(S.g, E.bx, E.by, 0, F.u + o, F.v + o, nullptr, F.solid + o, dt, F.tu + o, F.tv + o, nullptr);
    });
}
// vel_advect's samples at the trace ends kb_adv_backward kept in tu, tv (see k_vadv_sample)
__global__ void kb_vadv_sample(BView t, BFields F) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        int x, y, i;
        if (!cell2(S.g, E.bx, E.by, x, y, i)) return;
        float* tu = F.tu + o;
        float* tv = F.tv + o;
        float a, b;
        vinterp2(F.u + o, F.v + o, S.g, tu[i] - 0.5f, tv[i] - 0.5f, a, b);
        tu[i] = a;
        tv[i] = b;
    });
}
__global__ void kb_vadv_average(BView t, BFields F, ForceArgs f0) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        ForceArgs f = f0;
        f.gforce = S.gforce;
        f.fx = F.fx + o;
        f.fy = F.fy + o;
        d_vadv_average<2>(S.g, E.bx, E.by, 0, F.tu + o, F.tv + o, nullptr, F.solid + o, F.u + o, F.v + o, nullptr, f);
    });
}
__global__ void kb_add_force(BView t, BFields F, ForceArgs f0) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        ForceArgs f = f0;
        f.gforce = S.gforce;
        f.fx = F.fx + o;
        f.fy = F.fy + o;
        d_add_force<2>(S.g, E.bx, E.by, 0, F.solid + o, F.u + o, F.v + o, nullptr, f);
    });
}
__global__ void kb_project_pre(BView t, BFields F, ProjectArgs a) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_project_pre<2>(S.g, E.bx, 0, 0, F.u + o, F.v + o, nullptr, F.rho + o, F.solid + o, F.div + o, F.p + o,
                         F.rowinfo + o, F.chunk_flag + (o >> 5), a);
    });
}
__global__ void kb_project_post(BView t, BFields F) {
    for_entries(t, [&](const BScene& S, const BEntry& E) {
        const long long o = S.base;
        d_project_post<2>(S.g, E.bx, E.by, 0, F.u + o, F.v + o, nullptr, F.p + o, F.solid + o, F.sctl + E.scene, 1);
    });
}

inline unsigned bgrid(const BView& t, int grid) { return (unsigned)std::max(1, std::min(t.n, grid)); }

}  // namespace

cudaError_t batch_project_pre(const BLaunch& L) {
    ProjectArgs a;
    a.thrL = L.thrL; a.lp = L.lp; a.lm = L.lm; a.eta = L.eta; a.jacobi = 0;
    kb_project_pre<<<bgrid(L.linear, L.grid), 256, 0, L.stream>>>(L.linear, L.F, a);
    EFS_LAUNCH_CHECK();
    return cudaSuccess;
}

cudaError_t batch_project_post(const BLaunch& L) {
    kb_project_post<<<bgrid(L.post, L.grid), dim3(L.bx_dim, L.by_dim), 0, L.stream>>>(L.post, L.F);
    EFS_LAUNCH_CHECK();
    return cudaSuccess;
}

// One stage (0-5) of every scene; the project stage is batch_project_pre + the solve + batch_project_post.
cudaError_t batch_stage(const BLaunch& L, int stage, bool fuse_add_force, bool chain_traces) {
    const dim3 blk(L.bx_dim, L.by_dim);
    const unsigned gi = bgrid(L.interior, L.grid);
    cudaStream_t st = L.stream;
    const BFields& F = L.F;
    switch (stage) {
        case EFS_STAGE_VEL_DECAY:
            kb_vel_decay<<<gi, blk, 0, st>>>(L.interior, F, L.vel_decay);
            EFS_LAUNCH_CHECK();
            return cudaSuccess;
        case EFS_STAGE_VEL_EXTRAPOLATE:
            kb_extrap_init<<<bgrid(L.linear, L.grid), 256, 0, st>>>(L.linear, F);
            EFS_LAUNCH_CHECK();
            for (int it = 0; it < 6; it++) {
                kb_extrap_pass<<<gi, blk, 0, st>>>(L.interior, F, it & 1, it >= 1);
                EFS_LAUNCH_CHECK();
            }
            return cudaSuccess;
        case EFS_STAGE_RHO_SHARPEN: {
            cudaError_t e = cudaMemsetAsync(&F.ctl->sh_count, 0, sizeof(int), st);
            if (e != cudaSuccess) return e;
            kb_sharpen_calc<<<gi, blk, 0, st>>>(L.interior, F, L.dt * 3);
            EFS_LAUNCH_CHECK();
            kb_sharpen_apply<<<L.list_grid, 256, 0, st>>>(F);
            EFS_LAUNCH_CHECK();
            kb_sharpen_trace<<<L.list_grid, 256, 0, st>>>(F, L.interior.sc, L.rho_d);
            EFS_LAUNCH_CHECK();
            kb_sharpen_scatter<<<L.list_grid, 256, 0, st>>>(F, L.interior.sc);
            EFS_LAUNCH_CHECK();
            return cudaSuccess;
        }
        case EFS_STAGE_RHO_ADVECT: {
            const size_t bytes = (size_t)L.total_cells * sizeof(float);
            cudaError_t e;
            if ((e = cudaMemsetAsync(F.bsum, 0, bytes, st)) != cudaSuccess) return e;
            if ((e = cudaMemsetAsync(F.gsum, 0, bytes, st)) != cudaSuccess) return e;
            kb_adv_backward<<<gi, blk, 0, st>>>(L.interior, F, L.dt, chain_traces ? 1 : 0);
            EFS_LAUNCH_CHECK();
            kb_adv_forward<<<gi, blk, 0, st>>>(L.interior, F, L.dt);
            EFS_LAUNCH_CHECK();
            if ((e = cudaMemsetAsync(F.beta, 0, bytes, st)) != cudaSuccess) return e;
            kb_adv_rows<<<gi, blk, 0, st>>>(L.interior, F);
            EFS_LAUNCH_CHECK();
            kb_adv_cols<<<gi, blk, 0, st>>>(L.interior, F);
            EFS_LAUNCH_CHECK();
            kb_adv_apply_rows<<<bgrid(L.linear, L.grid), 256, 0, st>>>(L.linear, F);
            EFS_LAUNCH_CHECK();
            kb_adv_apply_cols<<<gi, blk, 0, st>>>(L.interior, F);
            EFS_LAUNCH_CHECK();
            for (int it = 0; it < 7; it++) {
                kb_diffuse_x<<<bgrid(L.dx, L.grid), 128, 0, st>>>(L.dx, F, it == 0 ? 1 : 0);
                EFS_LAUNCH_CHECK();
                kb_diffuse_y<<<bgrid(L.dy, L.grid), 128, 0, st>>>(L.dy, F);
                EFS_LAUNCH_CHECK();
            }
            return cudaSuccess;
        }
        case EFS_STAGE_VEL_ADVECT: {
            ForceArgs f{};
            f.enabled = fuse_add_force ? 1 : 0;
            f.has_forces = 1;
            f.gravity = L.gravity;
            f.dt = L.dt;
            if (chain_traces) kb_vadv_sample<<<gi, blk, 0, st>>>(L.interior, F);
            else kb_vadv_trace<<<gi, blk, 0, st>>>(L.interior, F, L.dt);
            EFS_LAUNCH_CHECK();
            kb_vadv_average<<<gi, blk, 0, st>>>(L.interior, F, f);
            EFS_LAUNCH_CHECK();
            return cudaSuccess;
        }
        case EFS_STAGE_ADD_FORCE: {
            ForceArgs f{};
            f.enabled = 1;
            f.has_forces = 1;
            f.gravity = L.gravity;
            f.dt = L.dt;
            kb_add_force<<<gi, blk, 0, st>>>(L.interior, F, f);
            EFS_LAUNCH_CHECK();
            return cudaSuccess;
        }
        default:
            return cudaErrorInvalidValue;
    }
}

}  // namespace efs
