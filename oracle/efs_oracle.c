/*
 * efs_oracle.c — CPU oracle for the Eulerian liquid step.  TEST INFRASTRUCTURE ONLY: the checker for the
 * CUDA path and the timed CPU baseline.  Built with -ffp-contract=off so that every float operation
 * rounds as written, like the reference's x86-64 build.
 *
 * Reference files restated (paths within MarQMark/EulerianFluidSimulation):
 *   R3  = src/simulation/simulator/CPUSimulator3D.cpp      R2  = src/simulation/simulator/CPUSimulator2D.cpp
 *   G3  = src/simulation/data/Grid3D.cpp                   G2  = src/simulation/data/Grid2D.cpp
 *   S3  = src/simulation/data/ScalField3D.cpp              S2  = src/simulation/data/ScalField2D.cpp
 *   V3  = src/simulation/data/VecField3D.cpp               V2  = src/simulation/data/VecField2D.cpp
 *   CG  = src/simulation/solver/CGSolver.cpp               JS  = src/simulation/solver/JacobiSolver.cpp
 *   IS  = include/simulation/simulator/ISimulator.h
 */
#include "efs_oracle.h"

#ifdef _OPENMP
#include <omp.h>
#endif
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define BOUNDARY 1.0f

/* Threads.  When built with OpenMP (oracle/Makefile adds -fopenmp where the compiler has it) the solvers'
 * per-cell loops (matrix products, vector updates, Jacobi sweeps) run on all host threads; each cell's result
 * is the same as in the serial loop.  FP64 dot products are summed in fixed blocks of ORC_DOT_BLOCK cells,
 * each block in cell order and the block sums in block order, so the value does not depend on the thread
 * count; grids of up to ORC_DOT_BLOCK cells form one block, i.e. the plain serial sum.  The float dot products
 * of the reference (ScalField3D.h:91-97) and every stage stay serial, in the reference's order. */
#define ORC_DOT_BLOCK ((size_t)1 << 20)
#define ORC_PAR_MIN 65536   /* smaller loops stay on the calling thread */

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* sum over [0, n) of f(k) in the fixed block order above; f is an expression in the index variable */
#define ORC_BLOCKED_SUM(result, n, idx, expr) do { \
    const size_t n_ = (n); \
    const size_t nb_ = (n_ + ORC_DOT_BLOCK - 1) / ORC_DOT_BLOCK; \
    if (nb_ <= 1) { double s_ = 0; for (size_t idx = 0; idx < n_; idx++) s_ += (expr); (result) = s_; break; } \
    double* part_ = (double*)malloc(nb_ * sizeof(double)); \
    _Pragma("omp parallel for schedule(static)") \
    for (long k_ = 0; k_ < (long)nb_; k_++) { \
        const size_t lo_ = (size_t)k_ * ORC_DOT_BLOCK, hi_ = lo_ + ORC_DOT_BLOCK < n_ ? lo_ + ORC_DOT_BLOCK : n_; \
        double s_ = 0; \
        for (size_t idx = lo_; idx < hi_; idx++) s_ += (expr); \
        part_[k_] = s_; \
    } \
    double t_ = 0; \
    for (size_t k_ = 0; k_ < nb_; k_++) t_ += part_[k_]; \
    free(part_); \
    (result) = t_; \
} while (0)

typedef struct orc_fent { int32_t i, j; float val; } orc_fent;

void orc_params_default(efs_params* p);

struct orc_grid {
    int dim, W, H, D;
    size_t N;
    efs_params prm;
    int mode;
    float *vel, *tmpvel, *forces;              /* dim floats per cell */
    float *rho, *tmps, *gamma, *beta, *div, *p, *boundary;
    float *cg_t, *cg_r, *cg_d, *jac_tmp;
    /* advection matrix: backward rows (8 corners of one base cell) + unmerged forward entries */
    int32_t* bbase;
    float* wb;
    orc_fent* fent;
    size_t nf, fcap;
    /* stats */
    int64_t frames;
    int solve_steps, converged, paused;
    double rr, bb, thr;
    int64_t active, total_solve_steps, solves;
};

static inline size_t I3(const orc_grid* g, size_t x, size_t y, size_t z) {
    return z * (size_t)g->W * (size_t)g->H + y * (size_t)g->W + x;   /* ScalField3D.h:19-21 */
}
static inline size_t I2(const orc_grid* g, size_t x, size_t y) { return y * (size_t)g->W + x; } /* ScalField2D.h:16 */

static inline float clampf(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }  /* std::clamp */
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (hi < v ? hi : v); }
static inline float maxf(float a, float b) { return (a < b) ? b : a; }   /* std::max */
static inline float minf(float a, float b) { return (b < a) ? b : a; }   /* std::min */
static inline double maxd(double a, double b) { return (a < b) ? b : a; }

/* ------------------------------------------------------------------------------------------------ */
/* lifetime                                                                                         */
/* ------------------------------------------------------------------------------------------------ */

static float* zalloc(size_t n) { return (float*)calloc(n ? n : 1, sizeof(float)); }

orc_grid* orc_create(int dim, int w, int h, int d, const efs_params* prm) {
    if (dim == 2) d = 1;
    if ((dim != 2 && dim != 3) || w < 4 || h < 4 || (dim == 3 && d < 4)) return NULL;
    orc_grid* g = (orc_grid*)calloc(1, sizeof(orc_grid));
    g->dim = dim; g->W = w; g->H = h; g->D = d;
    g->N = (size_t)w * h * d;
    if (prm) g->prm = *prm; else orc_params_default(&g->prm);
    size_t N = g->N;
    g->vel = zalloc(N * dim); g->tmpvel = zalloc(N * dim); g->forces = zalloc(N * dim);
    g->rho = zalloc(N); g->tmps = zalloc(N); g->gamma = zalloc(N); g->beta = zalloc(N);
    g->div = zalloc(N); g->p = zalloc(N); g->boundary = zalloc(N);
    g->cg_t = zalloc(N); g->cg_r = zalloc(N); g->cg_d = zalloc(N); g->jac_tmp = zalloc(N);
    g->bbase = (int32_t*)malloc(N * sizeof(int32_t));
    g->wb = zalloc(N * (dim == 3 ? 8 : 4));
    g->fcap = 1024; g->fent = (orc_fent*)malloc(g->fcap * sizeof(orc_fent));
    orc_reset(g);
    return g;
}

void orc_destroy(orc_grid* g) {
    if (!g) return;
    float* bufs[] = {g->vel, g->tmpvel, g->forces, g->rho, g->tmps, g->gamma, g->beta, g->div, g->p,
                     g->boundary, g->cg_t, g->cg_r, g->cg_d, g->jac_tmp, g->wb};
    for (size_t i = 0; i < sizeof(bufs) / sizeof(bufs[0]); i++) free(bufs[i]);
    free(g->bbase); free(g->fent); free(g);
}

void orc_set_params(orc_grid* g, const efs_params* prm) { g->prm = *prm; }
void orc_set_mode(orc_grid* g, int mode) { g->mode = mode; }

float* orc_field(orc_grid* g, int f) {
    switch (f) {
        case EFS_FIELD_VEL: return g->vel;
        case EFS_FIELD_RHO: return g->rho;
        case EFS_FIELD_GAMMA: return g->gamma;
        case EFS_FIELD_BETA: return g->beta;
        case EFS_FIELD_DIVERGENCE: return g->div;
        case EFS_FIELD_PRESSURE: return g->p;
        case EFS_FIELD_FORCES: return g->forces;
        case EFS_FIELD_BOUNDARY: return g->boundary;
        default: return NULL;
    }
}

/* Grid3D::Grid3D (G3:10-48) / Grid2D::Grid2D (G2:11-66 with INIT_SHAPE EMPTY): zero fields, gamma = 1,
 * border solid with rho 0. */
void orc_reset(orc_grid* g) {
    size_t N = g->N;
    memset(g->vel, 0, N * g->dim * sizeof(float)); memset(g->tmpvel, 0, N * g->dim * sizeof(float));
    memset(g->forces, 0, N * g->dim * sizeof(float));
    memset(g->rho, 0, N * 4); memset(g->tmps, 0, N * 4); memset(g->beta, 0, N * 4);
    memset(g->div, 0, N * 4); memset(g->p, 0, N * 4); memset(g->boundary, 0, N * 4);
    memset(g->cg_t, 0, N * 4); memset(g->cg_r, 0, N * 4); memset(g->cg_d, 0, N * 4); memset(g->jac_tmp, 0, N * 4);
    for (size_t i = 0; i < N; i++) g->gamma[i] = 1.0f;
    for (int z = 0; z < g->D; z++)
    for (int y = 0; y < g->H; y++)
    for (int x = 0; x < g->W; x++) {
        int border = (x == 0 || y == 0 || x == g->W - 1 || y == g->H - 1);
        if (g->dim == 3) border = border || z == 0 || z == g->D - 1;
        if (border) { size_t i = (size_t)z * g->W * g->H + (size_t)y * g->W + x; g->boundary[i] = 1.0f; g->rho[i] = 0.0f; }
    }
    g->frames = 0; g->solve_steps = 0; g->converged = 0; g->paused = 0;
    g->rr = g->bb = g->thr = 0; g->active = 0; g->total_solve_steps = 0; g->solves = 0;
}

void orc_stats(const orc_grid* g, efs_stats* s) {
    memset(s, 0, sizeof(*s));
    s->frames = g->frames; s->solve_steps = g->solve_steps; s->converged = g->converged; s->paused = g->paused;
    s->rr = g->rr; s->bb = g->bb; s->threshold = g->thr; s->active_cells = g->active;
    s->total_solve_steps = g->total_solve_steps; s->solves = g->solves;
}

double orc_total_mass(orc_grid* g) {
    double s = 0; for (size_t i = 0; i < g->N; i++) s += g->rho[i]; return s;
}

/* ------------------------------------------------------------------------------------------------ */
/* 3D interpolation and tracing                                                                     */
/* ------------------------------------------------------------------------------------------------ */

/* StaggeredOffset3D (V3:12-19) */
static const float OFF3[3][3] = {{-1.0f, -0.5f, -0.5f}, {-0.5f, -1.0f, -0.5f}, {-0.5f, -0.5f, -1.0f}};

/* VecField3D::trilinear_interpolation (V3:21-50) */
static float vtrilin3(const orc_grid* g, const float* vel, float px, float py, float pz, int lx, int ly, int lz, int c) {
    const float x0 = (float)lx + OFF3[c][0];
    const float y0 = (float)ly + OFF3[c][1];
    const float z0 = (float)lz + OFF3[c][2];
    const float tx = px - x0, ty = py - y0, tz = pz - z0;
    const float v000 = vel[3 * I3(g, lx, ly, lz) + c];
    const float v001 = vel[3 * I3(g, lx, ly, lz + 1) + c];
    const float v010 = vel[3 * I3(g, lx, ly + 1, lz) + c];
    const float v011 = vel[3 * I3(g, lx, ly + 1, lz + 1) + c];
    const float v100 = vel[3 * I3(g, lx + 1, ly, lz) + c];
    const float v101 = vel[3 * I3(g, lx + 1, ly, lz + 1) + c];
    const float v110 = vel[3 * I3(g, lx + 1, ly + 1, lz) + c];
    const float v111 = vel[3 * I3(g, lx + 1, ly + 1, lz + 1) + c];
    const float v00 = v000 * (1.0f - tz) + v001 * tz;
    const float v01 = v010 * (1.0f - tz) + v011 * tz;
    const float v10 = v100 * (1.0f - tz) + v101 * tz;
    const float v11 = v110 * (1.0f - tz) + v111 * tz;
    const float vLow = v00 * (1.0f - ty) + v01 * ty;
    const float vHigh = v10 * (1.0f - ty) + v11 * ty;
    return vLow * (1.0f - tx) + vHigh * tx;
}

/* VecField3D::interpolate (V3:54-78); lowIndex = (int)(floor(coord - offset) + 1e-10f) */
static void vinterp3(const orc_grid* g, const float* vel, float px, float py, float pz, float out[3]) {
    for (int c = 0; c < 3; c++) {
        const int lx = (int)(floorf(px - OFF3[c][0]) + 1.0e-10f);
        const int ly = (int)(floorf(py - OFF3[c][1]) + 1.0e-10f);
        const int lz = (int)(floorf(pz - OFF3[c][2]) + 1.0e-10f);
        out[c] = vtrilin3(g, vel, px, py, pz, lx, ly, lz, c);
    }
}

/* ScalField3D::interpolate (S3:18-107): samples at i + 0.5, clamped indices */
static float sinterp3(const orc_grid* g, const float* f, float px, float py, float pz) {
    const int x = (int)px, y = (int)py, z = (int)pz;
    int ix1 = x, ix2 = x + 1;
    if (px - (float)x < 0.5f) { ix1 = x - 1; ix2 = x; }
    int iy1 = y, iy2 = y + 1;
    if (py - (float)y < 0.5f) { iy1 = y - 1; iy2 = y; }
    int iz1 = z, iz2 = z + 1;
    if (pz - (float)z < 0.5f) { iz1 = z - 1; iz2 = z; }
    ix1 = clampi(ix1, 0, g->W - 1); ix2 = clampi(ix2, 0, g->W - 1);
    iy1 = clampi(iy1, 0, g->H - 1); iy2 = clampi(iy2, 0, g->H - 1);
    iz1 = clampi(iz1, 0, g->D - 1); iz2 = clampi(iz2, 0, g->D - 1);
    const float v[8] = {
        f[I3(g, ix1, iy1, iz1)], f[I3(g, ix1, iy1, iz2)], f[I3(g, ix1, iy2, iz1)], f[I3(g, ix1, iy2, iz2)],
        f[I3(g, ix2, iy1, iz1)], f[I3(g, ix2, iy1, iz2)], f[I3(g, ix2, iy2, iz1)], f[I3(g, ix2, iy2, iz2)],
    };
    const float x1 = (float)ix1 + 0.5f, x2 = (float)ix2 + 0.5f;
    const float y1 = (float)iy1 + 0.5f, y2 = (float)iy2 + 0.5f;
    const float z1 = (float)iz1 + 0.5f, z2 = (float)iz2 + 0.5f;
    const float dz2z1 = z2 - z1;
    float f00, f01, f10, f11;
    if (dz2z1 < 1e-9f) { f00 = v[1]; f01 = v[3]; f10 = v[5]; f11 = v[7]; }
    else {
        const float wz1 = (z2 - pz) / dz2z1, wz2 = (pz - z1) / dz2z1;
        f00 = wz1 * v[0] + wz2 * v[1]; f01 = wz1 * v[2] + wz2 * v[3];
        f10 = wz1 * v[4] + wz2 * v[5]; f11 = wz1 * v[6] + wz2 * v[7];
    }
    const float dy2y1 = y2 - y1;
    float fx1, fx2;
    if (dy2y1 < 1e-9f) { fx1 = f01; fx2 = f11; }
    else {
        const float wy1 = (y2 - py) / dy2y1, wy2 = (py - y1) / dy2y1;
        fx1 = wy1 * f00 + wy2 * f01; fx2 = wy1 * f10 + wy2 * f11;
    }
    const float dx2x1 = x2 - x1;
    if (dx2x1 < 1e-9f) return fx2;
    const float wx1 = (x2 - px) / dx2x1, wx2 = (px - x1) / dx2x1;
    return wx1 * fx1 + wx2 * fx2;
}

/* Grid3D::traceParticle inWall (G3:73-80) */
static int inwall3(const orc_grid* g, float px, float py, float pz) {
    const float W = (float)g->W, H = (float)g->H, D = (float)g->D;
    if (px < 1.f || px > W - 2.f || py < 1.f || py > H - 2.f || pz < 1.f || pz > D - 2.f) return 1;
    const int ix = clampi((int)px, 0, g->W - 1), iy = clampi((int)py, 0, g->H - 1), iz = clampi((int)pz, 0, g->D - 1);
    return g->boundary[I3(g, ix, iy, iz)] > 0.5f;
}

/* Grid3D::traceParticle (G3:66-122): RK2 midpoint, mid clamped, 8-step bisection at walls */
static void trace3(const orc_grid* g, float sx, float sy, float sz, float dt, int substeps, float out[3]) {
    const float W = (float)g->W, H = (float)g->H, D = (float)g->D;
    out[0] = sx; out[1] = sy; out[2] = sz;
    if (inwall3(g, sx, sy, sz)) return;
    const float subDt = dt / (float)substeps;
    float p[3] = {sx, sy, sz};
    for (int s = 0; s < substeps; s++) {
        float k1[3], k2[3], mid[3], nx[3];
        vinterp3(g, g->vel, p[0] - 0.5f, p[1] - 0.5f, p[2] - 0.5f, k1);
        const float h = subDt * 0.5f;
        mid[0] = clampf(p[0] + k1[0] * h, 1.f, W - 2.f);
        mid[1] = clampf(p[1] + k1[1] * h, 1.f, H - 2.f);
        mid[2] = clampf(p[2] + k1[2] * h, 1.f, D - 2.f);
        vinterp3(g, g->vel, mid[0] - 0.5f, mid[1] - 0.5f, mid[2] - 0.5f, k2);
        nx[0] = p[0] + k2[0] * subDt; nx[1] = p[1] + k2[1] * subDt; nx[2] = p[2] + k2[2] * subDt;
        if (inwall3(g, nx[0], nx[1], nx[2])) {
            float safe[3] = {p[0], p[1], p[2]}, unsafe[3] = {nx[0], nx[1], nx[2]};
            for (int b = 0; b < 8; b++) {
                float hw[3] = {(safe[0] + unsafe[0]) * 0.5f, (safe[1] + unsafe[1]) * 0.5f, (safe[2] + unsafe[2]) * 0.5f};
                if (inwall3(g, hw[0], hw[1], hw[2])) memcpy(unsafe, hw, sizeof hw); else memcpy(safe, hw, sizeof hw);
            }
            out[0] = safe[0]; out[1] = safe[1]; out[2] = safe[2];
            return;
        }
        p[0] = nx[0]; p[1] = nx[1]; p[2] = nx[2];
    }
    out[0] = p[0]; out[1] = p[1]; out[2] = p[2];
}

/* ------------------------------------------------------------------------------------------------ */
/* 3D stages                                                                                         */
/* ------------------------------------------------------------------------------------------------ */

#define LOOP3(g, off) for (int z = (off); z < (g)->D - (off); z++) \
                      for (int y = (off); y < (g)->H - (off); y++) \
                      for (int x = (off); x < (g)->W - (off); x++)

/* R3:54-59 */
static void vel_decay3(orc_grid* g) {
    const float k = g->prm.vel_decay;
    LOOP3(g, 1) {
        size_t i = I3(g, x, y, z);
        if ((double)g->rho[i] < 0.5) { g->vel[3*i] *= k; g->vel[3*i+1] *= k; g->vel[3*i+2] *= k; }
    }
}

/* R3:61-111: valid = rho >= 0.5 and not solid; 3 x (A->B, B->A) neighbour-average passes */
static void vel_extrapolate3(orc_grid* g) {
    const size_t N = g->N;
    float* validA = zalloc(N);
    float* validB = zalloc(N);
    LOOP3(g, 1) {
        size_t i = I3(g, x, y, z);
        validA[i] = (g->rho[i] >= 0.5f && g->boundary[i] != BOUNDARY) ? 1.f : 0.f;
    }
    for (int it = 0; it < 6; it++) {
        float* sv = (it & 1) ? g->tmpvel : g->vel;
        float* sV = (it & 1) ? validB : validA;
        float* dv = (it & 1) ? g->vel : g->tmpvel;
        float* dV = (it & 1) ? validA : validB;
        LOOP3(g, 1) {
            size_t i = I3(g, x, y, z);
            if (g->boundary[i] == BOUNDARY) { memcpy(&dv[3*i], &sv[3*i], 12); dV[i] = 0.f; continue; }
            if (sV[i] > 0.5f) { memcpy(&dv[3*i], &sv[3*i], 12); dV[i] = 1.f; continue; }
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, n = 0;
            const size_t nb[6] = {I3(g, x-1, y, z), I3(g, x+1, y, z), I3(g, x, y-1, z), I3(g, x, y+1, z),
                                  I3(g, x, y, z-1), I3(g, x, y, z+1)};
            for (int k = 0; k < 6; k++)
                if (sV[nb[k]] > 0.5f) { s0 += sv[3*nb[k]]; s1 += sv[3*nb[k]+1]; s2 += sv[3*nb[k]+2]; n++; }
            if (n > 0) { dv[3*i] = s0 / n; dv[3*i+1] = s1 / n; dv[3*i+2] = s2 / n; }
            else memcpy(&dv[3*i], &sv[3*i], 12);
            dV[i] = (n > 0) ? 1.f : 0.f;
        }
    }
    free(validA); free(validB);
}

/* trilinear weights on integer-centred corners (R3:140-159 and :195-214): corner k = (k&1, k>>1&1, k>>2&1) */
static float corner_weights3(const orc_grid* g, const float pos[3], int p0[3], float m[8]) {
    p0[0] = (int)floorf(pos[0]); p0[1] = (int)floorf(pos[1]); p0[2] = (int)floorf(pos[2]);
    const float dx0 = 1 - (pos[0] - (float)p0[0]);
    const float dy0 = 1 - (pos[1] - (float)p0[1]);
    const float dz0 = 1 - (pos[2] - (float)p0[2]);
    const float dx1 = 1 - ((float)(p0[0] + 1) - pos[0]);
    const float dy1 = 1 - ((float)(p0[1] + 1) - pos[1]);
    const float dz1 = 1 - ((float)(p0[2] + 1) - pos[2]);
    const float wx[2] = {dx0, dx1}, wy[2] = {dy0, dy1}, wz[2] = {dz0, dz1};
    float sum = 0;
    for (int k = 0; k < 8; k++) {
        const int ox = k & 1, oy = (k >> 1) & 1, oz = (k >> 2) & 1;
        m[k] = 0;
        if (g->boundary[I3(g, p0[0] + ox, p0[1] + oy, p0[2] + oz)] != BOUNDARY) m[k] = wx[ox] * wy[oy] * wz[oz];
    }
    for (int k = 0; k < 8; k++) sum += m[k];
    return sum;
}

static void fent_push(orc_grid* g, int32_t i, int32_t j, float val) {
    if (g->nf == g->fcap) { g->fcap *= 2; g->fent = (orc_fent*)realloc(g->fent, g->fcap * sizeof(orc_fent)); }
    g->fent[g->nf].i = i; g->fent[g->nf].j = j; g->fent[g->nf].val = val; g->nf++;
}

/* Grid3D::addA for a forward entry (i, j): merge into row i's backward entry for column j if it has one. */
static void add_forward3(orc_grid* g, int32_t i, int32_t j, float val) {
    const int32_t b = g->bbase[i];
    if (b >= 0) {
        const size_t W = g->W, WH = (size_t)g->W * g->H;
        const long dz = (long)(j / WH) - (long)(b / WH);
        const long dy = (long)((j % WH) / W) - (long)((b % WH) / W);
        const long dx = (long)(j % W) - (long)(b % W);
        if (dx >= 0 && dx <= 1 && dy >= 0 && dy <= 1 && dz >= 0 && dz <= 1) {
            g->wb[(size_t)i * 8 + (dx + 2 * dy + 4 * dz)] += val;
            return;
        }
    }
    fent_push(g, i, j, val);
}

/* iterate every entry (i, j, &val) of A: backward rows in cell order, then forward entries; with
 * ORC_REVERSE_SUMS the exact reverse order (a summation-order perturbation for drift bounds) */
#define FOR_ENTRIES3(g, BODY) do { \
    const size_t W_ = (g)->W, WH_ = (size_t)(g)->W * (g)->H; \
    const int rev_ = ((g)->mode & ORC_REVERSE_SUMS) != 0; \
    if (rev_) for (size_t e2_ = (g)->nf; e2_-- > 0;) { const size_t ci = (size_t)(g)->fent[e2_].i, cj = (size_t)(g)->fent[e2_].j; \
        float* cv = &(g)->fent[e2_].val; (void)ci; (void)cj; BODY } \
    for (size_t t_ = 0; t_ < (g)->N; t_++) { const size_t i_ = rev_ ? (g)->N - 1 - t_ : t_; \
        const int32_t b_ = (g)->bbase[i_]; if (b_ < 0) continue; \
        for (int q_ = 0; q_ < 8; q_++) { const int k_ = rev_ ? 7 - q_ : q_; const size_t ci = i_; \
            const size_t cj = (size_t)b_ + (k_ & 1) + ((k_ >> 1) & 1) * W_ + ((k_ >> 2) & 1) * WH_; \
            float* cv = &(g)->wb[i_ * 8 + k_]; (void)ci; (void)cj; BODY } } \
    if (!rev_) for (size_t e_ = 0; e_ < (g)->nf; e_++) { const size_t ci = (size_t)(g)->fent[e_].i, cj = (size_t)(g)->fent[e_].j; \
        float* cv = &(g)->fent[e_].val; (void)ci; (void)cj; BODY } } while (0)

/* R3:113-364 Chentanez-Mueller density advection */
static void rho_advect3(orc_grid* g) {
    float* rho = g->rho; float* gamma = g->gamma; float* beta = g->beta; const float* bnd = g->boundary;
    const size_t N = g->N;
    const float dt = g->prm.dt;
    (void)N;
    /* Step 1 (R3:121-131): gamma' = gamma at the back-traced position; zero elsewhere */
    float* advG = zalloc(g->N);
    LOOP3(g, 1) {
        size_t i = I3(g, x, y, z);
        if (bnd[i] == BOUNDARY) continue;
        float pp[3]; trace3(g, (float)x, (float)y, (float)z, -dt, 4, pp);
        advG[i] = sinterp3(g, gamma, pp[0], pp[1], pp[2]);
    }
    memcpy(gamma, advG, g->N * sizeof(float));
    free(advG);
    /* Step 2 (R3:133-173): backward weights m_k / sum */
    for (size_t i = 0; i < g->N; i++) g->bbase[i] = -1;
    g->nf = 0;
    LOOP3(g, 1) {
        size_t i = I3(g, x, y, z);
        float pp[3]; trace3(g, (float)x, (float)y, (float)z, -dt, 4, pp);
        int p0[3]; float m[8];
        const float sum = corner_weights3(g, pp, p0, m);
        if (sum == 0) continue;
        g->bbase[i] = (int32_t)I3(g, p0[0], p0[1], p0[2]);
        for (int k = 0; k < 8; k++) g->wb[i * 8 + k] = m[k] / sum;
    }
    /* Step 3 (R3:175-179) */
    FOR_ENTRIES3(g, { if (gamma[ci] > 1.e-5f) *cv /= gamma[ci]; });
    /* Step 4 (R3:181-185) */
    memset(beta, 0, g->N * 4);
    FOR_ENTRIES3(g, { beta[cj] += *cv; });
    /* Step 5 (R3:187-228): forward weights (1 - beta_j) m_k / sum for beta_j < 1 */
    LOOP3(g, 1) {
        const size_t j = I3(g, x, y, z);
        if (beta[j] >= 1) continue;
        float pp[3]; trace3(g, (float)x, (float)y, (float)z, +dt, 4, pp);
        int p0[3]; float m[8];
        const float sum = corner_weights3(g, pp, p0, m);
        if (sum == 0) continue;
        for (int k = 0; k < 8; k++) {
            const int32_t ti = (int32_t)I3(g, p0[0] + (k & 1), p0[1] + ((k >> 1) & 1), p0[2] + ((k >> 2) & 1));
            add_forward3(g, ti, (int32_t)j, (1 - beta[j]) * (m[k] / sum));
        }
    }
    /* Step 6 (R3:230-234) */
    memset(gamma, 0, g->N * 4);
    FOR_ENTRIES3(g, { gamma[ci] += *cv; });
    /* Step 7 (R3:236-240) */
    FOR_ENTRIES3(g, { if (gamma[ci] > 1.e-5f) *cv /= gamma[ci]; });
    /* Step 8 (R3:242-246) */
    memset(beta, 0, g->N * 4);
    FOR_ENTRIES3(g, { beta[cj] += *cv; });
    /* Step 9 (R3:248-252) */
    FOR_ENTRIES3(g, { if (beta[cj] > 1.e-5f) *cv /= beta[cj]; });
    /* Step 10 (R3:259-263) */
    memset(gamma, 0, g->N * 4);
    FOR_ENTRIES3(g, { gamma[ci] += *cv; });
    /* Step 11 (R3:265-272) */
    float* adv = g->tmps;
    memset(adv, 0, g->N * 4);
    FOR_ENTRIES3(g, { adv[ci] += *cv * rho[cj]; });
    LOOP3(g, 1) { size_t i = I3(g, x, y, z); rho[i] = adv[i]; }
    /* Step 12 (R3:274-363): 3 iterations of in-place pairwise gamma-equalising transfer along x, y, z */
    for (int it = 0; it < 3; it++) {
        for (int dirn = 0; dirn < 3; dirn++) {
            int na, nb2, nc; /* loop extents: outer, middle, inner (inner is the sweep axis) */
            if (dirn == 0) { na = g->D; nb2 = g->H; nc = g->W; }
            else if (dirn == 1) { na = g->D; nb2 = g->W; nc = g->H; }
            else { na = g->H; nb2 = g->W; nc = g->D; }
            for (int a = 1; a < na - 1; a++)
            for (int b = 1; b < nb2 - 1; b++)
            for (int c = 2; c < nc - 1; c++) {
                size_t ii, jj;
                if (dirn == 0) { ii = I3(g, c, b, a); jj = I3(g, c - 1, b, a); }
                else if (dirn == 1) { ii = I3(g, b, c, a); jj = I3(g, b, c - 1, a); }
                else { ii = I3(g, b, a, c); jj = I3(g, b, a, c - 1); }
                const float g_j = gamma[jj], g_i = gamma[ii];
                if (bnd[ii] == BOUNDARY || bnd[jj] == BOUNDARY) continue;
                if (g_j < 1e-5f || g_i < 1e-5f) continue;
                if (g_j == g_i) continue;
                const float avg = (g_j + g_i) / 2.f;
                if (g_j > g_i) {
                    const float dif = rho[jj] * (g_j - g_i) / (2.f * g_j);
                    rho[jj] -= dif; rho[ii] += dif;
                } else {
                    const float dif = rho[ii] * (g_i - g_j) / (2.f * g_i);
                    rho[ii] -= dif; rho[jj] += dif;
                }
                gamma[jj] = avg; gamma[ii] = avg;
            }
        }
    }
}

/* CPUSimulator3D::trace_along_field (R3:568-607) */
static void trace_field3(const orc_grid* g, float sx, float sy, float sz, float Dist, int substeps, float out[3]) {
    const float stepSize = Dist / (float)substeps;
    const float* rho = g->rho;
    float p[3] = {sx, sy, sz};
    for (int s = 0; s < substeps; s++) {
        if (sinterp3(g, rho, p[0], p[1], p[2]) >= 0.5f) break;
        const int ix = clampi((int)p[0], 1, g->W - 2), iy = clampi((int)p[1], 1, g->H - 2), iz = clampi((int)p[2], 1, g->D - 2);
        const float gx = rho[I3(g, ix + 1, iy, iz)] - rho[I3(g, ix - 1, iy, iz)];
        const float gy = rho[I3(g, ix, iy + 1, iz)] - rho[I3(g, ix, iy - 1, iz)];
        const float gz = rho[I3(g, ix, iy, iz + 1)] - rho[I3(g, ix, iy, iz - 1)];
        const float len = sqrtf(gx * gx + gy * gy + gz * gz);   /* glm::length: sqrt((x*x + y*y) + z*z) */
        if (len < 1e-6f) break;
        float nx = p[0] + (gx / len) * stepSize, ny = p[1] + (gy / len) * stepSize, nz = p[2] + (gz / len) * stepSize;
        nx = clampf(nx, 1.f, (float)g->W - 2.f); ny = clampf(ny, 1.f, (float)g->H - 2.f); nz = clampf(nz, 1.f, (float)g->D - 2.f);
        if (g->boundary[I3(g, (size_t)nx, (size_t)ny, (size_t)nz)] > 0.5f) break;
        p[0] = nx; p[1] = ny; p[2] = nz;
    }
    out[0] = p[0]; out[1] = p[1]; out[2] = p[2];
}

/* CPUSimulator3D::scatter_values (R3:609-655) */
static void scatter3(orc_grid* g, const float pos[3], float value) {
    float* rho = g->rho; const float* bnd = g->boundary;
    const int x0 = clampi((int)pos[0], 0, g->W - 1), y0 = clampi((int)pos[1], 0, g->H - 1), z0 = clampi((int)pos[2], 0, g->D - 1);
    const int x1 = clampi((int)pos[0] + 1, 0, g->W - 1), y1 = clampi((int)pos[1] + 1, 0, g->H - 1), z1 = clampi((int)pos[2] + 1, 0, g->D - 1);
    const float fx = pos[0] - (float)(int)pos[0], fy = pos[1] - (float)(int)pos[1], fz = pos[2] - (float)(int)pos[2];
    float w000 = (1.f - fx) * (1.f - fy) * (1.f - fz);
    float w100 = fx * (1.f - fy) * (1.f - fz);
    float w010 = (1.f - fx) * fy * (1.f - fz);
    float w110 = fx * fy * (1.f - fz);
    float w001 = (1.f - fx) * (1.f - fy) * fz;
    float w101 = fx * (1.f - fy) * fz;
    float w011 = (1.f - fx) * fy * fz;
    float w111 = fx * fy * fz;
    if (bnd[I3(g, x0, y0, z0)] > 0.5f) w000 = 0.f;
    if (bnd[I3(g, x1, y0, z0)] > 0.5f) w100 = 0.f;
    if (bnd[I3(g, x0, y1, z0)] > 0.5f) w010 = 0.f;
    if (bnd[I3(g, x1, y1, z0)] > 0.5f) w110 = 0.f;
    if (bnd[I3(g, x0, y0, z1)] > 0.5f) w001 = 0.f;
    if (bnd[I3(g, x1, y0, z1)] > 0.5f) w101 = 0.f;
    if (bnd[I3(g, x0, y1, z1)] > 0.5f) w011 = 0.f;
    if (bnd[I3(g, x1, y1, z1)] > 0.5f) w111 = 0.f;
    const float total = w000 + w100 + w010 + w110 + w001 + w101 + w011 + w111;
    if (total < 1e-6f) return;
    const float inv = 1.f / total;
    rho[I3(g, x0, y0, z0)] += value * w000 * inv;
    rho[I3(g, x1, y0, z0)] += value * w100 * inv;
    rho[I3(g, x0, y1, z0)] += value * w010 * inv;
    rho[I3(g, x1, y1, z0)] += value * w110 * inv;
    rho[I3(g, x0, y0, z1)] += value * w001 * inv;
    rho[I3(g, x1, y0, z1)] += value * w101 * inv;
    rho[I3(g, x0, y1, z1)] += value * w011 * inv;
    rho[I3(g, x1, y1, z1)] += value * w111 * inv;
}

/* the per-axis term of max_inc / max_dec (R3:390-418): std::pow(float, int) is evaluated in double */
static inline double sq_d(float v) { return (double)v * (double)v; }

/* CPUSimulator3D::rho_sharpen (R3:366-456) */
static void rho_sharpen3(orc_grid* g) {
    float* rho = g->rho;
    const float delT = g->prm.dt * 3;
    const size_t N = g->N;
    float* del_rho = zalloc(N);
    LOOP3(g, 1) {
        const size_t i = I3(g, x, y, z);
        const float r = rho[i];
        const float rxm = rho[I3(g, x-1, y, z)], rxp = rho[I3(g, x+1, y, z)];
        const float rym = rho[I3(g, x, y-1, z)], ryp = rho[I3(g, x, y+1, z)];
        const float rzm = rho[I3(g, x, y, z-1)], rzp = rho[I3(g, x, y, z+1)];
        const float dpx = -(r - rxm) * delT, dmx = -(rxp - r) * delT;
        const float dpy = -(r - rym) * delT, dmy = -(ryp - r) * delT;
        const float dpz = -(r - rzm) * delT, dmz = -(rzp - r) * delT;
        const float max_inc = (float)sqrt(maxd(sq_d(maxf(dpx, 0.f)), sq_d(minf(dmx, 0.f))) +
                                          maxd(sq_d(maxf(dpy, 0.f)), sq_d(minf(dmy, 0.f))) +
                                          maxd(sq_d(maxf(dpz, 0.f)), sq_d(minf(dmz, 0.f))));
        const float max_dec = (float)sqrt(maxd(sq_d(minf(dpx, 0.f)), sq_d(maxf(dmx, 0.f))) +
                                          maxd(sq_d(minf(dpy, 0.f)), sq_d(maxf(dmy, 0.f))) +
                                          maxd(sq_d(minf(dpz, 0.f)), sq_d(maxf(dmz, 0.f))));
        float mx = -INFINITY;
        mx = maxf(mx, fabsf(r - rxm)); mx = maxf(mx, fabsf(r - rxp));
        mx = maxf(mx, fabsf(r - rym)); mx = maxf(mx, fabsf(r - ryp));
        mx = maxf(mx, fabsf(r - rzm)); mx = maxf(mx, fabsf(r - rzp));
        const float w = powf(r - 0.5f, 3.f) * (1 - minf(1.f, mx / 0.2f));
        float dr = (w >= 0) ? w * max_inc : w * max_dec;
        if (r + dr < 0 || (double)r < 1e-5) dr = -r;
        else if (r > 0.5f) dr = 0;
        del_rho[i] = dr;
    }
    if (!(g->mode & ORC_SHARPEN_PARALLEL)) {
        LOOP3(g, 1) {
            const size_t i = I3(g, x, y, z);
            const float dr = del_rho[i];
            if (fabsf(dr) < 1e-6f) continue;
            rho[i] += dr;
            rho[i] = maxf(rho[i], 0.f);
            float pp[3]; trace_field3(g, (float)x, (float)y, (float)z, g->prm.rho_d, 10, pp);
            scatter3(g, pp, -dr);
        }
    } else {
        float* ends = (float*)malloc(N * 3 * sizeof(float));
        LOOP3(g, 1) {
            const size_t i = I3(g, x, y, z);
            const float dr = del_rho[i];
            if (fabsf(dr) < 1e-6f) continue;
            rho[i] += dr;
            rho[i] = maxf(rho[i], 0.f);
        }
        LOOP3(g, 1) {
            const size_t i = I3(g, x, y, z);
            if (fabsf(del_rho[i]) < 1e-6f) continue;
            trace_field3(g, (float)x, (float)y, (float)z, g->prm.rho_d, 10, &ends[3 * i]);
        }
        LOOP3(g, 1) {
            const size_t i = I3(g, x, y, z);
            if (fabsf(del_rho[i]) < 1e-6f) continue;
            scatter3(g, &ends[3 * i], -del_rho[i]);
        }
        free(ends);
    }
    free(del_rho);
}

/* R3:458-476 */
static void add_force3(orc_grid* g) {
    const float dt = g->prm.dt;
    LOOP3(g, 1) {
        const size_t i = I3(g, x, y, z);
        if (g->boundary[i] == BOUNDARY) continue;
        g->vel[3*i] += g->forces[3*i] * dt;
        g->vel[3*i+1] += g->forces[3*i+1] * dt;
        g->vel[3*i+2] += g->forces[3*i+2] * dt;
        if (g->prm.gravity_enabled) g->vel[3*i+1] -= g->prm.gravity_force * dt;
    }
}

/* R3:478-504 */
static void vel_advect3(orc_grid* g) {
    float* vel = g->vel; float* nv = g->tmpvel; const float* bnd = g->boundary;
    LOOP3(g, 1) {
        const size_t i = I3(g, x, y, z);
        float pp[3]; trace3(g, (float)x, (float)y, (float)z, -g->prm.dt, 4, pp);
        vinterp3(g, vel, pp[0] - 0.5f, pp[1] - 0.5f, pp[2] - 0.5f, &nv[3 * i]);
    }
    LOOP3(g, 1) {
        const size_t i = I3(g, x, y, z);
        const size_t ix = I3(g, x-1, y, z), iy = I3(g, x, y-1, z), iz = I3(g, x, y, z-1);
        if (x == 1 || bnd[i] == BOUNDARY || bnd[ix] == BOUNDARY) vel[3*i] = nv[3*i];
        else vel[3*i] = 0.5f * (nv[3*i] + nv[3*ix]);
        if (y == 1 || bnd[i] == BOUNDARY || bnd[iy] == BOUNDARY) vel[3*i+1] = nv[3*i+1];
        else vel[3*i+1] = 0.5f * (nv[3*i+1] + nv[3*iy+1]);
        if (z == 1 || bnd[i] == BOUNDARY || bnd[iz] == BOUNDARY) vel[3*i+2] = nv[3*i+2];
        else vel[3*i+2] = 0.5f * (nv[3*i+2] + nv[3*iz+2]);
    }
}

/* CPUSimulator3D::enforce_wall_boundaries (R3:657-679) */
static void enforce_walls3(orc_grid* g) {
    float* vel = g->vel; const float* bnd = g->boundary;
    LOOP3(g, 0) {
        if (x == 0 || y == 0 || z == 0) continue;
        const size_t i = I3(g, x, y, z);
        if (bnd[i] == 1.f && vel[3*i] > 0) vel[3*i] = 0.f;
        if (bnd[I3(g, x-1, y, z)] == 1.f && vel[3*i] < 0) vel[3*i] = 0.f;
        if (bnd[i] == 1.f && vel[3*i+1] > 0) vel[3*i+1] = 0.f;
        if (bnd[I3(g, x, y-1, z)] == 1.f && vel[3*i+1] < 0) vel[3*i+1] = 0.f;
        if (bnd[i] == 1.f && vel[3*i+2] > 0) vel[3*i+2] = 0.f;
        if (bnd[I3(g, x, y, z-1)] == 1.f && vel[3*i+2] < 0) vel[3*i+2] = 0.f;
    }
}

/* ------------------------------------------------------------------------------------------------ */
/* pressure solvers (both dimensions)                                                               */
/* ------------------------------------------------------------------------------------------------ */

/* CGSolverCPU3D::impl_mat_mul (CG:467-497) and CGSolverCPU2D::impl_mat_mul (CG:85-111) */
static void matmul(const orc_grid* g, float* res, const float* xf) {
    const float* rho = g->rho; const float* bnd = g->boundary;
    const int W = g->W, H = g->H, D = g->D;
    #pragma omp parallel for collapse(2) schedule(static) if (g->N >= ORC_PAR_MIN)
    for (int z = 0; z < D; z++)
    for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
        const size_t i = (size_t)z * W * H + (size_t)y * W + x;
        if (rho[i] <= 0.5f || bnd[i] == 1) { res[i] = xf[i]; continue; }
        float sum = 0.0f; int cnt = 0;
        const int nbx[6] = {x - 1, x + 1, x, x, x, x};
        const int nby[6] = {y, y, y - 1, y + 1, y, y};
        /* 3D order: x-1, x+1, y-1, y+1, z+1, z-1 (CG:489-494); 2D: x-1, x+1, y-1, y+1 */
        const int nbz[6] = {z, z, z, z, z + 1, z - 1};
        const int nn = (g->dim == 3) ? 6 : 4;
        for (int k = 0; k < nn; k++) {
            const int nx = nbx[k], ny = nby[k], nz = nbz[k];
            if (nx < 0 || nx >= W || ny < 0 || ny >= H || nz < 0 || nz >= D) continue;
            if (nx == 0 || nx == W - 1 || ny == 0 || ny == H - 1) continue;
            if (g->dim == 3 && (nz == 0 || nz == D - 1)) continue;
            const size_t j = (size_t)nz * W * H + (size_t)ny * W + nx;
            if (bnd[j] > 0.5f) continue;
            cnt++;
            if (rho[j] > 0.5f) sum += xf[j];
        }
        res[i] = sum - (float)cnt * xf[i];
    }
}

static float fdot(const orc_grid* g, const float* a, const float* b) {  /* ScalField3D::dot (ScalField3D.h:91-97) */
    float s = 0; for (size_t i = 0; i < g->N; i++) s += a[i] * b[i]; return s;
}
static double ddot(const orc_grid* g, const float* a, const float* b) {
    double s; ORC_BLOCKED_SUM(s, g->N, i, (double)a[i] * (double)b[i]); return s;
}
static double dddot(size_t n, const double* a, const double* b) {
    double s; ORC_BLOCKED_SUM(s, n, i, a[i] * b[i]); return s;
}

/* the solver threshold the step uses (PROPERTY_F(SOLVER_THRESHOLD), or the relative-residual hook) */
static float solver_threshold(orc_grid* g) {
    g->bb = ddot(g, g->div, g->div);
    if (g->prm.tol_rel > 0) {
        float t = (float)((double)g->prm.tol_rel * (double)g->prm.tol_rel * g->bb);
        return t > 0 ? t : FLT_MIN;
    }
    return g->prm.solver_threshold;
}

static void count_active(orc_grid* g) {
    int64_t a = 0;
    for (size_t i = 0; i < g->N; i++) if (g->rho[i] > 0.5f && g->boundary[i] != 1.f) a++;
    g->active = a;
}

/* FP64 masked Laplacian row sums: the same rows as matmul, accumulated in double */
static void matmul_d(const orc_grid* g, double* res, const double* xf);

/* CGSolverCPU3D::solve (CG:416-465) == CGSolverCPU2D::solve (CG:32-83), EFS_CG_REFERENCE */
static float cg_solve_reference(orc_grid* g, float thr) {
    const size_t N = g->N;
    float *t = g->cg_t, *r = g->cg_r, *d = g->cg_d, *p = g->p;
    const float* b = g->div;
    const int fp64 = (g->mode & ORC_DOTS_FP64) != 0;
    const int steps = g->prm.max_steps;
    memset(t, 0, N * 4);
    memcpy(r, b, N * 4);
    memcpy(p, b, N * 4);
    matmul(g, t, p);
    for (size_t i = 0; i < N; i++) r[i] -= t[i];
    memcpy(d, r, N * 4);
    double rr = fp64 ? ddot(g, r, r) : (double)fdot(g, r, r);
    g->rr = rr;
    g->solve_steps = 0;
    if (rr < (double)thr) { g->converged = 1; return (float)rr; }
    int i;
    for (i = 0; i < steps; i++) {
        matmul(g, t, d);
        float alpha;
        if (fp64) alpha = (float)(rr / ddot(g, d, t));
        else alpha = (float)rr / fdot(g, d, t);
        for (size_t c = 0; c < N; c++) p[c] += alpha * d[c];
        if (i & 0x3F) {
            for (size_t c = 0; c < N; c++) r[c] += (-alpha) * t[c];
        } else {
            matmul(g, t, p);
            for (size_t c = 0; c < N; c++) r[c] = b[c] - t[c];
        }
        const double old = rr;
        rr = fp64 ? ddot(g, r, r) : (double)fdot(g, r, r);
        if (rr < (double)thr) break;
        const float beta = fp64 ? (float)(rr / old) : (float)rr / (float)old;
        for (size_t c = 0; c < N; c++) { d[c] *= beta; d[c] += r[c]; }
    }
    g->solve_steps = i + 1;
    g->rr = rr;
    g->converged = rr < (double)thr;
    return (float)rr;
}

/* EFS_CG_MIXED: the same iteration with the pressure held as p64 (FP64) + e (FP32 increment); at every
 * recomputation point ((i & 63) == 0, as CG:444) e is folded into p64 and the residual is recomputed as
 * b - L p64 in FP64; a recurrence residual below the threshold triggers one more recomputation, and the
 * solve stops only if that true residual is below the threshold too. */
static float cg_solve_mixed(orc_grid* g, float thr) {
    const size_t N = g->N;
    float *t = g->cg_t, *r = g->cg_r, *d = g->cg_d, *e = g->jac_tmp;
    const float* b = g->div;
    const int steps = g->prm.max_steps;
    double* p64 = (double*)malloc(N * sizeof(double));
    double* t64 = (double*)malloc(N * sizeof(double));
    double rr;
    #define ORC_REPLACE() do { \
        _Pragma("omp parallel for schedule(static) if (N >= ORC_PAR_MIN)") \
        for (long c = 0; c < (long)N; c++) { p64[c] += (double)e[c]; e[c] = 0.f; } \
        matmul_d(g, t64, p64); \
        _Pragma("omp parallel for schedule(static) if (N >= ORC_PAR_MIN)") \
        for (long c = 0; c < (long)N; c++) r[c] = (float)((double)b[c] - t64[c]); \
        rr = ddot(g, r, r); \
    } while (0)
    for (size_t c = 0; c < N; c++) { p64[c] = (double)b[c]; e[c] = 0.f; }
    ORC_REPLACE();
    memcpy(d, r, N * 4);
    g->solve_steps = 0;
    int conv = rr < (double)thr;
    if (!conv) {
        int i;
        for (i = 0; i < steps; i++) {
            matmul(g, t, d);
            const float alpha = (float)(rr / ddot(g, d, t));
            #pragma omp parallel for schedule(static) if (N >= ORC_PAR_MIN)
            for (long c = 0; c < (long)N; c++) e[c] += alpha * d[c];
            const double old = rr;
            int replaced = 0;
            if (i & 0x3F) {
                #pragma omp parallel for schedule(static) if (N >= ORC_PAR_MIN)
                for (long c = 0; c < (long)N; c++) r[c] += (-alpha) * t[c];
                rr = ddot(g, r, r);
            } else { ORC_REPLACE(); replaced = 1; }
            if (rr < (double)thr) {
                if (!replaced) ORC_REPLACE();
                if (rr < (double)thr) { conv = 1; break; }
            }
            const float beta = (float)(rr / old);
            #pragma omp parallel for schedule(static) if (N >= ORC_PAR_MIN)
            for (long c = 0; c < (long)N; c++) { d[c] *= beta; d[c] += r[c]; }
        }
        g->solve_steps = i + 1;
    }
    #undef ORC_REPLACE
    for (size_t c = 0; c < N; c++) g->p[c] = (float)(p64[c] + (double)e[c]);
    free(p64); free(t64);
    g->rr = rr;
    g->converged = conv;
    if (conv) return (float)rr;
    return ((float)rr > thr) ? (float)rr : nextafterf(thr, INFINITY);
}

/* EFS_CG_MIXED_RECURRENCE: the iteration of cg_solve_mixed with beta from the residual-norm recurrence
 * r'.r' = alpha^2 t.t - r.r, so that d, r and the increment are updated together once t = L d is known; the
 * exact r'.r' is still summed for the stop test.  Every 64th iteration, and any iteration whose recurrence
 * value is not positive, recomputes the residual in FP64 and takes beta from it.  When the stop test is met by the recurrence residual but not by the recomputed one, the
 * search direction restarts from the recomputed residual.  A non-finite alpha (a singular block) stops the
 * solve, not converged. */
static float cg_solve_mixed_recurrence(orc_grid* g, float thr) {
    const size_t N = g->N;
    float *t = g->cg_t, *r = g->cg_r, *d = g->cg_d, *e = g->jac_tmp;
    const float* b = g->div;
    const int steps = g->prm.max_steps;
    double* p64 = (double*)malloc(N * sizeof(double));
    double* t64 = (double*)malloc(N * sizeof(double));
    double rr;
    #define ORC_REPLACE() do { \
        _Pragma("omp parallel for schedule(static) if (N >= ORC_PAR_MIN)") \
        for (long c = 0; c < (long)N; c++) { p64[c] += (double)e[c]; e[c] = 0.f; } \
        matmul_d(g, t64, p64); \
        _Pragma("omp parallel for schedule(static) if (N >= ORC_PAR_MIN)") \
        for (long c = 0; c < (long)N; c++) r[c] = (float)((double)b[c] - t64[c]); \
        rr = ddot(g, r, r); \
    } while (0)
    for (size_t c = 0; c < N; c++) { p64[c] = (double)b[c]; e[c] = 0.f; }
    ORC_REPLACE();
    memcpy(d, r, N * 4);
    g->solve_steps = 0;
    int conv = rr < (double)thr;
    if (!conv) {
        int i;
        for (i = 0; i < steps; i++) {
            matmul(g, t, d);
            const double dt = ddot(g, d, t), tt = ddot(g, t, t);
            if (!(dt != 0.0) || !isfinite(rr / dt)) break;   /* breakdown: stop, not converged */
            const double ad = rr / dt;
            const float alpha = (float)ad;
            const double old = rr;
            const double est = ad * ad * tt - old;            /* r'.r' from the CG recurrence */
            int replaced = 0;
            if ((i & 0x3F) && est > 0.0) {
                const float beta = (float)(est / old);
                #pragma omp parallel for schedule(static) if (N >= ORC_PAR_MIN)
                for (long c = 0; c < (long)N; c++) {
                    e[c] += alpha * d[c];
                    const float rn = r[c] + (-alpha) * t[c];
                    r[c] = rn;
                    d[c] = d[c] * beta + rn;
                }
                rr = ddot(g, r, r);
            } else {
                #pragma omp parallel for schedule(static) if (N >= ORC_PAR_MIN)
                for (long c = 0; c < (long)N; c++) e[c] += alpha * d[c];
                ORC_REPLACE();
                replaced = 1;
                const float beta = (float)(rr / old);
                #pragma omp parallel for schedule(static) if (N >= ORC_PAR_MIN)
                for (long c = 0; c < (long)N; c++) d[c] = d[c] * beta + r[c];
            }
            if (rr < (double)thr) {
                if (!replaced) {
                    ORC_REPLACE();
                    /* d was formed from the recurrence residual; after the replacement r.d != r.r, so the
                     * direction restarts from the true residual */
                    if (!(rr < (double)thr)) memcpy(d, r, N * 4);
                }
                if (rr < (double)thr) { conv = 1; break; }
            }
        }
        g->solve_steps = i + 1;
    }
    #undef ORC_REPLACE
    for (size_t c = 0; c < N; c++) g->p[c] = (float)(p64[c] + (double)e[c]);
    free(p64); free(t64);
    g->rr = rr;
    g->converged = conv;
    if (conv) return (float)rr;
    return ((float)rr > thr) ? (float)rr : nextafterf(thr, INFINITY);
}

/* EFS_CG_PIPELINED: pipelined CG (P. Ghysels and W. Vanroose, Parallel Computing 40, 2014, Alg. 4) on the same
 * matrix and start (p0 = b), with the pressure held as p64 + e as in cg_solve_mixed.  Auxiliary vectors
 * w = L r, s = L p, z = L s are carried by recurrences, so that one sweep per iteration computes q = L w and
 * updates z, s, p, e, r, w, and the two dot products gamma = r.r and delta = w.r of the next iteration:
 *   beta = gamma / gamma_old, alpha = gamma / (delta - beta gamma / alpha_old)   (beta = 0 at a restart)
 *   z = q + beta z; s = w + beta s; p = r + beta p; e += alpha p; r -= alpha s; w -= alpha z.
 * Every 64th iteration, and before stopping, the residual is recomputed in FP64 from p64 and w, s, z are
 * recomputed from r and p (residual replacement, S. Cools et al., SIAM J. Sci. Comput. 40, 2018); a stop test
 * that the recomputed residual does not confirm restarts the recurrences (beta = 0). */
static float cg_solve_pipelined(orc_grid* g, float thr) {
    const size_t N = g->N;
    float *r = g->cg_r, *e = g->jac_tmp;
    const float* b = g->div;
    const int steps = g->prm.max_steps;
    float* w = (float*)calloc(N, 4);
    float* p = (float*)calloc(N, 4);
    float* s = (float*)calloc(N, 4);
    float* z = (float*)calloc(N, 4);
    float* q = (float*)calloc(N, 4);
    double* p64 = (double*)malloc(N * sizeof(double));
    double* t64 = (double*)malloc(N * sizeof(double));
    double gamma = 0, delta = 0;
    #define ORC_PREPLACE() do { \
        for (size_t c = 0; c < N; c++) { p64[c] += (double)e[c]; e[c] = 0.f; } \
        matmul_d(g, t64, p64); \
        for (size_t c = 0; c < N; c++) r[c] = (float)((double)b[c] - t64[c]); \
        matmul(g, w, r); matmul(g, s, p); matmul(g, z, s); \
        gamma = ddot(g, r, r); delta = ddot(g, w, r); \
    } while (0)
    for (size_t c = 0; c < N; c++) { p64[c] = (double)b[c]; e[c] = 0.f; }
    ORC_PREPLACE();
    g->solve_steps = 0;
    int conv = gamma < (double)thr;
    if (!conv) {
        int i, restart = 1;
        double gamma_old = 0, alpha_old = 0;
        for (i = 0; i < steps; i++) {
            double alpha, beta;
            if (restart) { beta = 0.0; alpha = gamma / delta; }
            else { beta = gamma / gamma_old; alpha = gamma / (delta - beta * gamma / alpha_old); }
            if (!isfinite(alpha) || alpha == 0.0) break;    /* breakdown: stop, not converged */
            const float a = (float)alpha, bt = (float)beta;
            matmul(g, q, w);
            for (size_t c = 0; c < N; c++) {
                z[c] = q[c] + bt * z[c];
                s[c] = w[c] + bt * s[c];
                p[c] = r[c] + bt * p[c];
                e[c] += a * p[c];
                r[c] = r[c] + (-a) * s[c];
                w[c] = w[c] + (-a) * z[c];
            }
            gamma_old = gamma; alpha_old = alpha; restart = 0;
            gamma = ddot(g, r, r); delta = ddot(g, w, r);
            int replaced = 0;
            if (((i + 1) & 0x1F) == 0) { ORC_PREPLACE(); replaced = 1; }
            if (gamma < (double)thr) {
                if (!replaced) ORC_PREPLACE();
                if (gamma < (double)thr) { conv = 1; break; }
                restart = 1;
            }
        }
        g->solve_steps = i + 1 > steps ? steps : i + 1;
    }
    #undef ORC_PREPLACE
    for (size_t c = 0; c < N; c++) g->p[c] = (float)(p64[c] + (double)e[c]);
    free(w); free(p); free(s); free(z); free(q); free(p64); free(t64);
    g->rr = gamma;
    g->converged = conv;
    if (conv) return (float)gamma;
    return ((float)gamma > thr) ? (float)gamma : nextafterf(thr, INFINITY);
}

static float cg_solve(orc_grid* g, float thr) {
    if (g->prm.cg_variant == EFS_CG_REFERENCE) return cg_solve_reference(g, thr);
    if (g->prm.cg_variant == EFS_CG_PIPELINED) return cg_solve_pipelined(g, thr);
    if (g->prm.cg_variant == EFS_CG_MIXED_RECURRENCE) return cg_solve_mixed_recurrence(g, thr);
    return cg_solve_mixed(g, thr);
}

/* JacobiSolverCPU3D::solve (JS:154-212) == JacobiSolverCPU2D::solve (JS:18-71): returns 0 */
static float jacobi_solve(orc_grid* g) {
    const int iters = g->prm.max_steps / 2;
    const float* rho = g->rho; const float* bnd = g->boundary; const float* b = g->div;
    const int W = g->W, H = g->H, D = g->D;
    for (int it = 0; it < iters; it++) {
        float* p = g->p; float* tmp = g->jac_tmp;
        #pragma omp parallel for collapse(2) schedule(static) if (g->N >= ORC_PAR_MIN)
        for (int z = 0; z < D; z++)
        for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const size_t i = (size_t)z * W * H + (size_t)y * W + x;
            if (rho[i] <= 0.5f || bnd[i] >= 0.5f) { tmp[i] = p[i]; continue; }
            float sum = 0.0f; int cnt = 0;
            const int nbx[6] = {x - 1, x + 1, x, x, x, x};
            const int nby[6] = {y, y, y - 1, y + 1, y, y};
            const int nbz[6] = {z, z, z, z, z - 1, z + 1};   /* JS:189-194 order */
            const int nn = (g->dim == 3) ? 6 : 4;
            for (int k = 0; k < nn; k++) {
                const int nx = nbx[k], ny = nby[k], nz = nbz[k];
                if (nx < 0 || nx >= W || ny < 0 || ny >= H || nz < 0 || nz >= D) continue;
                if (nx == 0 || nx == W - 1 || ny == 0 || ny == H - 1) continue;
                if (g->dim == 3 && (nz == 0 || nz == D - 1)) continue;
                const size_t j = (size_t)nz * W * H + (size_t)ny * W + nx;
                if (bnd[j] > 0.5f) continue;
                cnt++;
                if (rho[j] > 0.5f) sum += p[j];
            }
            tmp[i] = cnt > 0 ? (sum - b[i]) / (float)cnt : 0.0f;
        }
        g->jac_tmp = p; g->p = tmp;   /* std::swap(p, tmp) exchanges the contents */
    }
    g->solve_steps = iters;
    g->converged = 1;
    g->rr = 0;
    return 0;
}

static float run_solver(orc_grid* g, float thr) {
    count_active(g);
    float err = (g->prm.solver == EFS_SOLVER_JACOBI) ? jacobi_solve(g) : cg_solve(g, thr);
    g->total_solve_steps += g->solve_steps;
    g->solves++;
    return err;
}

float orc_solve(orc_grid* g) {
    g->thr = solver_threshold(g);
    return run_solver(g, (float)g->thr);
}

/* CPUSimulator3D::project (R3:506-566) */
static void project3(orc_grid* g) {
    float* vel = g->vel; const float* rho = g->rho; const float* bnd = g->boundary;
    memset(g->p, 0, g->N * 4);
    memset(g->div, 0, g->N * 4);
    enforce_walls3(g);
    const float thrL = g->prm.liquid_threshold, lp = g->prm.lambda_plus, lm = g->prm.lambda_minus, eta = g->prm.eta;
    LOOP3(g, 1) {
        const size_t i = I3(g, x, y, z);
        if (rho[i] < thrL) continue;
        if (bnd[i] == BOUNDARY) continue;
        const float dx = vel[3 * I3(g, x+1, y, z)] - vel[3*i];
        const float dy = vel[3 * I3(g, x, y+1, z) + 1] - vel[3*i+1];
        const float dz = vel[3 * I3(g, x, y, z+1) + 2] - vel[3*i+2];
        g->div[i] = dx + dy + dz;
        if (rho[i] > 1.f) g->div[i] -= minf(lm * (rho[i] - 1.f), eta);
        if (rho[i] < 1.f) g->div[i] += minf(lp * (1.f - rho[i]), eta);
    }
    const float thr = solver_threshold(g);
    g->thr = thr;
    const float err = run_solver(g, thr);
    if (err > thr) { g->paused = 1; return; }
    const float* p = g->p;
    LOOP3(g, 1) {
        const size_t i = I3(g, x, y, z);
        if (bnd[i] == BOUNDARY) continue;
        float gx = 0, gy = 0, gz = 0;
        if (x > 1) gx = p[i] - p[I3(g, x-1, y, z)];
        if (y > 1) gy = p[i] - p[I3(g, x, y-1, z)];
        if (z > 1) gz = p[i] - p[I3(g, x, y, z-1)];
        vel[3*i] -= gx; vel[3*i+1] -= gy; vel[3*i+2] -= gz;
    }
    enforce_walls3(g);
}

/* ------------------------------------------------------------------------------------------------ */
/* 2D                                                                                                */
/* ------------------------------------------------------------------------------------------------ */

#define LOOP2(g, off) for (int y = (off); y < (g)->H - (off); y++) \
                      for (int x = (off); x < (g)->W - (off); x++)

/* VecField2D::bilinear_interpolation / interpolate (V2:26-63) */
static const float OFF2[2][2] = {{-1.0f, -0.5f}, {-0.5f, -1.0f}};
static void vinterp2(const orc_grid* g, const float* vel, float px, float py, float out[2]) {
    for (int c = 0; c < 2; c++) {
        const int lx = (int)(floorf(px - OFF2[c][0]) + 1.0e-10f);
        const int ly = (int)(floorf(py - OFF2[c][1]) + 1.0e-10f);
        const float x0 = (float)lx + OFF2[c][0], y0 = (float)ly + OFF2[c][1];
        const float tx = px - x0, ty = py - y0;
        const float v00 = vel[2 * I2(g, lx, ly) + c];
        const float v01 = vel[2 * I2(g, lx, ly + 1) + c];
        const float v10 = vel[2 * I2(g, lx + 1, ly) + c];
        const float v11 = vel[2 * I2(g, lx + 1, ly + 1) + c];
        const float vLow = v00 * (1.0f - ty) + v01 * ty;
        const float vHigh = v10 * (1.0f - ty) + v11 * ty;
        out[c] = vLow * (1.0f - tx) + vHigh * tx;
    }
}

/* ScalField2D::interpolate (S2:20-69), including its pos += 1 shift */
static float sinterp2(const orc_grid* g, const float* f, float px, float py) {
    px += 1.f; py += 1.f;
    const int x = (int)px, y = (int)py;
    int ix1 = x, ix2 = x + 1;
    if (px - (float)x < 0.5f) { ix1 = x - 1; ix2 = x; }
    int iy1 = y, iy2 = y + 1;
    if (py - (float)y < 0.5f) { iy1 = y - 1; iy2 = y; }
    ix1 = clampi(ix1, 0, g->W - 1); ix2 = clampi(ix2, 0, g->W - 1);
    iy1 = clampi(iy1, 0, g->H - 1); iy2 = clampi(iy2, 0, g->H - 1);
    const float v[4] = {f[I2(g, ix1, iy1)], f[I2(g, ix1, iy2)], f[I2(g, ix2, iy1)], f[I2(g, ix2, iy2)]};
    const float x1 = (float)ix1 + 0.5f, x2 = (float)ix2 + 0.5f, y1 = (float)iy1 + 0.5f, y2 = (float)iy2 + 0.5f;
    const float dx2x1 = x2 - x1;
    float fxy1 = ((x2 - px) / dx2x1) * v[0] + ((px - x1) / dx2x1) * v[2];
    float fxy2 = ((x2 - px) / dx2x1) * v[1] + ((px - x1) / dx2x1) * v[3];
    if ((double)dx2x1 < 1e-9) { fxy1 = v[1]; fxy2 = v[3]; }
    const float dy2y1 = y2 - y1;
    float fxy = ((y2 - py) / dy2y1) * fxy1 + ((py - y1) / dy2y1) * fxy2;
    if ((double)dy2y1 < 1e-9) fxy = fxy1;
    return fxy;
}

/* Grid2D::traceParticle (G2:84-137) */
static int inwall2(const orc_grid* g, float px, float py) {
    const float W = (float)g->W, H = (float)g->H;
    if (px < 1.f || px > W - 2.f || py < 1.f || py > H - 2.f) return 1;
    const int ix = clampi((int)px, 0, g->W - 1), iy = clampi((int)py, 0, g->H - 1);
    return g->boundary[I2(g, ix, iy)] > 0.5f;
}
static void trace2(const orc_grid* g, float sx, float sy, float dt, int substeps, float out[2]) {
    const float W = (float)g->W, H = (float)g->H;
    out[0] = sx; out[1] = sy;
    if (inwall2(g, sx, sy)) return;
    const float subDt = dt / (float)substeps;
    float p[2] = {sx, sy};
    for (int s = 0; s < substeps; s++) {
        float k1[2], k2[2], mid[2], nx[2];
        vinterp2(g, g->vel, p[0] - 0.5f, p[1] - 0.5f, k1);
        const float h = subDt * 0.5f;
        mid[0] = clampf(p[0] + k1[0] * h, 1.f, W - 2.f);
        mid[1] = clampf(p[1] + k1[1] * h, 1.f, H - 2.f);
        vinterp2(g, g->vel, mid[0] - 0.5f, mid[1] - 0.5f, k2);
        nx[0] = p[0] + k2[0] * subDt; nx[1] = p[1] + k2[1] * subDt;
        if (inwall2(g, nx[0], nx[1])) {
            float safe[2] = {p[0], p[1]}, unsafe[2] = {nx[0], nx[1]};
            for (int b = 0; b < 8; b++) {
                float hw[2] = {(safe[0] + unsafe[0]) * 0.5f, (safe[1] + unsafe[1]) * 0.5f};
                if (inwall2(g, hw[0], hw[1])) { unsafe[0] = hw[0]; unsafe[1] = hw[1]; }
                else { safe[0] = hw[0]; safe[1] = hw[1]; }
            }
            out[0] = safe[0]; out[1] = safe[1];
            return;
        }
        p[0] = nx[0]; p[1] = nx[1];
    }
    out[0] = p[0]; out[1] = p[1];
}

/* R2:65-70 */
static void vel_decay2(orc_grid* g) {
    const float k = g->prm.vel_decay;
    LOOP2(g, 1) { size_t i = I2(g, x, y); if ((double)g->rho[i] < 0.5) { g->vel[2*i] *= k; g->vel[2*i+1] *= k; } }
}

/* R2:72-120 */
static void vel_extrapolate2(orc_grid* g) {
    float* validA = zalloc(g->N); float* validB = zalloc(g->N);
    LOOP2(g, 1) { size_t i = I2(g, x, y); validA[i] = (g->rho[i] >= 0.5f && g->boundary[i] != BOUNDARY) ? 1.f : 0.f; }
    for (int it = 0; it < 6; it++) {
        float* sv = (it & 1) ? g->tmpvel : g->vel; float* sV = (it & 1) ? validB : validA;
        float* dv = (it & 1) ? g->vel : g->tmpvel; float* dV = (it & 1) ? validA : validB;
        LOOP2(g, 1) {
            size_t i = I2(g, x, y);
            if (g->boundary[i] == BOUNDARY) { dv[2*i] = sv[2*i]; dv[2*i+1] = sv[2*i+1]; dV[i] = 0.f; continue; }
            if (sV[i] > 0.5f) { dv[2*i] = sv[2*i]; dv[2*i+1] = sv[2*i+1]; dV[i] = 1.f; continue; }
            float s0 = 0.f, s1 = 0.f, n = 0;
            const size_t nb[4] = {I2(g, x-1, y), I2(g, x+1, y), I2(g, x, y-1), I2(g, x, y+1)};
            for (int k = 0; k < 4; k++) if (sV[nb[k]] > 0.5f) { s0 += sv[2*nb[k]]; s1 += sv[2*nb[k]+1]; n++; }
            if (n > 0) { dv[2*i] = s0 / n; dv[2*i+1] = s1 / n; } else { dv[2*i] = sv[2*i]; dv[2*i+1] = sv[2*i+1]; }
            dV[i] = (n > 0) ? 1.f : 0.f;
        }
    }
    free(validA); free(validB);
}

static float corner_weights2(const orc_grid* g, const float pos[2], int p0[2], float m[4]) {
    p0[0] = (int)floorf(pos[0]); p0[1] = (int)floorf(pos[1]);
    const float dx0 = 1 - (pos[0] - (float)p0[0]), dy0 = 1 - (pos[1] - (float)p0[1]);
    const float dx1 = 1 - ((float)(p0[0] + 1) - pos[0]), dy1 = 1 - ((float)(p0[1] + 1) - pos[1]);
    m[0] = m[1] = m[2] = m[3] = 0;
    if (g->boundary[I2(g, p0[0], p0[1])] != BOUNDARY) m[0] = dx0 * dy0;
    if (g->boundary[I2(g, p0[0] + 1, p0[1])] != BOUNDARY) m[1] = dx1 * dy0;
    if (g->boundary[I2(g, p0[0], p0[1] + 1)] != BOUNDARY) m[2] = dx0 * dy1;
    if (g->boundary[I2(g, p0[0] + 1, p0[1] + 1)] != BOUNDARY) m[3] = dx1 * dy1;
    return m[0] + m[1] + m[2] + m[3];
}

static void add_forward2(orc_grid* g, int32_t i, int32_t j, float val) {
    const int32_t b = g->bbase[i];
    if (b >= 0) {
        const long dy = (long)(j / g->W) - (long)(b / g->W), dx = (long)(j % g->W) - (long)(b % g->W);
        if (dx >= 0 && dx <= 1 && dy >= 0 && dy <= 1) { g->wb[(size_t)i * 4 + (dx + 2 * dy)] += val; return; }
    }
    fent_push(g, i, j, val);
}

#define FOR_ENTRIES2(g, BODY) do { \
    const size_t W_ = (g)->W; \
    const int rev_ = ((g)->mode & ORC_REVERSE_SUMS) != 0; \
    if (rev_) for (size_t e2_ = (g)->nf; e2_-- > 0;) { const size_t ci = (size_t)(g)->fent[e2_].i, cj = (size_t)(g)->fent[e2_].j; \
        float* cv = &(g)->fent[e2_].val; (void)ci; (void)cj; BODY } \
    for (size_t t_ = 0; t_ < (g)->N; t_++) { const size_t i_ = rev_ ? (g)->N - 1 - t_ : t_; \
        const int32_t b_ = (g)->bbase[i_]; if (b_ < 0) continue; \
        for (int q_ = 0; q_ < 4; q_++) { const int k_ = rev_ ? 3 - q_ : q_; const size_t ci = i_; \
            const size_t cj = (size_t)b_ + (k_ & 1) + ((k_ >> 1) & 1) * W_; \
            float* cv = &(g)->wb[i_ * 4 + k_]; (void)ci; (void)cj; BODY } } \
    if (!rev_) for (size_t e_ = 0; e_ < (g)->nf; e_++) { const size_t ci = (size_t)(g)->fent[e_].i, cj = (size_t)(g)->fent[e_].j; \
        float* cv = &(g)->fent[e_].val; (void)ci; (void)cj; BODY } } while (0)

/* R2:122-318 */
static void rho_advect2(orc_grid* g) {
    float* rho = g->rho; float* gamma = g->gamma; float* beta = g->beta; const float* bnd = g->boundary;
    const float dt = g->prm.dt;
    float* advG = zalloc(g->N);
    LOOP2(g, 1) {
        size_t i = I2(g, x, y);
        if (bnd[i] == BOUNDARY) continue;
        float pp[2]; trace2(g, (float)x, (float)y, -dt, 4, pp);
        advG[i] = sinterp2(g, gamma, pp[0], pp[1]);
    }
    memcpy(gamma, advG, g->N * 4); free(advG);
    for (size_t i = 0; i < g->N; i++) g->bbase[i] = -1;
    g->nf = 0;
    LOOP2(g, 1) {
        size_t i = I2(g, x, y);
        float pp[2]; trace2(g, (float)x, (float)y, -dt, 4, pp);
        int p0[2]; float m[4];
        const float sum = corner_weights2(g, pp, p0, m);
        if (sum == 0) continue;
        g->bbase[i] = (int32_t)I2(g, p0[0], p0[1]);
        for (int k = 0; k < 4; k++) g->wb[i * 4 + k] = m[k] / sum;
    }
    FOR_ENTRIES2(g, { if (gamma[ci] > 1.e-5f) *cv /= gamma[ci]; });
    memset(beta, 0, g->N * 4);
    FOR_ENTRIES2(g, { beta[cj] += *cv; });
    LOOP2(g, 1) {
        const size_t j = I2(g, x, y);
        if (beta[j] >= 1) continue;
        float pp[2]; trace2(g, (float)x, (float)y, +dt, 4, pp);
        int p0[2]; float m[4];
        const float sum = corner_weights2(g, pp, p0, m);
        if (sum == 0) continue;
        for (int k = 0; k < 4; k++) {
            const int32_t ti = (int32_t)I2(g, p0[0] + (k & 1), p0[1] + ((k >> 1) & 1));
            add_forward2(g, ti, (int32_t)j, (1 - beta[j]) * (m[k] / sum));
        }
    }
    memset(gamma, 0, g->N * 4);
    FOR_ENTRIES2(g, { gamma[ci] += *cv; });
    FOR_ENTRIES2(g, { if (gamma[ci] > 1.e-5f) *cv /= gamma[ci]; });
    memset(beta, 0, g->N * 4);
    FOR_ENTRIES2(g, { beta[cj] += *cv; });
    FOR_ENTRIES2(g, { if (beta[cj] > 1.e-5f) *cv /= beta[cj]; });
    memset(gamma, 0, g->N * 4);
    FOR_ENTRIES2(g, { gamma[ci] += *cv; });
    float* adv = g->tmps;
    memset(adv, 0, g->N * 4);
    FOR_ENTRIES2(g, { adv[ci] += *cv * rho[cj]; });
    LOOP2(g, 1) { size_t i = I2(g, x, y); rho[i] = adv[i]; }
    /* Step 12 (R2:259-317): 7 iterations of x then y sweeps */
    for (int it = 0; it < 7; it++) {
        for (int dirn = 0; dirn < 2; dirn++) {
            const int na = (dirn == 0) ? g->H : g->W, nc = (dirn == 0) ? g->W : g->H;
            for (int a = 1; a < na - 1; a++)
            for (int c = 2; c < nc - 1; c++) {
                size_t ii, jj;
                if (dirn == 0) { ii = I2(g, c, a); jj = I2(g, c - 1, a); }
                else { ii = I2(g, a, c); jj = I2(g, a, c - 1); }
                const float g_j = gamma[jj], g_i = gamma[ii];
                if (bnd[ii] == BOUNDARY || bnd[jj] == BOUNDARY) continue;
                if (g_j < 1e-5f || g_i < 1e-5f) continue;
                if (g_j == g_i) continue;
                const float avg = (g_j + g_i) / 2.f;
                if (g_j > g_i) { const float dif = rho[jj] * (g_j - g_i) / (2.f * g_j); rho[jj] -= dif; rho[ii] += dif; }
                else { const float dif = rho[ii] * (g_i - g_j) / (2.f * g_i); rho[ii] -= dif; rho[jj] += dif; }
                gamma[jj] = avg; gamma[ii] = avg;
            }
        }
    }
}

/* R2:526-562 */
static void trace_field2(const orc_grid* g, float sx, float sy, float Dist, int substeps, float out[2]) {
    const float stepSize = Dist / (float)substeps;
    const float* rho = g->rho;
    float p[2] = {sx, sy};
    for (int s = 0; s < substeps; s++) {
        if (sinterp2(g, rho, p[0], p[1]) >= 0.5f) break;
        const int ix = clampi((int)p[0], 1, g->W - 2), iy = clampi((int)p[1], 1, g->H - 2);
        const float gx = rho[I2(g, ix + 1, iy)] - rho[I2(g, ix - 1, iy)];
        const float gy = rho[I2(g, ix, iy + 1)] - rho[I2(g, ix, iy - 1)];
        const float len = sqrtf(gx * gx + gy * gy);
        if (len < 1e-6f) break;
        float nx = p[0] + (gx / len) * stepSize, ny = p[1] + (gy / len) * stepSize;
        nx = clampf(nx, 1.f, (float)g->W - 2.f); ny = clampf(ny, 1.f, (float)g->H - 2.f);
        if (g->boundary[I2(g, (size_t)nx, (size_t)ny)] > 0.5f) break;
        p[0] = nx; p[1] = ny;
    }
    out[0] = p[0]; out[1] = p[1];
}

/* R2:564-595 */
static void scatter2(orc_grid* g, const float pos[2], float value) {
    float* rho = g->rho; const float* bnd = g->boundary;
    const int x0 = clampi((int)pos[0], 0, g->W - 1), y0 = clampi((int)pos[1], 0, g->H - 1);
    const int x1 = clampi((int)pos[0] + 1, 0, g->W - 1), y1 = clampi((int)pos[1] + 1, 0, g->H - 1);
    const float fx = pos[0] - (float)(int)pos[0], fy = pos[1] - (float)(int)pos[1];
    float w00 = (1.f - fx) * (1.f - fy), w10 = fx * (1.f - fy), w01 = (1.f - fx) * fy, w11 = fx * fy;
    if (bnd[I2(g, x0, y0)] > 0.5f) w00 = 0.f;
    if (bnd[I2(g, x1, y0)] > 0.5f) w10 = 0.f;
    if (bnd[I2(g, x0, y1)] > 0.5f) w01 = 0.f;
    if (bnd[I2(g, x1, y1)] > 0.5f) w11 = 0.f;
    const float total = w00 + w10 + w01 + w11;
    if (total < 1e-6f) return;
    const float inv = 1.f / total;
    rho[I2(g, x0, y0)] += value * w00 * inv;
    rho[I2(g, x1, y0)] += value * w10 * inv;
    rho[I2(g, x0, y1)] += value * w01 * inv;
    rho[I2(g, x1, y1)] += value * w11 * inv;
}

/* R2:320-402 */
static void rho_sharpen2(orc_grid* g) {
    float* rho = g->rho;
    const float delT = g->prm.dt * 3;
    float* del_rho = zalloc(g->N);
    LOOP2(g, 1) {
        const size_t i = I2(g, x, y);
        const float r = rho[i];
        const float rxm = rho[I2(g, x-1, y)], rxp = rho[I2(g, x+1, y)], rym = rho[I2(g, x, y-1)], ryp = rho[I2(g, x, y+1)];
        const float dpx = -(r - rxm) * delT, dmx = -(rxp - r) * delT, dpy = -(r - rym) * delT, dmy = -(ryp - r) * delT;
        const float max_inc = (float)sqrt(maxd(sq_d(maxf(dpx, 0.f)), sq_d(minf(dmx, 0.f))) +
                                          maxd(sq_d(maxf(dpy, 0.f)), sq_d(minf(dmy, 0.f))));
        const float max_dec = (float)sqrt(maxd(sq_d(minf(dpx, 0.f)), sq_d(maxf(dmx, 0.f))) +
                                          maxd(sq_d(minf(dpy, 0.f)), sq_d(maxf(dmy, 0.f))));
        float mx = -INFINITY;
        mx = maxf(mx, fabsf(r - rxm)); mx = maxf(mx, fabsf(r - rxp)); mx = maxf(mx, fabsf(r - rym)); mx = maxf(mx, fabsf(r - ryp));
        const float w = powf(r - 0.5f, 3.f) * (1 - minf(1.f, mx / 0.2f));
        float dr = (w >= 0) ? w * max_inc : w * max_dec;
        if (r + dr < 0 || (double)r < 1e-5) dr = -r;
        else if (r > 0.5f) dr = 0;
        del_rho[i] = dr;
    }
    if (!(g->mode & ORC_SHARPEN_PARALLEL)) {
        LOOP2(g, 1) {
            const size_t i = I2(g, x, y);
            const float dr = del_rho[i];
            if (fabsf(dr) < 1e-6f) continue;
            rho[i] += dr; rho[i] = maxf(rho[i], 0.f);
            float pp[2]; trace_field2(g, (float)x, (float)y, g->prm.rho_d, 10, pp);
            scatter2(g, pp, -dr);
        }
    } else {
        float* ends = (float*)malloc(g->N * 2 * sizeof(float));
        LOOP2(g, 1) { const size_t i = I2(g, x, y); if (fabsf(del_rho[i]) < 1e-6f) continue; rho[i] += del_rho[i]; rho[i] = maxf(rho[i], 0.f); }
        LOOP2(g, 1) { const size_t i = I2(g, x, y); if (fabsf(del_rho[i]) < 1e-6f) continue; trace_field2(g, (float)x, (float)y, g->prm.rho_d, 10, &ends[2*i]); }
        LOOP2(g, 1) { const size_t i = I2(g, x, y); if (fabsf(del_rho[i]) < 1e-6f) continue; scatter2(g, &ends[2*i], -del_rho[i]); }
        free(ends);
    }
    free(del_rho);
}

/* R2:404-425 (face based) */
static void add_force2(orc_grid* g) {
    const float dt = g->prm.dt; const float* bnd = g->boundary; float* vel = g->vel;
    LOOP2(g, 1) {
        const size_t i = I2(g, x, y);
        if (bnd[i] != BOUNDARY || bnd[I2(g, x-1, y)] != BOUNDARY) vel[2*i] += g->forces[2*i] * dt;
        else vel[2*i] = 0.f;
        if (bnd[i] != BOUNDARY || bnd[I2(g, x, y-1)] != BOUNDARY) {
            vel[2*i+1] += g->forces[2*i+1] * dt;
            if (g->prm.gravity_enabled) vel[2*i+1] -= g->prm.gravity_force * dt;
        } else vel[2*i+1] = 0.f;
    }
}

/* R2:427-448 */
static void vel_advect2(orc_grid* g) {
    float* vel = g->vel; float* nv = g->tmpvel; const float* bnd = g->boundary;
    LOOP2(g, 1) {
        const size_t i = I2(g, x, y);
        float pp[2]; trace2(g, (float)x, (float)y, -g->prm.dt, 4, pp);
        vinterp2(g, vel, pp[0] - 0.5f, pp[1] - 0.5f, &nv[2 * i]);
    }
    LOOP2(g, 1) {
        const size_t i = I2(g, x, y), ix = I2(g, x-1, y), iy = I2(g, x, y-1);
        if (x == 1 || bnd[i] == BOUNDARY || bnd[ix] == BOUNDARY) vel[2*i] = nv[2*i];
        else vel[2*i] = 0.5f * (nv[2*i] + nv[2*ix]);
        if (y == 1 || bnd[i] == BOUNDARY || bnd[iy] == BOUNDARY) vel[2*i+1] = nv[2*i+1];
        else vel[2*i+1] = 0.5f * (nv[2*i+1] + nv[2*iy+1]);
    }
}

/* R2:597-607 */
static void enforce_walls2(orc_grid* g) {
    float* vel = g->vel; const float* bnd = g->boundary;
    LOOP2(g, 0) {
        const size_t i = I2(g, x, y);
        if (bnd[i] == BOUNDARY || (x > 0 && bnd[I2(g, x-1, y)] == BOUNDARY)) vel[2*i] = 0.f;
        if (bnd[i] == BOUNDARY || (y > 0 && bnd[I2(g, x, y-1)] == BOUNDARY)) vel[2*i+1] = 0.f;
    }
}

static void divergence2(orc_grid* g) {
    const float* vel = g->vel; const float* rho = g->rho; const float* bnd = g->boundary;
    const float thrL = g->prm.liquid_threshold, lp = g->prm.lambda_plus, lm = g->prm.lambda_minus, eta = g->prm.eta;
    LOOP2(g, 1) {
        const size_t i = I2(g, x, y);
        if (rho[i] < thrL) continue;
        if (bnd[i] == 1) continue;
        const float dx = vel[2 * I2(g, x+1, y)] - vel[2*i];
        const float dy = vel[2 * I2(g, x, y+1) + 1] - vel[2*i+1];
        g->div[i] = dx + dy;
        if (rho[i] > 1.f) g->div[i] -= minf(lm * (rho[i] - 1.f), eta);
        if (rho[i] < 1.f) g->div[i] += minf(lp * (1.f - rho[i]), eta);
    }
}

/* R2:450-524 */
static void project2(orc_grid* g) {
    float* vel = g->vel; const float* bnd = g->boundary;
    memset(g->p, 0, g->N * 4);
    memset(g->div, 0, g->N * 4);
    enforce_walls2(g);
    divergence2(g);
    const float thr = solver_threshold(g);
    g->thr = thr;
    const float err = run_solver(g, thr);
    if (err > thr) { g->paused = 1; return; }
    const float* p = g->p;
    LOOP2(g, 1) {
        const size_t i = I2(g, x, y);
        if (bnd[i] != BOUNDARY && bnd[I2(g, x-1, y)] != BOUNDARY) vel[2*i] -= (p[i] - p[I2(g, x-1, y)]);
        else vel[2*i] = 0.f;
        if (bnd[i] != BOUNDARY && bnd[I2(g, x, y-1)] != BOUNDARY) vel[2*i+1] -= (p[i] - p[I2(g, x, y-1)]);
        else vel[2*i+1] = 0.f;
    }
    if (g->prm.re_calc_div) divergence2(g);
    enforce_walls2(g);
}

/* ------------------------------------------------------------------------------------------------ */
/* dispatch                                                                                          */
/* ------------------------------------------------------------------------------------------------ */

void orc_stage(orc_grid* g, int s) {
    if (g->dim == 3) {
        switch (s) {
            case EFS_STAGE_VEL_DECAY: vel_decay3(g); break;
            case EFS_STAGE_VEL_EXTRAPOLATE: vel_extrapolate3(g); break;
            case EFS_STAGE_RHO_SHARPEN: rho_sharpen3(g); break;
            case EFS_STAGE_RHO_ADVECT: rho_advect3(g); break;
            case EFS_STAGE_VEL_ADVECT: vel_advect3(g); break;
            case EFS_STAGE_ADD_FORCE: add_force3(g); break;
            case EFS_STAGE_PROJECT: project3(g); break;
            default: break;
        }
    } else {
        switch (s) {
            case EFS_STAGE_VEL_DECAY: vel_decay2(g); break;
            case EFS_STAGE_VEL_EXTRAPOLATE: vel_extrapolate2(g); break;
            case EFS_STAGE_RHO_SHARPEN: rho_sharpen2(g); break;
            case EFS_STAGE_RHO_ADVECT: rho_advect2(g); break;
            case EFS_STAGE_VEL_ADVECT: vel_advect2(g); break;
            case EFS_STAGE_ADD_FORCE: add_force2(g); break;
            case EFS_STAGE_PROJECT: project2(g); break;
            default: break;
        }
    }
}

/* ISimulator::update (IS:12-38) */
void orc_step(orc_grid* g, int n) {
    for (int k = 0; k < n; k++) {
        for (int s = 0; s < EFS_STAGE_COUNT; s++)
            if (!(g->prm.disable_mask & (1u << s))) orc_stage(g, s);
        g->frames++;
    }
}

/* ------------------------------------------------------------------------------------------------ */
/* FP64 ground truth                                                                                */
/* ------------------------------------------------------------------------------------------------ */

static void matmul_d(const orc_grid* g, double* res, const double* xf) {
    const float* rho = g->rho; const float* bnd = g->boundary;
    const int W = g->W, H = g->H, D = g->D;
    #pragma omp parallel for collapse(2) schedule(static) if (g->N >= ORC_PAR_MIN)
    for (int z = 0; z < D; z++)
    for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
        const size_t i = (size_t)z * W * H + (size_t)y * W + x;
        if (rho[i] <= 0.5f || bnd[i] == 1) { res[i] = xf[i]; continue; }
        double sum = 0.0; int cnt = 0;
        const int nbx[6] = {x - 1, x + 1, x, x, x, x}, nby[6] = {y, y, y - 1, y + 1, y, y}, nbz[6] = {z, z, z, z, z + 1, z - 1};
        const int nn = (g->dim == 3) ? 6 : 4;
        for (int k = 0; k < nn; k++) {
            const int nx = nbx[k], ny = nby[k], nz = nbz[k];
            if (nx < 0 || nx >= W || ny < 0 || ny >= H || nz < 0 || nz >= D) continue;
            if (nx == 0 || nx == W - 1 || ny == 0 || ny == H - 1) continue;
            if (g->dim == 3 && (nz == 0 || nz == D - 1)) continue;
            const size_t j = (size_t)nz * W * H + (size_t)ny * W + nx;
            if (bnd[j] > 0.5f) continue;
            cnt++;
            if (rho[j] > 0.5f) sum += xf[j];
        }
        res[i] = sum - (double)cnt * xf[i];
    }
}

int orc_solve_fp64(orc_grid* g, double tol, int maxit, double* p) {
    const size_t N = g->N;
    double* r = (double*)malloc(N * 8); double* d = (double*)malloc(N * 8); double* t = (double*)malloc(N * 8);
    for (size_t i = 0; i < N; i++) { p[i] = 0; r[i] = g->div[i]; d[i] = r[i]; }
    const double bb = dddot(N, r, r);
    double rr = bb;
    int it = 0;
    const double thr = tol * tol * bb;
    while (it < maxit && rr > thr && rr > 0) {
        matmul_d(g, t, d);
        const double dt = dddot(N, d, t);
        const double a = rr / dt;
        #pragma omp parallel for schedule(static) if (N >= ORC_PAR_MIN)
        for (long i = 0; i < (long)N; i++) { p[i] += a * d[i]; r[i] -= a * t[i]; }
        const double rn = dddot(N, r, r);
        const double b = rn / rr; rr = rn;
        #pragma omp parallel for schedule(static) if (N >= ORC_PAR_MIN)
        for (long i = 0; i < (long)N; i++) d[i] = r[i] + b * d[i];
        it++;
    }
    free(r); free(d); free(t);
    return it;
}

double orc_relres_fp64(orc_grid* g, const float* pf) {
    const size_t N = g->N;
    double* p = (double*)malloc(N * 8); double* t = (double*)malloc(N * 8);
    for (size_t i = 0; i < N; i++) p[i] = pf[i];
    matmul_d(g, t, p);
    double rr = 0, bb = 0;
    for (size_t i = 0; i < N; i++) { const double r = (double)g->div[i] - t[i]; rr += r * r; bb += (double)g->div[i] * g->div[i]; }
    free(p); free(t);
    return bb > 0 ? sqrt(rr / bb) : sqrt(rr);
}

/* ------------------------------------------------------------------------------------------------ */
/* parameter preset                                                                                  */
/* ------------------------------------------------------------------------------------------------ */

/* reference Properties defaults (Properties.h:141-162) */
void orc_params_default(efs_params* p) {
    memset(p, 0, sizeof(*p));
    p->dt = 0.0167f; p->gravity_force = 10.f; p->gravity_enabled = 1; p->vel_decay = 0.8f;
    p->lambda_minus = .5f; p->lambda_plus = .1f; p->eta = 1.f; p->liquid_threshold = 0.5f; p->rho_d = 3.f;
    p->solver = EFS_SOLVER_CG; p->max_steps = 2000; p->solver_threshold = 1e-5f; p->tol_rel = 0.f;
    p->disable_mask = 0; p->re_calc_div = 0; p->sharpen_mode = EFS_SHARPEN_PARALLEL;
    p->cg_variant = EFS_CG_MIXED_RECURRENCE;
    p->fcg_levels = -1; p->fcg_bottom = EFS_FCG_BOTTOM_UNET;
}

/* ------------------------------------------------------------------------------------------------ */
/* seeded scenes (the same header the library and the reference harness use)                        */
/* ------------------------------------------------------------------------------------------------ */
#include "../include/efs_scene.h"

int orc_scene_dam3d(int w, int h, int d, int n_min, int n_max, uint64_t seed, float* boundary, float* rho) {
    return efs_scene_dam3d_fill(w, h, d, n_min, n_max, seed, boundary, rho);
}
int orc_scene_dam2d(int w, int h, float* boundary, float* rho) { return efs_scene_dam2d_fill(w, h, boundary, rho); }
int orc_scene_batch2d(uint64_t seed, int* side, float* boundary, float* rho) {
    return efs_scene_batch2d_fill(seed, side, boundary, rho);
}
