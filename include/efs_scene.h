/*
 * efs_scene.h — header-only seeded synthetic scenes for the Eulerian liquid step (plain C99).
 *
 * The reference voxelises its scenes with OpenGL compute shaders (src/core/Editor.cpp:90-258,
 * assets/shaders/sdf.comp, baseFluidFill.comp), which need a graphics stack.  These generators write the
 * same two arrays the reference Editor writes through IGrid3D::boundary()/rho() (Editor.cpp:21-38):
 * `boundary` (1.0 solid, 0.0 otherwise) and `rho` (1.0 liquid, 0.0 otherwise), in the reference layout
 * (index z*W*H + y*W + x, one-cell solid border included).
 *
 * Geometry: the domain is the unit square / cube; cell (i,j,k) has centre ((i+0.5)/W, (j+0.5)/H, (k+0.5)/D).
 * A cell is solid when it is on the border or its centre lies in an obstacle; liquid when its centre
 * satisfies the fluid predicate and it is not solid (rho = 0 in solids, as Editor.cpp:256 does).
 * Cavities: non-solid cells that are not connected (through faces of non-solid cells) to the open top row of
 * the domain (y = H-2) become solid.  Overlapping obstacles can leave such cells; a liquid cell inside one
 * gives the pressure matrix a row with no free neighbour (or a closed Neumann block), which no solver can
 * satisfy once its divergence is non-zero, so the reference's project() would pause for good.  For the same
 * reason a connected set of non-solid cells that holds no air cell (rho <= 0.5) at all, such as a pocket the
 * obstacles close off that a fluid blob fills, becomes solid as well (rho 0).
 *
 * Random numbers: PCG32 (M. E. O'Neill, "PCG: A Family of Simple Fast Space-Efficient Statistically Good
 * Algorithms for Random Number Generation", 2014), XSH-RR output, 64-bit LCG state with multiplier
 * 6364136223846793005; seeded with (initstate = seed, initseq = EFS_SCENE_STREAM) by the paper's
 * srandom procedure.  A uniform draw U(a,b) is a + (b - a) * ((next() >> 8) * 2^-24) in double;
 * an integer draw in [lo, hi] is lo + next() % (hi - lo + 1).
 *
 * Draw order
 *   dam3d:   n = int[n_min, n_max]; then per sphere: cx, cy, cz = U(0.2, 0.8), r = U(0.04, 0.10).
 *            Fluid: x < 0.4 and y < 0.6 (all z).  Cavities filled (all generators).
 *   dam2d:   no draws.  Fluid: x < 0.4 and y < 0.6.
 *   batch2d: side = {64, 96, 128, 192, 256}[int[0, 4]]; n_rect = int[1, 4]; per rectangle:
 *            x0 = U(0.05, 0.80), y0 = U(0.05, 0.60), wx = U(0.05, 0.25), wy = U(0.03, 0.15);
 *            n_blob = int[1, 3]; per circle: cx = U(0.25, 0.75), cy = U(0.35, 0.75), r = U(0.10, 0.25).
 *            Solid: inside any rectangle [x0, x0+wx] x [y0, y0+wy]; fluid: inside any circle.
 */
#ifndef EFS_SCENE_H
#define EFS_SCENE_H

#include <stdint.h>
#include <stddef.h>
#include <stdlib.h>

#define EFS_SCENE_STREAM 0x0EF5u

typedef struct efs_pcg32 { uint64_t state, inc; } efs_pcg32;

static inline uint32_t efs_pcg32_next(efs_pcg32* g) {
    uint64_t old = g->state;
    g->state = old * 6364136223846793005ULL + g->inc;
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((-rot) & 31u));
}

static inline void efs_pcg32_seed(efs_pcg32* g, uint64_t initstate, uint64_t initseq) {
    g->state = 0u;
    g->inc = (initseq << 1u) | 1u;
    efs_pcg32_next(g);
    g->state += initstate;
    efs_pcg32_next(g);
}

static inline double efs_pcg32_uniform(efs_pcg32* g, double a, double b) {
    double u = (double)(efs_pcg32_next(g) >> 8) * (1.0 / 16777216.0);
    return a + (b - a) * u;
}

static inline int efs_pcg32_int(efs_pcg32* g, int lo, int hi) {
    return lo + (int)(efs_pcg32_next(g) % (uint32_t)(hi - lo + 1));
}

#define EFS_SCENE_MAX_OBJECTS 64

/* Make every non-solid cell that cannot reach the top interior row through face neighbours solid (rho 0),
 * and every connected set of non-solid cells without an air cell.  Returns the number of cells filled, or -1
 * when the work queue cannot be allocated. */
static inline long efs_scene_fill_cavities(int W, int H, int D, float* boundary, float* rho) {
    const size_t N = (size_t)W * H * D, WH = (size_t)W * H;
    unsigned char* seen = (unsigned char*)calloc(N, 1);
    size_t* q = (size_t*)malloc(N * sizeof(size_t));
    if (!seen || !q) { free(seen); free(q); return -1; }
    size_t head = 0, tail = 0;
    const int yt = H - 2;
    for (int z = 0; z < D; z++)
    for (int x = 0; x < W; x++) {
        const size_t i = (size_t)z * WH + (size_t)yt * W + x;
        if (boundary[i] != 1.0f && !seen[i]) { seen[i] = 1; q[tail++] = i; }
    }
    while (head < tail) {
        const size_t i = q[head++];
        const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)(i / WH);
        const long nb[6][3] = {{x - 1, y, z}, {x + 1, y, z}, {x, y - 1, z}, {x, y + 1, z}, {x, y, z - 1}, {x, y, z + 1}};
        for (int k = 0; k < 6; k++) {
            const long nx = nb[k][0], ny = nb[k][1], nz = nb[k][2];
            if (nx < 0 || ny < 0 || nz < 0 || nx >= W || ny >= H || nz >= D) continue;
            const size_t j = (size_t)nz * WH + (size_t)ny * W + (size_t)nx;
            if (seen[j] || boundary[j] == 1.0f) continue;
            seen[j] = 1;
            q[tail++] = j;
        }
    }
    long filled = 0;
    for (size_t i = 0; i < N; i++)
        if (boundary[i] != 1.0f && !seen[i]) { boundary[i] = 1.0f; rho[i] = 0.0f; filled++; }
    /* components of non-solid cells without an air cell: seen[] is reused as 2 = labelled */
    for (size_t s0 = 0; s0 < N; s0++) {
        if (boundary[s0] == 1.0f || seen[s0] == 2) continue;
        head = tail = 0;
        seen[s0] = 2;
        q[tail++] = s0;
        int air = 0;
        while (head < tail) {
            const size_t i = q[head++];
            if (!(rho[i] > 0.5f)) air = 1;
            const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)(i / WH);
            const long nb[6][3] = {{x - 1, y, z}, {x + 1, y, z}, {x, y - 1, z}, {x, y + 1, z}, {x, y, z - 1}, {x, y, z + 1}};
            for (int k = 0; k < 6; k++) {
                const long nx = nb[k][0], ny = nb[k][1], nz = nb[k][2];
                if (nx < 0 || ny < 0 || nz < 0 || nx >= W || ny >= H || nz >= D) continue;
                const size_t j = (size_t)nz * WH + (size_t)ny * W + (size_t)nx;
                if (seen[j] == 2 || boundary[j] == 1.0f) continue;
                seen[j] = 2;
                q[tail++] = j;
            }
        }
        if (!air)
            for (size_t k = 0; k < tail; k++) { boundary[q[k]] = 1.0f; rho[q[k]] = 0.0f; filled++; }
    }
    free(seen);
    free(q);
    return filled;
}

/* 3D dam break with seeded solid spheres.  Returns the number of spheres, or -1 on bad arguments. */
static inline int efs_scene_dam3d_fill(int W, int H, int D, int n_min, int n_max, uint64_t seed,
                                       float* boundary, float* rho) {
    if (W < 4 || H < 4 || D < 4 || n_min < 0 || n_max < n_min || n_max > EFS_SCENE_MAX_OBJECTS) return -1;
    efs_pcg32 g;
    efs_pcg32_seed(&g, seed, EFS_SCENE_STREAM);
    int n = efs_pcg32_int(&g, n_min, n_max);
    double sc[EFS_SCENE_MAX_OBJECTS][4];
    for (int s = 0; s < n; s++) {
        sc[s][0] = efs_pcg32_uniform(&g, 0.2, 0.8);
        sc[s][1] = efs_pcg32_uniform(&g, 0.2, 0.8);
        sc[s][2] = efs_pcg32_uniform(&g, 0.2, 0.8);
        sc[s][3] = efs_pcg32_uniform(&g, 0.04, 0.10);
    }
    for (int z = 0; z < D; z++)
    for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
        size_t i = ((size_t)z * H + y) * W + x;
        double px = (x + 0.5) / W, py = (y + 0.5) / H, pz = (z + 0.5) / D;
        int solid = (x == 0 || y == 0 || z == 0 || x == W - 1 || y == H - 1 || z == D - 1);
        for (int s = 0; s < n && !solid; s++) {
            double dx = px - sc[s][0], dy = py - sc[s][1], dz = pz - sc[s][2];
            if (dx * dx + dy * dy + dz * dz <= sc[s][3] * sc[s][3]) solid = 1;
        }
        int fluid = (px < 0.4 && py < 0.6);
        boundary[i] = solid ? 1.0f : 0.0f;
        rho[i] = (!solid && fluid) ? 1.0f : 0.0f;
    }
    if (efs_scene_fill_cavities(W, H, D, boundary, rho) < 0) return -1;
    return n;
}

/* 2D dam break without obstacles (fluid x < 0.4, y < 0.6). */
static inline int efs_scene_dam2d_fill(int W, int H, float* boundary, float* rho) {
    if (W < 4 || H < 4) return -1;
    for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
        size_t i = (size_t)y * W + x;
        double px = (x + 0.5) / W, py = (y + 0.5) / H;
        int solid = (x == 0 || y == 0 || x == W - 1 || y == H - 1);
        boundary[i] = solid ? 1.0f : 0.0f;
        rho[i] = (!solid && px < 0.4 && py < 0.6) ? 1.0f : 0.0f;
    }
    if (efs_scene_fill_cavities(W, H, 1, boundary, rho) < 0) return -1;
    return 0;
}

static const int efs_scene_batch_sides[5] = {64, 96, 128, 192, 256};

/* One scene of the uneven 2D batch.  Writes the side length to *side; fills boundary/rho (side*side
 * floats each) only when both pointers are non-NULL.  Returns 0, or -1 on bad arguments. */
static inline int efs_scene_batch2d_fill(uint64_t seed, int* side, float* boundary, float* rho) {
    efs_pcg32 g;
    efs_pcg32_seed(&g, seed, EFS_SCENE_STREAM);
    int S = efs_scene_batch_sides[efs_pcg32_int(&g, 0, 4)];
    if (side) *side = S;
    int nr = efs_pcg32_int(&g, 1, 4);
    double rc[4][4];
    for (int r = 0; r < nr; r++) {
        rc[r][0] = efs_pcg32_uniform(&g, 0.05, 0.80);
        rc[r][1] = efs_pcg32_uniform(&g, 0.05, 0.60);
        rc[r][2] = efs_pcg32_uniform(&g, 0.05, 0.25);
        rc[r][3] = efs_pcg32_uniform(&g, 0.03, 0.15);
    }
    int nb = efs_pcg32_int(&g, 1, 3);
    double bc[3][3];
    for (int b = 0; b < nb; b++) {
        bc[b][0] = efs_pcg32_uniform(&g, 0.25, 0.75);
        bc[b][1] = efs_pcg32_uniform(&g, 0.35, 0.75);
        bc[b][2] = efs_pcg32_uniform(&g, 0.10, 0.25);
    }
    if (!boundary || !rho) return 0;
    for (int y = 0; y < S; y++)
    for (int x = 0; x < S; x++) {
        size_t i = (size_t)y * S + x;
        double px = (x + 0.5) / S, py = (y + 0.5) / S;
        int solid = (x == 0 || y == 0 || x == S - 1 || y == S - 1);
        for (int r = 0; r < nr && !solid; r++)
            if (px >= rc[r][0] && px <= rc[r][0] + rc[r][2] && py >= rc[r][1] && py <= rc[r][1] + rc[r][3]) solid = 1;
        int fluid = 0;
        for (int b = 0; b < nb && !fluid; b++) {
            double dx = px - bc[b][0], dy = py - bc[b][1];
            if (dx * dx + dy * dy <= bc[b][2] * bc[b][2]) fluid = 1;
        }
        boundary[i] = solid ? 1.0f : 0.0f;
        rho[i] = (!solid && fluid) ? 1.0f : 0.0f;
    }
    if (efs_scene_fill_cavities(S, S, 1, boundary, rho) < 0) return -1;
    return 0;
}

#endif /* EFS_SCENE_H */
