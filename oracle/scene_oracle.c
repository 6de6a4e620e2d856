/* scene_oracle.c — CPU restatement of the reference's scene construction and query arithmetic.
 * TEST INFRASTRUCTURE ONLY: tests/ use it as the checker of efs_mesh_label / efs_mesh_cells / efs_query_box.
 *
 * - orc_mesh_label restates the SDF compute shader (assets/shaders/sdf.comp:25-114) as the reference's GPU
 *   runs it per cell: the unsigned triangle distance (sdf.comp:29-51), the solid angle of a triangle
 *   (:53-68), the winding number (:70-78) and the signed distance (:80-92), then the label (:107-113).  It
 *   keeps every step of the shader, including the square roots and the running minimum that the CUDA kernel
 *   reduces to a zero test, so it also checks that reduction.  GLSL's dot and cross are written out in the
 *   order of the GLSL specification; normalize(v) is v / length(v); min/max/clamp use fminf/fmaxf.
 * - orc_query_box restates QueryNode::update's loop (src/simulation/scene/nodes/QueryNode.cpp:47-84) with
 *   the reference's float accumulators in its loop order (z, y, x).
 *
 * Compiled with -ffp-contract=off like efs_oracle.c, so products and sums round separately.
 */
#include <math.h>
#include <stdint.h>

typedef struct { float x, y, z; } v3;

static v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 scl(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float dot2(v3 a) { return dot(a, a); }
static v3 cross(v3 a, v3 b) { return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
static float sgn(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
static float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
static v3 normalize(v3 a) { const float l = sqrtf(dot(a, a)); return mk(a.x / l, a.y / l, a.z / l); }

/* sdf.comp:29-51 */
static float distance_triangle(v3 p, v3 v1, v3 v2, v3 v3_) {
    const v3 v21 = sub(v2, v1), v32 = sub(v3_, v2), v13 = sub(v1, v3_);
    const v3 p1 = sub(p, v1), p2 = sub(p, v2), p3 = sub(p, v3_);
    const v3 normal = cross(v21, v13);
    if (sgn(dot(cross(v21, normal), p1)) + sgn(dot(cross(v32, normal), p2)) + sgn(dot(cross(v13, normal), p3)) < 2.0f) {
        return sqrtf(fminf(fminf(dot2(sub(scl(v21, clampf(dot(v21, p1) / dot2(v21), 0.0f, 1.0f)), p1)),
                                 dot2(sub(scl(v32, clampf(dot(v32, p2) / dot2(v32), 0.0f, 1.0f)), p2))),
                           dot2(sub(scl(v13, clampf(dot(v13, p3) / dot2(v13), 0.0f, 1.0f)), p3))));
    }
    return sqrtf(dot(normal, p1) * dot(normal, p1) / dot2(normal));
}

/* sdf.comp:53-68 */
static float solid_angle(v3 position, v3 v0, v3 v1, v3 v2) {
    const v3 a = normalize(sub(v0, position)), b = normalize(sub(v1, position)), c = normalize(sub(v2, position));
    const float numerator = dot(a, cross(b, c));
    const float denom = 1.0f + dot(a, b) + dot(b, c) + dot(c, a);
    return 2.0f * atan2f(numerator, denom);
}

static v3 tri_vertex(const float* t, int k) { return mk(t[4 * k], t[4 * k + 1], t[4 * k + 2]); }

/* sdf.comp:80-92 */
static float calculate_sdf(v3 position, const float* tris, int n) {
    float best = 1e20f;
    for (int i = 0; i < n; i++) {
        const float* t = tris + 12 * (long)i;
        const float dist = distance_triangle(position, tri_vertex(t, 0), tri_vertex(t, 1), tri_vertex(t, 2));
        if (dist < best) best = dist;
    }
    float winding = 0.0f;
    for (int i = 0; i < n; i++) {
        const float* t = tris + 12 * (long)i;
        winding += solid_angle(position, tri_vertex(t, 0), tri_vertex(t, 1), tri_vertex(t, 2));
    }
    return fabsf(winding) > 3.1415926f ? -best : best;
}

/* sdf.comp:94-114 over the whole grid: cells of [0, W-1) x [0, H-1) x [0, D-1) get vin / vout. */
void orc_mesh_label(int W, int H, int D, const float* tris, int n, const float center[3], const float size[3],
                    float vin, float vout, float* out) {
    const float csx = size[0] / (float)W, csy = size[1] / (float)H, csz = size[2] / (float)D;
    const float mx = center[0] - 0.5f * size[0], my = center[1] - 0.5f * size[1], mz = center[2] - 0.5f * size[2];
    for (int z = 0; z < D - 1; z++)
        for (int y = 0; y < H - 1; y++)
            for (int x = 0; x < W - 1; x++) {
                const v3 q = mk(mx + csx * (float)x + csx * 0.5f, my + csy * (float)y + csy * 0.5f,
                                mz + csz * (float)z + csz * 0.5f);
                out[(long)z * W * H + (long)y * W + x] = calculate_sdf(q, tris, n) > 0.0f ? vout : vin;
            }
}

/* QueryNode.cpp:47-84.  out: max_position[3], min_position[3], avg_position[3], velocity[3], pressure;
 * returns the cell count.  w may be NULL (2D: z ignored, one layer). */
long long orc_query_box(int dim, int W, int H, int D, const float* rho, const float* u, const float* v,
                        const float* w, const float* p, const int position[3], const int scale[3], int only_fluid,
                        float* out) {
    float mxp[3] = {-INFINITY, -INFINITY, -INFINITY}, mnp[3] = {INFINITY, INFINITY, INFINITY};
    float avg[3] = {0, 0, 0}, vel[3] = {0, 0, 0}, pres = 0.0f;
    int count = 0;
    const int z0 = dim == 3 ? (position[2] > 0 ? position[2] : 0) : 0;
    const int z1 = dim == 3 ? ((D - 1) < position[2] + scale[2] ? (D - 1) : position[2] + scale[2]) : 1;
    const int y0 = position[1] > 0 ? position[1] : 0, y1 = (H - 1) < position[1] + scale[1] ? (H - 1) : position[1] + scale[1];
    const int x0 = position[0] > 0 ? position[0] : 0, x1 = (W - 1) < position[0] + scale[0] ? (W - 1) : position[0] + scale[0];
    for (int z = z0; z < z1; z++)
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++) {
                const long i = (long)z * W * H + (long)y * W + x;
                if (only_fluid && rho[i] < 0.5f) continue;
                const float c[3] = {(float)x, (float)y, (float)z};
                for (int d = 0; d < 3; d++) {
                    mxp[d] = fmaxf(mxp[d], c[d]);
                    mnp[d] = fminf(mnp[d], c[d]);
                }
                count++;
                for (int d = 0; d < 3; d++) avg[d] += c[d];
                vel[0] += u[i];
                vel[1] += v[i];
                vel[2] += w ? w[i] : 0.0f;
                pres += p[i];
            }
    if (count != 0) {
        for (int d = 0; d < 3; d++) {
            avg[d] /= (float)count;
            vel[d] /= (float)count;
        }
        pres /= (float)count;
    } else {
        for (int d = 0; d < 3; d++) mxp[d] = mnp[d] = 0.0f;
    }
    for (int d = 0; d < 3; d++) {
        out[d] = mxp[d];
        out[3 + d] = mnp[d];
        out[6 + d] = avg[d];
        out[9 + d] = vel[d];
    }
    out[12] = pres;
    return count;
}
