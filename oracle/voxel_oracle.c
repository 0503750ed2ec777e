/*
 * voxel_oracle.c — CPU restatement of the voxelizer's inside test (TEST
 * INFRASTRUCTURE ONLY: the oracle).
 *
 * Counts ray/triangle hits over ALL triangles (no BVH). This equals the
 * reference's BVH count (aeros/src/mesh_bvh.h:116-160): its float slab test
 * only rejects a node when the ray's perpendicular coordinates lie outside
 * the node box or the box lies entirely behind the origin, and a triangle
 * hit with t > 1e-7 needs neither, so culling never drops a hit.
 * Triangle test: double-precision Moller-Trumbore, mesh_bvh.h:62-96.
 * Three-ray vote: mesh_bvh.h:168-185. Degenerate filter: mesh_bvh.h:50-53 and
 * voxel_grid.cpp:313-325. Grid plan: voxel_grid.cpp:172-215.
 * Built with -ffp-contract=off so every float/double operation rounds as the
 * reference's x86-64 build does.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "aeros_oracle.h"

typedef struct { float x, y, z; } v3;

static inline v3 v3sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
/* glm::cross operand order */
static inline v3 v3cross(v3 a, v3 b) {
    v3 r = {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
    return r;
}
/* glm::length = sqrt((x*x + y*y) + z*z) */
static inline float v3len(v3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }

static int ray_triangle(v3 o, v3 d, v3 v0, v3 v1, v3 v2, double minT, double maxT) {
    const double e1x = (double)v1.x - v0.x, e1y = (double)v1.y - v0.y, e1z = (double)v1.z - v0.z;
    const double e2x = (double)v2.x - v0.x, e2y = (double)v2.y - v0.y, e2z = (double)v2.z - v0.z;
    const double dx = d.x, dy = d.y, dz = d.z;
    const double px = dy * e2z - dz * e2y;
    const double py = dz * e2x - dx * e2z;
    const double pz = dx * e2y - dy * e2x;
    const double det = e1x * px + e1y * py + e1z * pz;
    const double scale = fabs(e1x * e2y - e1y * e2x) + fabs(e1y * e2z - e1z * e2y) + fabs(e1z * e2x - e1x * e2z) + 1e-30;
    if (fabs(det) < 1e-12 * scale) return 0;
    const double inv = 1.0 / det;
    const double tx = (double)o.x - v0.x, ty = (double)o.y - v0.y, tz = (double)o.z - v0.z;
    const double u = (tx * px + ty * py + tz * pz) * inv;
    if (u < 0.0 || u > 1.0) return 0;
    const double qx = ty * e1z - tz * e1y;
    const double qy = tz * e1x - tx * e1z;
    const double qz = tx * e1y - ty * e1x;
    const double v = (dx * qx + dy * qy + dz * qz) * inv;
    if (v < 0.0 || u + v > 1.0) return 0;
    const double t = (e2x * qx + e2y * qy + e2z * qz) * inv;
    if (!(t > minT) || t >= maxT) return 0;
    return 1;
}

/* Keeps finite, non-degenerate triangles (voxel_grid.cpp:313-325). */
static int64_t filter_tris(const float* tris, int64_t ntri, v3* out) {
    int64_t k = 0;
    for (int64_t i = 0; i < ntri; ++i) {
        const float* t = tris + 9 * i;
        int ok = 1;
        for (int j = 0; j < 9; ++j) if (!isfinite(t[j])) ok = 0;
        if (!ok) continue;
        v3 a = {t[0], t[1], t[2]}, b = {t[3], t[4], t[5]}, c = {t[6], t[7], t[8]};
        const float area2 = v3len(v3cross(v3sub(b, a), v3sub(c, a)));
        if (!(area2 > 1e-14f) || !isfinite(area2)) continue;
        out[3 * k] = a; out[3 * k + 1] = b; out[3 * k + 2] = c;
        ++k;
    }
    return k;
}

static int count_hits(const v3* tv, int64_t n, v3 o, v3 d) {
    int hits = 0;
    for (int64_t i = 0; i < n; ++i)
        if (ray_triangle(o, d, tv[3 * i], tv[3 * i + 1], tv[3 * i + 2], 1e-7, 1e30)) ++hits;
    return hits;
}

int ao_count_hits_brute(const float* tris, int64_t ntri, const float o[3], int axis) {
    v3* tv = (v3*)malloc(sizeof(v3) * 3 * (size_t)(ntri > 0 ? ntri : 1));
    if (!tv) return -1;
    const int64_t n = filter_tris(tris, ntri, tv);
    v3 org = {o[0], o[1], o[2]};
    v3 d = {axis == 0 ? 1.0f : 0.0f, axis == 1 ? 1.0f : 0.0f, axis == 2 ? 1.0f : 0.0f};
    const int h = count_hits(tv, n, org, d);
    free(tv);
    return h;
}

int ao_voxelize_brute(const float* tris, int64_t ntri, const aeros_voxel_grid* g, uint8_t* mask) {
    if (!g || !mask || g->nx <= 0 || g->ny <= 0 || g->nz <= 0) return -1;
    const size_t total = (size_t)g->nx * g->ny * g->nz;
    memset(mask, 0, total);
    if (ntri <= 0) return 0;
    v3* tv = (v3*)malloc(sizeof(v3) * 3 * (size_t)ntri);
    if (!tv) return -1;
    const int64_t n = filter_tris(tris, ntri, tv);
    if (n == 0) { free(tv); return 0; }
    const float csx = g->cell[0], csy = g->cell[1], csz = g->cell[2];
    /* jitter, mesh_bvh.h:176-178 */
    const float jx = 0.731f * 1e-3f * csx, jy = 0.377f * 1e-3f * csy, jz = 0.557f * 1e-3f * csz;
    const v3 dx = {1, 0, 0}, dy = {0, 1, 0}, dz = {0, 0, 1};
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                const float px = g->min[0] + (i + 0.5f) * csx;
                const float py = g->min[1] + (j + 0.5f) * csy;
                const float pz = g->min[2] + (k + 0.5f) * csz;
                int votes = 0;
                v3 o1 = {px, py + jy, pz + jz};
                v3 o2 = {px + jz, py, pz + jx};
                v3 o3 = {px + jy, py + jx, pz};
                if (count_hits(tv, n, o1, dx) & 1) ++votes;
                if (count_hits(tv, n, o2, dy) & 1) ++votes;
                if (count_hits(tv, n, o3, dz) & 1) ++votes;
                mask[((size_t)k * g->ny + j) * g->nx + i] = votes >= 2 ? 1 : 0;
            }
    free(tv);
    return 0;
}

/* voxelPlan, aeros/src/voxel_grid.cpp:172-215 (224 bytes per cell, res in [8,512]). */
static void plan_dims(int rr, float sy, float sz, float m, int* nx, int* ny, int* nz) {
    *nx = rr;
    *ny = (int)floorf(rr * sy / m); if (*ny < 4) *ny = 4;
    *nz = (int)floorf(rr * sz / m); if (*nz < 4) *nz = 4;
}

void ao_voxel_plan(const float size[3], int res, uint64_t budget, aeros_voxel_plan_t* p) {
    memset(p, 0, sizeof(*p));
    p->requested_res = res;
    int r = res < 8 ? 8 : (res > 512 ? 512 : res);
    float sx = size[0], sy = size[1], sz = size[2];
    if (!(sx > 1e-6f) || !isfinite(sx)) sx = 1.0f;
    if (!(sy > 1e-6f) || !isfinite(sy)) sy = 1.0f;
    if (!(sz > 1e-6f) || !isfinite(sz)) sz = 1.0f;
    float m = sy > sz ? sy : sz;      /* std::max(sx, std::max(sy, sz)) */
    m = sx < m ? m : sx;
    int nx, ny, nz;
    plan_dims(r, sy, sz, m, &nx, &ny, &nz);
    p->nx = nx; p->ny = ny; p->nz = nz;
    p->cells = (int64_t)nx * ny * nz;
    p->bytes = (uint64_t)p->cells * 224ull;
    p->fits = (budget == 0) || (p->bytes <= budget);
    if (!p->fits && budget > 0) {
        double scale = cbrt((double)budget / (double)p->bytes) * 0.95;
        int cand = (int)(r * scale);
        for (int guard = 0; guard < 64 && cand >= 8; ++guard, --cand) {
            int a, b, c;
            plan_dims(cand, sy, sz, m, &a, &b, &c);
            if ((uint64_t)a * b * c * 224ull <= budget) { p->suggested_res = cand; break; }
        }
        if (p->suggested_res < 8) p->suggested_res = 0;
    }
}
