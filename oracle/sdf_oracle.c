/*
 * sdf_oracle.c — CPU restatement of the voxel grid's signed distance field
 * (TEST INFRASTRUCTURE ONLY: the oracle).
 *
 * ao_sdf_reference follows buildVoxelGrid's distance-field part
 * (aeros/src/voxel_grid.cpp:384-553) step by step:
 *   - seeds: a cell is on the surface when a 6-neighbour inside the grid has
 *     the other solidity (solid means mask == 1); it starts at -0.5 or +0.5
 *     of the smallest cell size, every other cell at 1e6 (:384-410);
 *   - 26 neighbours in dz, dy, dx order with weight sqrtf(wx^2 + wy^2 + wz^2)
 *     (:412-422);
 *   - four raster sweeps (+++, -++, +-+, ---) that push |d| + w to a
 *     neighbour when it improves it by more than 1e-4 (:424-455);
 *   - a FIFO pass from the seed list that pushes improvements of more than
 *     1e-3 and queues the improved cell (:457-477);
 *   - two rounds of x, y, z smoothing passes (kernel 0.25 0.5 0.25, blended
 *     0.35 / 0.65) on interior cells farther than 3 cells from the surface
 *     (:479-540).
 * Its result depends on the visiting order and on the two thresholds.
 *
 * ao_sdf_exact is what the device computes: the same seeds and weights, but
 * the propagation is run to the least fixed point of
 *     |d(c)| = min(|d0(c)|, min_n fl(|d(n)| + w(n, c))),
 * the float shortest-path length over all 26-neighbour paths from a seed
 * (unique because float addition of a positive weight is monotone), with the
 * sign of the seed the path starts from; equal magnitudes keep the negative
 * (inside) sign. Computed here by a label-correcting queue; any order gives
 * the same field. Then the same smoothing.
 *
 * Built with -ffp-contract=off so every float operation rounds as the
 * reference's x86-64 build does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "aeros_oracle.h"

typedef struct {
    int dx, dy, dz;
    float w;
} sdf_nb;

static void sdf_neighbours(const float cs[3], sdf_nb nb[26]) {
    int k = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                if (dx == 0 && dy == 0 && dz == 0) continue;
                const float wx = dx * cs[0], wy = dy * cs[1], wz = dz * cs[2];
                nb[k].dx = dx; nb[k].dy = dy; nb[k].dz = dz;
                nb[k].w = sqrtf(wx * wx + wy * wy + wz * wz);
                ++k;
            }
}

/* Seeds (voxel_grid.cpp:384-410). Returns the seed count; seeds[] gets their
 * indices in raster order. */
static int64_t sdf_seed(const uint8_t* mask, int nx, int ny, int nz, const float cs[3], float* d, int64_t* seeds) {
    static const int off6[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    const float m = fminf(cs[0], fminf(cs[1], cs[2]));
    int64_t ns = 0;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const int64_t idx = ((int64_t)k * ny + j) * nx + i;
                const int here = mask[idx] == 1;
                int surf = 0;
                for (int o = 0; o < 6 && !surf; ++o) {
                    const int ni = i + off6[o][0], nj = j + off6[o][1], nk = k + off6[o][2];
                    if (ni < 0 || ni >= nx || nj < 0 || nj >= ny || nk < 0 || nk >= nz) continue;
                    if ((mask[((int64_t)nk * ny + nj) * nx + ni] == 1) != here) surf = 1;
                }
                d[idx] = 1e6f;
                if (surf) {
                    d[idx] = here ? -0.5f * m : 0.5f * m;
                    seeds[ns++] = idx;
                }
            }
    return ns;
}

/* Smoothing (voxel_grid.cpp:479-540): 2 rounds of x, y, z passes. */
static void sdf_smooth(float* d, float* temp, int nx, int ny, int nz, const float cs[3]) {
    const int64_t total = (int64_t)nx * ny * nz;
    const int64_t sx = 1, sy = nx, sz = (int64_t)nx * ny;
    const int64_t stride[3] = {sx, sy, sz};
    memcpy(temp, d, (size_t)total * sizeof(float));
    for (int iter = 0; iter < 2; ++iter)
        for (int axis = 0; axis < 3; ++axis) {
            const float lim = cs[axis] * 3.0f;
            const int64_t s = stride[axis];
            for (int k = 1; k < nz - 1; ++k)
                for (int j = 1; j < ny - 1; ++j)
                    for (int i = 1; i < nx - 1; ++i) {
                        const int64_t idx = ((int64_t)k * ny + j) * nx + i;
                        if (fabsf(temp[idx]) < lim) continue;
                        const float sum = temp[idx - s] * 0.25f + temp[idx] * 0.5f + temp[idx + s] * 0.25f;
                        d[idx] = sum * 0.35f + temp[idx] * 0.65f;
                    }
            memcpy(temp, d, (size_t)total * sizeof(float));
        }
}

typedef struct {
    int64_t* v;
    int64_t n, cap;
} i64vec;

static int push(i64vec* q, int64_t x) {
    if (q->n == q->cap) {
        const int64_t cap = q->cap ? 2 * q->cap : 1024;
        int64_t* nv = (int64_t*)realloc(q->v, (size_t)cap * sizeof(int64_t));
        if (!nv) return -1;
        q->v = nv;
        q->cap = cap;
    }
    q->v[q->n++] = x;
    return 0;
}

int ao_sdf_reference(const uint8_t* mask, int nx, int ny, int nz, const float cs[3], float* d) {
    if (!mask || !d || nx <= 0 || ny <= 0 || nz <= 0) return -1;
    const int64_t total = (int64_t)nx * ny * nz;
    i64vec q = {0, 0, 0};
    float* temp = (float*)malloc((size_t)total * sizeof(float));
    int64_t* seeds = (int64_t*)malloc((size_t)total * sizeof(int64_t));
    if (!temp || !seeds) { free(temp); free(seeds); return -1; }
    const int64_t ns = sdf_seed(mask, nx, ny, nz, cs, d, seeds);
    for (int64_t s = 0; s < ns; ++s)
        if (push(&q, seeds[s])) { free(temp); free(seeds); free(q.v); return -1; }
    free(seeds);
    sdf_nb nb[26];
    sdf_neighbours(cs, nb);

    /* four sweeps (voxel_grid.cpp:424-455) */
    for (int sweep = 0; sweep < 4; ++sweep) {
        const int ri = sweep == 1 || sweep == 3, rj = sweep == 2 || sweep == 3, rk = sweep == 3;
        for (int kk = 0; kk < nz; ++kk)
            for (int jj = 0; jj < ny; ++jj)
                for (int ii = 0; ii < nx; ++ii) {
                    const int k = rk ? nz - 1 - kk : kk, j = rj ? ny - 1 - jj : jj, i = ri ? nx - 1 - ii : ii;
                    const int64_t idx = ((int64_t)k * ny + j) * nx + i;
                    const float cur = d[idx];
                    if (fabsf(cur) > 1e5f) continue;
                    for (int n = 0; n < 26; ++n) {
                        const int ni = i + nb[n].dx, nj = j + nb[n].dy, nk = k + nb[n].dz;
                        if (ni < 0 || ni >= nx || nj < 0 || nj >= ny || nk < 0 || nk >= nz) continue;
                        const int64_t nidx = ((int64_t)nk * ny + nj) * nx + ni;
                        const float nd = (cur < 0) ? (cur - nb[n].w) : (cur + nb[n].w);
                        if (fabsf(nd) < fabsf(d[nidx]) - 1e-4f) d[nidx] = nd;
                    }
                }
    }

    /* FIFO pass (voxel_grid.cpp:457-477) */
    for (int64_t head = 0; head < q.n; ++head) {
        const int64_t idx = q.v[head];
        const int i = (int)(idx % nx);
        const int j = (int)((idx / nx) % ny);
        const int k = (int)(idx / ((int64_t)nx * ny));
        const float v = d[idx];
        if (!(isfinite(v) && fabsf(v) < 1e6f)) continue;
        for (int n = 0; n < 26; ++n) {
            const int ni = i + nb[n].dx, nj = j + nb[n].dy, nk = k + nb[n].dz;
            if (ni < 0 || ni >= nx || nj < 0 || nj >= ny || nk < 0 || nk >= nz) continue;
            const int64_t nidx = ((int64_t)nk * ny + nj) * nx + ni;
            const float nd = (v < 0) ? (v - nb[n].w) : (v + nb[n].w);
            if (fabsf(nd) < fabsf(d[nidx]) - 0.001f) {
                d[nidx] = nd;
                if (push(&q, nidx)) { free(temp); free(q.v); return -1; }
            }
        }
    }
    free(q.v);
    sdf_smooth(d, temp, nx, ny, nz, cs);
    free(temp);
    return 0;
}

/* magnitude first, then the negative sign on equal magnitudes */
static int better(float cand, float cur) {
    const float a = fabsf(cand), b = fabsf(cur);
    return a < b || (a == b && cand < 0.0f && !(cur < 0.0f));
}

int ao_sdf_exact(const uint8_t* mask, int nx, int ny, int nz, const float cs[3], float* d) {
    if (!mask || !d || nx <= 0 || ny <= 0 || nz <= 0) return -1;
    const int64_t total = (int64_t)nx * ny * nz;
    float* temp = (float*)malloc((size_t)total * sizeof(float));
    int64_t* seeds = (int64_t*)malloc((size_t)total * sizeof(int64_t));
    uint8_t* queued = (uint8_t*)calloc((size_t)total, 1);
    i64vec q = {0, 0, 0};
    if (!temp || !seeds || !queued) { free(temp); free(seeds); free(queued); return -1; }
    const int64_t ns = sdf_seed(mask, nx, ny, nz, cs, d, seeds);
    for (int64_t s = 0; s < ns; ++s) {
        if (push(&q, seeds[s])) { free(temp); free(seeds); free(queued); free(q.v); return -1; }
        queued[seeds[s]] = 1;
    }
    free(seeds);
    sdf_nb nb[26];
    sdf_neighbours(cs, nb);
    /* label-correcting queue (circular reuse of the vector as a FIFO) */
    int64_t head = 0;
    while (head < q.n) {
        const int64_t idx = q.v[head++];
        queued[idx] = 0;
        const int i = (int)(idx % nx);
        const int j = (int)((idx / nx) % ny);
        const int k = (int)(idx / ((int64_t)nx * ny));
        const float v = d[idx];
        for (int n = 0; n < 26; ++n) {
            const int ni = i + nb[n].dx, nj = j + nb[n].dy, nk = k + nb[n].dz;
            if (ni < 0 || ni >= nx || nj < 0 || nj >= ny || nk < 0 || nk >= nz) continue;
            const int64_t nidx = ((int64_t)nk * ny + nj) * nx + ni;
            const float nd = (v < 0) ? (v - nb[n].w) : (v + nb[n].w);
            if (better(nd, d[nidx])) {
                d[nidx] = nd;
                if (!queued[nidx]) {
                    queued[nidx] = 1;
                    if (push(&q, nidx)) { free(temp); free(queued); free(q.v); return -1; }
                }
            }
        }
        if (head > (1 << 22) && head * 2 > q.n) {   /* compact the consumed front */
            memmove(q.v, q.v + head, (size_t)(q.n - head) * sizeof(int64_t));
            q.n -= head;
            head = 0;
        }
    }
    free(q.v);
    free(queued);
    sdf_smooth(d, temp, nx, ny, nz, cs);
    free(temp);
    return 0;
}

/* ---- samplers: sampleSDFCPU and sdfNormalCPU (voxel_grid.cpp:32-123) ---- */

typedef struct {
    const float* d;
    int nx, ny, nz;
    float min[3], cs[3];
} sdf_view;

static int valid_f(float v) { return isfinite(v) && fabsf(v) < 1e6f; }

/* (int)floorf(v) for |v| below 2^30; larger magnitudes map to +-2^30, which
 * every caller treats as outside the grid (the reference's (int) conversion
 * of such values is undefined in C; both land outside). */
static int ifloor(float v) {
    const float f = floorf(v);
    if (!(f > -1073741824.0f)) return -1073741824;
    if (!(f < 1073741824.0f)) return 1073741824;
    return (int)f;
}

static float sdf_get(const sdf_view* g, int x, int y, int z) {
    if (x < 0 || x >= g->nx || y < 0 || y >= g->ny || z < 0 || z >= g->nz) return 1000.0f;
    const float v = g->d[((int64_t)z * g->ny + y) * g->nx + x];
    return valid_f(v) ? v : 1000.0f;
}

static float sdf_sample1(const sdf_view* g, float px, float py, float pz) {
    if (!valid_f(px) || !valid_f(py) || !valid_f(pz)) return 1000.0f;
    float csx = g->cs[0], csy = g->cs[1], csz = g->cs[2];
    if (!valid_f(csx) || fabsf(csx) < 1e-8f) return 1000.0f;
    if (!valid_f(csy) || fabsf(csy) < 1e-8f) csy = csx;
    if (!valid_f(csz) || fabsf(csz) < 1e-8f) csz = csx;
    const float fx = (px - g->min[0]) / csx - 0.5f;
    const float fy = (py - g->min[1]) / csy - 0.5f;
    const float fz = (pz - g->min[2]) / csz - 0.5f;
    const int ix0 = ifloor(fx), iy0 = ifloor(fy), iz0 = ifloor(fz);
    const int ix1 = ix0 + 1, iy1 = iy0 + 1, iz1 = iz0 + 1;
    float tx = fx - ix0, ty = fy - iy0, tz = fz - iz0;
    tx = fminf(fmaxf(tx, 0.0f), 1.0f);
    ty = fminf(fmaxf(ty, 0.0f), 1.0f);
    tz = fminf(fmaxf(tz, 0.0f), 1.0f);
    if (ix0 < 0 || iy0 < 0 || iz0 < 0 || ix1 >= g->nx || iy1 >= g->ny || iz1 >= g->nz) {
        const int ix = ifloor((px - g->min[0]) / csx);
        const int iy = ifloor((py - g->min[1]) / csy);
        const int iz = ifloor((pz - g->min[2]) / csz);
        if (ix < 0 || ix >= g->nx || iy < 0 || iy >= g->ny || iz < 0 || iz >= g->nz) return 1000.0f;
        return g->d[((int64_t)iz * g->ny + iy) * g->nx + ix];
    }
    const float c000 = sdf_get(g, ix0, iy0, iz0), c100 = sdf_get(g, ix1, iy0, iz0);
    const float c010 = sdf_get(g, ix0, iy1, iz0), c110 = sdf_get(g, ix1, iy1, iz0);
    const float c001 = sdf_get(g, ix0, iy0, iz1), c101 = sdf_get(g, ix1, iy0, iz1);
    const float c011 = sdf_get(g, ix0, iy1, iz1), c111 = sdf_get(g, ix1, iy1, iz1);
    const float c00 = c000 * (1 - tx) + c100 * tx;
    const float c10 = c010 * (1 - tx) + c110 * tx;
    const float c01 = c001 * (1 - tx) + c101 * tx;
    const float c11 = c011 * (1 - tx) + c111 * tx;
    const float c0 = c00 * (1 - ty) + c10 * ty;
    const float c1 = c01 * (1 - ty) + c11 * ty;
    return c0 * (1 - tz) + c1 * tz;
}

static float sdf_get0(const sdf_view* g, int x, int y, int z) {
    if (x < 0 || x >= g->nx || y < 0 || y >= g->ny || z < 0 || z >= g->nz) return 0.0f;
    const float v = g->d[((int64_t)z * g->ny + y) * g->nx + x];
    return valid_f(v) ? v : 0.0f;
}

static void sdf_normal1(const sdf_view* g, float px, float py, float pz, float* n3) {
    n3[0] = 0.0f; n3[1] = 1.0f; n3[2] = 0.0f;
    if (g->nx <= 1 || g->ny <= 1 || g->nz <= 1) return;
    if (!valid_f(px) || !valid_f(py) || !valid_f(pz)) return;
    float csx = g->cs[0], csy = g->cs[1], csz = g->cs[2];
    if (!valid_f(csx) || fabsf(csx) < 1e-8f) return;
    if (!valid_f(csy) || fabsf(csy) < 1e-8f) csy = csx;
    if (!valid_f(csz) || fabsf(csz) < 1e-8f) csz = csx;
    float eps = fminf(csx, fminf(csy, csz)) * 0.5f;
    if (eps < 1e-4f) eps = 0.01f;
    float dx = sdf_sample1(g, px + eps, py, pz) - sdf_sample1(g, px - eps, py, pz);
    float dy = sdf_sample1(g, px, py + eps, pz) - sdf_sample1(g, px, py - eps, pz);
    float dz = sdf_sample1(g, px, py, pz + eps) - sdf_sample1(g, px, py, pz - eps);
    float len = sqrtf(dx * dx + dy * dy + dz * dz);
    if (!valid_f(len) || len < 1e-6f) {
        const int ix = ifloor((px - g->min[0]) / csx);
        const int iy = ifloor((py - g->min[1]) / csy);
        const int iz = ifloor((pz - g->min[2]) / csz);
        if (ix <= 0 || ix >= g->nx - 1 || iy <= 0 || iy >= g->ny - 1 || iz <= 0 || iz >= g->nz - 1) return;
        dx = sdf_get0(g, ix + 1, iy, iz) - sdf_get0(g, ix - 1, iy, iz);
        dy = sdf_get0(g, ix, iy + 1, iz) - sdf_get0(g, ix, iy - 1, iz);
        dz = sdf_get0(g, ix, iy, iz + 1) - sdf_get0(g, ix, iy, iz - 1);
        len = sqrtf(dx * dx + dy * dy + dz * dz);
        if (len < 1e-6f) return;
    }
    n3[0] = dx / len; n3[1] = dy / len; n3[2] = dz / len;
}

int ao_sdf_sample(const float* sdf, int nx, int ny, int nz, const float mn[3], const float cs[3], const float* pts,
                  int64_t n, float* dist, float* normal) {
    if (nx <= 0 || ny <= 0 || nz <= 0) {   /* no field: sampleSDFCPU's 1000, the default normal */
        for (int64_t i = 0; i < n; ++i) {
            if (dist) dist[i] = 1000.0f;
            if (normal) { normal[3 * i] = 0.0f; normal[3 * i + 1] = 1.0f; normal[3 * i + 2] = 0.0f; }
        }
        return 0;
    }
    sdf_view g = {sdf, nx, ny, nz, {mn[0], mn[1], mn[2]}, {cs[0], cs[1], cs[2]}};
    for (int64_t i = 0; i < n; ++i) {
        if (dist) dist[i] = sdf_sample1(&g, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        if (normal) sdf_normal1(&g, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], normal + 3 * i);
    }
    return 0;
}
