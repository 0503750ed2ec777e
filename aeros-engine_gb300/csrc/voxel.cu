// voxel.cu — voxelizer: solid mask of a closed triangle mesh at the grid's
// cell centres (the mask loop of buildVoxelGrid,
// aeros/src/voxel_grid.cpp:337-351, and its inside test, mesh_bvh.h:168-185).
//
// The reference's decision per cell: three axis rays from jittered origins,
// parity of the double-precision Moller-Trumbore hits with t > 1e-7 (mesh_bvh.h:
// 62-96), majority of the three. Its BVH only culls work: a node is skipped
// when the ray's perpendicular coordinates lie strictly outside the node box
// (or the box lies behind the origin), which no hit needs, so the count is
// the count over all triangles.
//
// Design here (rows, not cells): every cell of a grid row shares its ray's two
// perpendicular origin coordinates (the jitter is per axis, not per cell), and
// with an axis-aligned direction the determinant, u and v of the triangle test
// do not depend on the origin's coordinate along the ray (their terms in it are
// multiplied by the direction's exact zeros). So one traversal per row finds
// the triangles whose (det, u, v) pass; each cell then only evaluates t for
// those candidates — the same expression tree as the full test, hence the same
// decision bit for bit. Rows with more candidates than a row holds fall back to
// the per-cell traversal.
//
// The BVH: Morton codes (10 bits per axis) of the triangle centroids over their
// bounding box, sorted; ranges split at the highest bit in which their first and
// last codes differ (at the middle when the codes are equal), leaves of at most
// four triangles; the children of a node are stored side by side. Boxes are the
// exact float min / max of the triangles' vertices. Built on the host.
//
// Compiled with --fmad=false: every float and double operation of the triangle
// test and the cell centres rounds as in the reference's x86-64 build.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/aeros_lbm.h"

namespace aeros {

struct HTri {
    float v[9];
};
// 32 bytes. Leaf: a = first triangle, b = count (> 0). Inner: a = index of the
// left child (the right child is a + 1), b = 0.
struct DNode {
    float mn[3], mx[3];
    int a, b;
};

namespace {

// The reference's triangle filter (mesh_bvh.h:40-53 and voxel_grid.cpp:313-325):
// finite vertices, twice the area (glm::length of the edge cross product, in its
// operand order) above 1e-14. The mask depends on which triangles are kept.
bool keep_tri(const float* t) {
    for (int j = 0; j < 9; ++j)
        if (!std::isfinite(t[j])) return false;
    const float e1x = t[3] - t[0], e1y = t[4] - t[1], e1z = t[5] - t[2];
    const float e2x = t[6] - t[0], e2y = t[7] - t[1], e2z = t[8] - t[2];
    const float cx = e1y * e2z - e2y * e1z, cy = e1z * e2x - e2z * e1x, cz = e1x * e2y - e2x * e1y;
    const float area2 = sqrtf(cx * cx + cy * cy + cz * cz);
    return area2 > 1e-14f && std::isfinite(area2);
}

uint32_t spread10(uint32_t v) {   // bits 0..9 -> bits 0, 3, 6, ..., 27
    v &= 1023u;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

constexpr int LEAF = 4;
constexpr int MAX_DEPTH = 60;   // Morton splits end within 30 levels, equal codes within log2(n)

struct MortonBvh {
    std::vector<HTri> tris;       // sorted by Morton code
    std::vector<uint32_t> code;
    std::vector<DNode> nodes;
    int depth = 0;

    void box_of(int start, int count, DNode& n) const {
        for (int a = 0; a < 3; ++a) {
            n.mn[a] = INFINITY;
            n.mx[a] = -INFINITY;
        }
        for (int i = start; i < start + count; ++i)
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) {
                    const float v = tris[i].v[3 * k + a];
                    n.mn[a] = std::min(n.mn[a], v);
                    n.mx[a] = std::max(n.mx[a], v);
                }
    }

    int split_of(int start, int count) const {
        const uint32_t c0 = code[start], c1 = code[start + count - 1];
        if (c0 == c1) return start + count / 2;
        const int bit = 31 - __builtin_clz(c0 ^ c1);
        // first index whose code has `bit` set (the codes are sorted)
        const uint32_t* lo = code.data() + start;
        const uint32_t* p = std::partition_point(lo, lo + count, [&](uint32_t c) { return !((c >> bit) & 1u); });
        return start + (int)(p - lo);
    }

    // Fills node `ni` for triangles [start, start + count).
    void build(int ni, int start, int count, int d) {
        depth = std::max(depth, d);
        if (count <= LEAF || d >= MAX_DEPTH) {
            box_of(start, count, nodes[ni]);
            nodes[ni].a = start;
            nodes[ni].b = count;
            return;
        }
        const int mid = split_of(start, count);
        const int left = (int)nodes.size();
        nodes.push_back(DNode{});
        nodes.push_back(DNode{});
        build(left, start, mid - start, d + 1);
        build(left + 1, mid, start + count - mid, d + 1);
        DNode& n = nodes[ni];
        const DNode &l = nodes[left], &r = nodes[left + 1];
        for (int a = 0; a < 3; ++a) {
            n.mn[a] = std::min(l.mn[a], r.mn[a]);
            n.mx[a] = std::max(l.mx[a], r.mx[a]);
        }
        n.a = left;
        n.b = 0;
    }

    void make(const float* in, int64_t ntri) {
        std::vector<HTri> kept;
        kept.reserve((size_t)std::max<int64_t>(ntri, 0));
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t i = 0; i < ntri; ++i) {
            const float* t = in + 9 * i;
            if (!keep_tri(t)) continue;
            HTri h;
            memcpy(h.v, t, sizeof(h.v));
            kept.push_back(h);
            for (int a = 0; a < 3; ++a) {
                const float c = (t[a] + t[3 + a] + t[6 + a]) / 3.0f;
                lo[a] = std::min(lo[a], c);
                hi[a] = std::max(hi[a], c);
            }
        }
        const size_t n = kept.size();
        nodes.clear();
        tris.clear();
        code.clear();
        if (!n) return;
        std::vector<std::pair<uint32_t, uint32_t>> key(n);
        for (size_t i = 0; i < n; ++i) {
            uint32_t m = 0;
            for (int a = 0; a < 3; ++a) {
                const float c = (kept[i].v[a] + kept[i].v[3 + a] + kept[i].v[6 + a]) / 3.0f;
                const float ext = hi[a] - lo[a];
                int q = ext > 0.0f ? (int)((c - lo[a]) / ext * 1024.0f) : 0;
                q = std::min(1023, std::max(0, q));
                m |= spread10((uint32_t)q) << (2 - a);
            }
            key[i] = {m, (uint32_t)i};
        }
        std::sort(key.begin(), key.end());   // ties by input order: deterministic
        tris.resize(n);
        code.resize(n);
        for (size_t i = 0; i < n; ++i) {
            tris[i] = kept[key[i].second];
            code[i] = key[i].first;
        }
        nodes.reserve(2 * (n / 2 + 1));
        nodes.push_back(DNode{});
        depth = 0;
        build(0, 0, (int)n, 0);
    }
};

// ---- device ------------------------------------------------------------------
// Moller-Trumbore in double, as mesh_bvh.h:62-96 (minT 1e-7, maxT 1e30).
__device__ __forceinline__ bool ray_tri(const float o[3], const float d[3], const float* v) {
    const double e1x = (double)v[3] - v[0], e1y = (double)v[4] - v[1], e1z = (double)v[5] - v[2];
    const double e2x = (double)v[6] - v[0], e2y = (double)v[7] - v[1], e2z = (double)v[8] - v[2];
    const double dx = d[0], dy = d[1], dz = d[2];
    const double px = dy * e2z - dz * e2y;
    const double py = dz * e2x - dx * e2z;
    const double pz = dx * e2y - dy * e2x;
    const double det = e1x * px + e1y * py + e1z * pz;
    const double scale = fabs(e1x * e2y - e1y * e2x) + fabs(e1y * e2z - e1z * e2y) + fabs(e1z * e2x - e1x * e2z) + 1e-30;
    if (fabs(det) < 1e-12 * scale) return false;
    const double inv = 1.0 / det;
    const double tx = (double)o[0] - v[0], ty = (double)o[1] - v[1], tz = (double)o[2] - v[2];
    const double u = (tx * px + ty * py + tz * pz) * inv;
    if (u < 0.0 || u > 1.0) return false;
    const double qx = ty * e1z - tz * e1y;
    const double qy = tz * e1x - tx * e1z;
    const double qz = tx * e1y - ty * e1x;
    const double vv = (dx * qx + dy * qy + dz * qz) * inv;
    if (vv < 0.0 || u + vv > 1.0) return false;
    const double t = (e2x * qx + e2y * qy + e2z * qz) * inv;
    if (!(t > 1e-7) || t >= 1e30) return false;
    return true;
}

// The part of ray_tri that does not depend on the origin's coordinate along
// an axis-aligned direction: whether u and v place the line inside.
__device__ __forceinline__ bool line_tri(const float o[3], const float d[3], const float* v) {
    const double e1x = (double)v[3] - v[0], e1y = (double)v[4] - v[1], e1z = (double)v[5] - v[2];
    const double e2x = (double)v[6] - v[0], e2y = (double)v[7] - v[1], e2z = (double)v[8] - v[2];
    const double dx = d[0], dy = d[1], dz = d[2];
    const double px = dy * e2z - dz * e2y;
    const double py = dz * e2x - dx * e2z;
    const double pz = dx * e2y - dy * e2x;
    const double det = e1x * px + e1y * py + e1z * pz;
    const double scale = fabs(e1x * e2y - e1y * e2x) + fabs(e1y * e2z - e1z * e2y) + fabs(e1z * e2x - e1x * e2z) + 1e-30;
    if (fabs(det) < 1e-12 * scale) return false;
    const double inv = 1.0 / det;
    const double tx = (double)o[0] - v[0], ty = (double)o[1] - v[1], tz = (double)o[2] - v[2];
    const double u = (tx * px + ty * py + tz * pz) * inv;
    if (u < 0.0 || u > 1.0) return false;
    const double qx = ty * e1z - tz * e1y;
    const double qy = tz * e1x - tx * e1z;
    const double qz = tx * e1y - ty * e1x;
    const double vv = (dx * qx + dy * qy + dz * qz) * inv;
    return !(vv < 0.0 || u + vv > 1.0);
}

// Perpendicular culling of an axis-aligned line: the point (o_b, o_c) lies in
// the node box's [mn, mx] on both other axes (exact float comparisons, what
// the reference's slab test decides for those axes).
__device__ __forceinline__ bool box_line(const DNode& n, const float o[3], int axis) {
    const int b = axis == 0 ? 1 : 0, c = axis == 2 ? 1 : 2;
    return !(o[b] < n.mn[b] || o[b] > n.mx[b] || o[c] < n.mn[c] || o[c] > n.mx[c]);
}

// The same for the ray from o: also skip boxes entirely behind the origin.
__device__ __forceinline__ bool box_ray(const DNode& n, const float o[3], int axis) {
    const int b = axis == 0 ? 1 : 0, c = axis == 2 ? 1 : 2;
    if (o[b] < n.mn[b] || o[b] > n.mx[b] || o[c] < n.mn[c] || o[c] > n.mx[c]) return false;
    return n.mx[axis] - o[axis] >= 0.0f;
}

constexpr int STACK = 64;   // > MAX_DEPTH + 1: a depth-first stack holds at most depth + 1 nodes
constexpr int ROW_CAP = 32; // candidate triangles kept per row

// Per-cell traversal (rows whose candidates overflow, and the fixed-scratch
// entry point): hit count along +axis from o, -1 on stack overflow.
__device__ int count_hits(const DNode* nodes, const float* tris, const float o[3], int axis) {
    const float d[3] = {axis == 0 ? 1.0f : 0.0f, axis == 1 ? 1.0f : 0.0f, axis == 2 ? 1.0f : 0.0f};
    int stack[STACK];
    int sp = 0, hits = 0;
    if (!box_ray(nodes[0], o, axis)) return 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const DNode n = nodes[stack[--sp]];
        if (n.b > 0) {
            for (int i = 0; i < n.b; ++i)
                if (ray_tri(o, d, tris + 9 * (long long)(n.a + i))) ++hits;
            continue;
        }
        for (int k = 0; k < 2; ++k)
            if (box_ray(nodes[n.a + k], o, axis)) {
                if (sp >= STACK) return -1;
                stack[sp++] = n.a + k;
            }
    }
    return hits;
}

struct RowGrid {
    aeros_voxel_grid g;
    int rows[3];        // rows of each ray family: ny*nz, nx*nz, nx*ny
};

__device__ __forceinline__ void centre(const aeros_voxel_grid& g, int i, int j, int k, float p[3]) {
    p[0] = g.min[0] + (i + 0.5f) * g.cell[0];
    p[1] = g.min[1] + (j + 0.5f) * g.cell[1];
    p[2] = g.min[2] + (k + 0.5f) * g.cell[2];
}

// Ray origins of cell (i, j, k), mesh_bvh.h:168-185: jitter 1e-3 cell times
// (0.731, 0.377, 0.557), applied per axis as the reference does.
__device__ __forceinline__ void origin(const aeros_voxel_grid& g, int axis, int i, int j, int k, float o[3]) {
    float p[3];
    centre(g, i, j, k, p);
    const float jx = 0.731f * 1e-3f * g.cell[0], jy = 0.377f * 1e-3f * g.cell[1], jz = 0.557f * 1e-3f * g.cell[2];
    if (axis == 0) { o[0] = p[0]; o[1] = p[1] + jy; o[2] = p[2] + jz; }
    else if (axis == 1) { o[0] = p[0] + jz; o[1] = p[1]; o[2] = p[2] + jx; }
    else { o[0] = p[0] + jy; o[1] = p[1] + jx; o[2] = p[2]; }
}

// Row r of family `axis`: its first cell's indices.
__device__ __forceinline__ void row_cell(const aeros_voxel_grid& g, int axis, int r, int& i, int& j, int& k) {
    if (axis == 0) { i = 0; j = r % g.ny; k = r / g.ny; }
    else if (axis == 1) { i = r % g.nx; j = 0; k = r / g.nx; }
    else { i = r % g.nx; j = r / g.nx; k = 0; }
}

// One thread per row of the three families: the triangles whose (det, u, v)
// pass for the row's line; rows[] = count (> ROW_CAP: overflow), then ids.
__global__ void k_row_candidates(const DNode* nodes, const float* tris, RowGrid rg, int* rows) {
    const int total = rg.rows[0] + rg.rows[1] + rg.rows[2];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int axis = t < rg.rows[0] ? 0 : (t < rg.rows[0] + rg.rows[1] ? 1 : 2);
        const int r = t - (axis > 0 ? rg.rows[0] : 0) - (axis > 1 ? rg.rows[1] : 0);
        int i, j, k;
        row_cell(rg.g, axis, r, i, j, k);
        float o[3];
        origin(rg.g, axis, i, j, k, o);
        const float d[3] = {axis == 0 ? 1.0f : 0.0f, axis == 1 ? 1.0f : 0.0f, axis == 2 ? 1.0f : 0.0f};
        int* out = rows + (long long)t * (ROW_CAP + 1);
        int cnt = 0;
        int stack[STACK];
        int sp = 0;
        if (box_line(nodes[0], o, axis)) stack[sp++] = 0;
        while (sp > 0) {
            const DNode n = nodes[stack[--sp]];
            if (n.b > 0) {
                for (int m = 0; m < n.b; ++m)
                    if (line_tri(o, d, tris + 9 * (long long)(n.a + m))) {
                        if (cnt < ROW_CAP) out[1 + cnt] = n.a + m;
                        ++cnt;
                    }
                continue;
            }
            for (int c = 0; c < 2; ++c)
                if (box_line(nodes[n.a + c], o, axis)) {
                    if (sp >= STACK) { cnt = ROW_CAP + 1; sp = 0; break; }   // overflow: per-cell path
                    stack[sp++] = n.a + c;
                }
        }
        out[0] = cnt;
    }
}

// One thread per cell: t of the row's candidates from the cell's own origin
// (the full triangle test, so the decision is the reference's bit for bit).
__global__ void k_voxelize_rows(const DNode* nodes, const float* tris, RowGrid rg, const int* rows, uint8_t* mask,
                                int* overflow) {
    const aeros_voxel_grid& g = rg.g;
    const long long total = (long long)g.nx * g.ny * g.nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % g.nx);
        const long long q = c / g.nx;
        const int j = (int)(q % g.ny), k = (int)(q / g.ny);
        int votes = 0;
#pragma unroll 1
        for (int axis = 0; axis < 3; ++axis) {
            const long long r = axis == 0 ? (long long)k * g.ny + j
                              : axis == 1 ? (long long)rg.rows[0] + (long long)k * g.nx + i
                                          : (long long)rg.rows[0] + rg.rows[1] + (long long)j * g.nx + i;
            const int* row = rows + r * (ROW_CAP + 1);
            float o[3];
            origin(g, axis, i, j, k, o);
            int hits;
            const int cnt = row[0];
            if (cnt <= ROW_CAP) {
                const float d[3] = {axis == 0 ? 1.0f : 0.0f, axis == 1 ? 1.0f : 0.0f, axis == 2 ? 1.0f : 0.0f};
                hits = 0;
                for (int m = 0; m < cnt; ++m) hits += ray_tri(o, d, tris + 9 * (long long)row[1 + m]) ? 1 : 0;
            } else {
                hits = count_hits(nodes, tris, o, axis);
                if (hits < 0) { atomicExch(overflow, 1); hits = 0; }
            }
            votes += hits & 1;
        }
        mask[c] = votes >= 2 ? 1 : 0;
    }
}

// One thread per cell, per-cell traversal of all three rays.
__global__ void k_voxelize_cells(const DNode* nodes, const float* tris, aeros_voxel_grid g, uint8_t* mask,
                                 int* overflow) {
    const long long total = (long long)g.nx * g.ny * g.nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % g.nx);
        const long long q = c / g.nx;
        const int j = (int)(q % g.ny), k = (int)(q / g.ny);
        int votes = 0;
        for (int axis = 0; axis < 3; ++axis) {
            float o[3];
            origin(g, axis, i, j, k, o);
            const int h = count_hits(nodes, tris, o, axis);
            if (h < 0) atomicExch(overflow, 1);
            votes += h & 1;
        }
        mask[c] = votes >= 2 ? 1 : 0;
    }
}

int grid_blocks(long long work, int threads, int per_sm) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long b = (work + threads - 1) / threads;
    return (int)std::max<long long>(1, std::min<long long>(b, (long long)std::max(1, sms) * per_sm));
}

}  // namespace

// Returns AEROS_OK or a negative status; messages through `err`.
int voxelize_impl(const float* tris, int64_t ntri, const aeros_voxel_grid* g, uint8_t* d_mask, cudaStream_t s,
                  char* err, size_t errn) {
    MortonBvh bvh;
    bvh.make(tris, ntri);
    const long long total = (long long)g->nx * g->ny * g->nz;
    if (bvh.tris.empty()) {
        cudaError_t e = cudaMemsetAsync(d_mask, 0, (size_t)total, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { snprintf(err, errn, "memset: %s", cudaGetErrorString(e)); return AEROS_ERR_CUDA; }
        return AEROS_OK;
    }
    RowGrid rg;
    rg.g = *g;
    rg.rows[0] = g->ny * g->nz;
    rg.rows[1] = g->nx * g->nz;
    rg.rows[2] = g->nx * g->ny;
    const long long nrows = (long long)rg.rows[0] + rg.rows[1] + rg.rows[2];
    DNode* dn = nullptr;
    float* dt = nullptr;
    int *dof = nullptr, *drows = nullptr;
    const size_t nb = bvh.nodes.size() * sizeof(DNode), tb = bvh.tris.size() * sizeof(HTri);
    // stream-ordered scratch: voxelizing does not wait for other streams' work
    cudaError_t e = cudaMallocAsync((void**)&dn, nb, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dt, tb, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dof, 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&drows, (size_t)nrows * (ROW_CAP + 1) * sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dn, bvh.nodes.data(), nb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, bvh.tris.data(), tb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dof, 0, 4, s);
    if (e == cudaSuccess) {
        k_row_candidates<<<grid_blocks(nrows, 128, 16), 128, 0, s>>>(dn, dt, rg, drows);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_voxelize_rows<<<grid_blocks(total, 128, 16), 128, 0, s>>>(dn, dt, rg, drows, d_mask, dof);
        e = cudaGetLastError();
    }
    int overflow = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&overflow, dof, 4, cudaMemcpyDeviceToHost, s);
    if (dn) cudaFreeAsync(dn, s);
    if (dt) cudaFreeAsync(dt, s);
    if (dof) cudaFreeAsync(dof, s);
    if (drows) cudaFreeAsync(drows, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { snprintf(err, errn, "voxelize: %s", cudaGetErrorString(e)); return AEROS_ERR_CUDA; }
    if (overflow) { snprintf(err, errn, "voxelize: BVH traversal stack overflow"); return AEROS_ERR_UNSUPPORTED; }
    return AEROS_OK;
}

// ---- voxelizing without device allocation -----------------------------------
// Callers that cannot allocate device memory while they voxelize: a serving
// loop that has handed its whole HBM budget to resident domains (an extra
// allocation can fail mid-session), and a caller whose other streams must not
// be stalled by the device-wide synchronization cudaFree implies. The BVH,
// the triangles and the overflow flag go to one fixed device array instead,
// VOXEL_SCRATCH_BYTES long (24 MiB: the level-7 icosphere's 327,680 triangles
// fit, about 36 bytes per triangle plus 32 per BVH node); a mesh needing more
// is rejected before any device work. The array exists in every context that
// loads this library, from module load on, whether or not the entry point is
// called. It is shared by every call on a device, so calls must not overlap
// (each call returns after its work has completed on the caller's stream).
constexpr size_t VOXEL_SCRATCH_BYTES = size_t(24) << 20;
static __device__ __align__(256) unsigned char g_voxel_scratch[VOXEL_SCRATCH_BYTES];

namespace {
size_t align256(size_t v) { return (v + 255) & ~size_t(255); }
}  // namespace

int voxelize_noalloc_impl(const float* tris, int64_t ntri, const aeros_voxel_grid* g, uint8_t* d_mask,
                          cudaStream_t s, char* err, size_t errn) {
    if ((size_t)ntri * sizeof(HTri) > VOXEL_SCRATCH_BYTES) {
        snprintf(err, errn, "%lld triangles exceed the %zu-byte voxelizer scratch", (long long)ntri, VOXEL_SCRATCH_BYTES);
        return AEROS_ERR_INVALID;
    }
    MortonBvh bvh;
    bvh.make(tris, ntri);
    const long long total = (long long)g->nx * g->ny * g->nz;
    if (bvh.tris.empty()) {
        cudaError_t e = cudaMemsetAsync(d_mask, 0, (size_t)total, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { snprintf(err, errn, "memset: %s", cudaGetErrorString(e)); return AEROS_ERR_CUDA; }
        return AEROS_OK;
    }
    // layout: overflow flag | nodes | triangles, each 256-byte aligned
    const size_t off_nodes = 256;
    const size_t off_tris = align256(off_nodes + bvh.nodes.size() * sizeof(DNode));
    const size_t need = off_tris + bvh.tris.size() * sizeof(HTri);
    if (need > VOXEL_SCRATCH_BYTES) {
        snprintf(err, errn, "mesh needs %zu bytes of the %zu-byte voxelizer scratch", need, VOXEL_SCRATCH_BYTES);
        return AEROS_ERR_INVALID;
    }
    // the array's device address in the current context, looked up on every
    // call (the host-side symbol is not a device address; a lookup allocates
    // nothing and stays valid across context re-creation)
    void* base = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&base, g_voxel_scratch);
    if (e != cudaSuccess || !base) {
        snprintf(err, errn, "scratch symbol: %s", cudaGetErrorString(e));
        return AEROS_ERR_CUDA;
    }
    unsigned char* sc = static_cast<unsigned char*>(base);
    int* dof = reinterpret_cast<int*>(sc);
    DNode* dn = reinterpret_cast<DNode*>(sc + off_nodes);
    float* dt = reinterpret_cast<float*>(sc + off_tris);
    e = cudaMemsetAsync(dof, 0, sizeof(int), s);   // the flag starts at zero
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dn, bvh.nodes.data(), bvh.nodes.size() * sizeof(DNode), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dt, bvh.tris.data(), bvh.tris.size() * sizeof(HTri), cudaMemcpyHostToDevice, s);
    int overflow = 0;
    if (e == cudaSuccess) {
        k_voxelize_cells<<<grid_blocks(total, 128, 16), 128, 0, s>>>(dn, dt, *g, d_mask, dof);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&overflow, dof, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { snprintf(err, errn, "voxelize: %s", cudaGetErrorString(e)); return AEROS_ERR_CUDA; }
    if (overflow) { snprintf(err, errn, "voxelize: BVH traversal stack overflow"); return AEROS_ERR_UNSUPPORTED; }
    return AEROS_OK;
}

}  // namespace aeros
