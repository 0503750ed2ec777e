// voxel.cu — BVH voxelizer: solid mask of a closed triangle mesh at the
// grid's cell centres (the mask loop of buildVoxelGrid,
// aeros/src/voxel_grid.cpp:337-351).
//
// Host: finite / non-degenerate filter (voxel_grid.cpp:313-325,
// mesh_bvh.h:50-53) and a median-split BVH, leaf size 4, depth limit 48
// (mesh_bvh.h:219-266), built with std::nth_element so the tree has the same
// shape as the reference's. Device: one thread per cell, three axis rays from
// jittered origins, hit parity, majority vote (mesh_bvh.h:168-185); float slab
// culling and the double-precision Moller-Trumbore test (mesh_bvh.h:62-96,
// 198-217). Compiled with --fmad=false: every float and double operation
// rounds as in the reference's x86-64 build, so the mask is bit-exact.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/aeros_lbm.h"

namespace aeros {

struct HTri {
    float v[9];
    float mn[3], mx[3], cen[3];
};
struct DNode {
    float mn[3], mx[3];
    int left, right, start, count;
};

namespace {

inline float fmin_glm(float a, float b) { return (b < a) ? b : a; }
inline float fmax_glm(float a, float b) { return (a < b) ? b : a; }

// makeTriangle / isDegenerate (mesh_bvh.h:40-53) with glm's operand order
bool make_tri(const float* t, HTri& o) {
    for (int j = 0; j < 9; ++j)
        if (!std::isfinite(t[j])) return false;
    memcpy(o.v, t, sizeof(o.v));
    const float e1x = t[3] - t[0], e1y = t[4] - t[1], e1z = t[5] - t[2];
    const float e2x = t[6] - t[0], e2y = t[7] - t[1], e2z = t[8] - t[2];
    const float cx = e1y * e2z - e2y * e1z, cy = e1z * e2x - e2z * e1x, cz = e1x * e2y - e2x * e1y;
    const float area2 = sqrtf(cx * cx + cy * cy + cz * cz);
    if (!(area2 > 1e-14f) || !std::isfinite(area2)) return false;
    for (int a = 0; a < 3; ++a) {
        o.mn[a] = fmin_glm(t[a], fmin_glm(t[3 + a], t[6 + a]));
        o.mx[a] = fmax_glm(t[a], fmax_glm(t[3 + a], t[6 + a]));
        o.cen[a] = (t[a] + t[3 + a] + t[6 + a]) * (1.0f / 3.0f);
    }
    return true;
}

struct Builder {
    std::vector<HTri>& tris;
    std::vector<DNode> nodes;
    explicit Builder(std::vector<HTri>& t) : tris(t) {}
    int build(int start, int count, int depth) {
        const int index = (int)nodes.size();
        nodes.push_back(DNode{});
        float lo[3], hi[3], cmin[3], cmax[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = tris[start].mn[a]; hi[a] = tris[start].mx[a];
            cmin[a] = cmax[a] = tris[start].cen[a];
        }
        for (int i = start + 1; i < start + count; ++i)
            for (int a = 0; a < 3; ++a) {
                lo[a] = fmin_glm(lo[a], tris[i].mn[a]);
                hi[a] = fmax_glm(hi[a], tris[i].mx[a]);
                cmin[a] = fmin_glm(cmin[a], tris[i].cen[a]);
                cmax[a] = fmax_glm(cmax[a], tris[i].cen[a]);
            }
        for (int a = 0; a < 3; ++a) { nodes[index].mn[a] = lo[a]; nodes[index].mx[a] = hi[a]; }
        nodes[index].left = nodes[index].right = -1;
        if (count <= 4 || depth >= 48) {
            nodes[index].start = start;
            nodes[index].count = count;
            return index;
        }
        const float ext[3] = {cmax[0] - cmin[0], cmax[1] - cmin[1], cmax[2] - cmin[2]};
        int axis = 0;
        if (ext[1] > ext[0]) axis = 1;
        if (ext[2] > ext[axis]) axis = 2;
        if (!(ext[axis] > 1e-12f)) {
            nodes[index].start = start;
            nodes[index].count = count;
            return index;
        }
        const int mid = count / 2;
        std::nth_element(tris.begin() + start, tris.begin() + start + mid, tris.begin() + start + count,
                         [axis](const HTri& a, const HTri& b) { return a.cen[axis] < b.cen[axis]; });
        const int l = build(start, mid, depth + 1);
        const int r = build(start + mid, count - mid, depth + 1);
        nodes[index].left = l;
        nodes[index].right = r;
        nodes[index].start = 0;
        nodes[index].count = 0;
        return index;
    }
};

__device__ __forceinline__ bool slab(const DNode& n, const float o[3], const float inv[3]) {
    float t0 = -INFINITY, t1 = INFINITY;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float tn = (n.mn[a] - o[a]) * inv[a];
        float tf = (n.mx[a] - o[a]) * inv[a];
        if (tn > tf) { const float t = tn; tn = tf; tf = t; }
        if (isnan(tn) || isnan(tf)) continue;
        if (tn > t0) t0 = tn;
        if (tf < t1) t1 = tf;
        if (t1 < t0) return false;
    }
    return t1 >= 0.0f;
}

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

constexpr int STACK = 64;   // depth limit 48 keeps the stack below 50 entries

// Hit count along +axis; every leaf whose box the ray reaches is visited
// (a count does not depend on the visiting order). Returns -1 on stack
// overflow (not reachable with the depth limit).
__device__ int count_hits(const DNode* nodes, const float* tris, const float o[3], int axis) {
    const float d[3] = {axis == 0 ? 1.0f : 0.0f, axis == 1 ? 1.0f : 0.0f, axis == 2 ? 1.0f : 0.0f};
    const float inv[3] = {axis == 0 ? 1.0f : INFINITY, axis == 1 ? 1.0f : INFINITY, axis == 2 ? 1.0f : INFINITY};
    int stack[STACK];
    int sp = 0;
    if (!slab(nodes[0], o, inv)) return 0;
    stack[sp++] = 0;
    int hits = 0;
    while (sp > 0) {
        const DNode n = nodes[stack[--sp]];
        if (n.count > 0) {
            for (int i = 0; i < n.count; ++i)
                if (ray_tri(o, d, tris + 9 * (long long)(n.start + i))) ++hits;
            continue;
        }
        if (slab(nodes[n.left], o, inv)) {
            if (sp >= STACK) return -1;
            stack[sp++] = n.left;
        }
        if (slab(nodes[n.right], o, inv)) {
            if (sp >= STACK) return -1;
            stack[sp++] = n.right;
        }
    }
    return hits;
}

__global__ void k_voxelize(const DNode* nodes, const float* tris, aeros_voxel_grid g, uint8_t* mask, int* overflow) {
    const long long total = (long long)g.nx * g.ny * g.nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % g.nx);
        const long long r = c / g.nx;
        const int j = (int)(r % g.ny), k = (int)(r / g.ny);
        const float px = g.min[0] + (i + 0.5f) * g.cell[0];
        const float py = g.min[1] + (j + 0.5f) * g.cell[1];
        const float pz = g.min[2] + (k + 0.5f) * g.cell[2];
        const float jx = 0.731f * 1e-3f * g.cell[0], jy = 0.377f * 1e-3f * g.cell[1], jz = 0.557f * 1e-3f * g.cell[2];
        const float o1[3] = {px, py + jy, pz + jz};
        const float o2[3] = {px + jz, py, pz + jx};
        const float o3[3] = {px + jy, py + jx, pz};
        const int h1 = count_hits(nodes, tris, o1, 0);
        const int h2 = count_hits(nodes, tris, o2, 1);
        const int h3 = count_hits(nodes, tris, o3, 2);
        if (h1 < 0 || h2 < 0 || h3 < 0) atomicExch(overflow, 1);
        const int votes = (h1 & 1) + (h2 & 1) + (h3 & 1);
        mask[c] = votes >= 2 ? 1 : 0;
    }
}

}  // namespace

// Returns AEROS_OK or a negative status; messages through `err`.
int voxelize_impl(const float* tris, int64_t ntri, const aeros_voxel_grid* g, uint8_t* d_mask, cudaStream_t s,
                  char* err, size_t errn) {
    std::vector<HTri> tv;
    tv.reserve((size_t)std::max<int64_t>(ntri, 0));
    for (int64_t i = 0; i < ntri; ++i) {
        HTri t;
        if (make_tri(tris + 9 * i, t)) tv.push_back(t);
    }
    const long long total = (long long)g->nx * g->ny * g->nz;
    if (tv.empty()) {
        cudaError_t e = cudaMemsetAsync(d_mask, 0, (size_t)total, s);
        if (e != cudaSuccess) { snprintf(err, errn, "memset: %s", cudaGetErrorString(e)); return AEROS_ERR_CUDA; }
        return AEROS_OK;
    }
    Builder b(tv);
    b.nodes.reserve(tv.size() * 2 / 4 + 2);
    b.build(0, (int)tv.size(), 0);
    std::vector<float> flat(tv.size() * 9);
    for (size_t i = 0; i < tv.size(); ++i) memcpy(&flat[9 * i], tv[i].v, 36);
    DNode* dn = nullptr;
    float* dt = nullptr;
    int* dof = nullptr;
    // stream-ordered scratch: voxelizing does not wait for other streams' work
    cudaError_t e = cudaMallocAsync((void**)&dn, b.nodes.size() * sizeof(DNode), s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dt, flat.size() * 4, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dof, 4, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dn, b.nodes.data(), b.nodes.size() * sizeof(DNode), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, flat.data(), flat.size() * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dof, 0, 4, s);
    int overflow = 0;
    if (e == cudaSuccess) {
        int sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        long long blocks = (total + 127) / 128;
        blocks = std::min<long long>(blocks, (long long)std::max(1, sms) * 16);
        k_voxelize<<<(int)std::max<long long>(1, blocks), 128, 0, s>>>(dn, dt, *g, d_mask, dof);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&overflow, dof, 4, cudaMemcpyDeviceToHost, s);
    if (dn) cudaFreeAsync(dn, s);
    if (dt) cudaFreeAsync(dt, s);
    if (dof) cudaFreeAsync(dof, s);
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
// VOXEL_SCRATCH_BYTES long (24 MiB: up to about 330,000 triangles, the
// level-7 icosphere); a mesh needing more is rejected before any device work.
// The array is shared by every call on a device, so calls must not overlap
// (the caller serializes them: each call returns after its work completed).
// The array's address is looked up once per device on the first call, which
// must therefore come before any stream capture on that device.
constexpr size_t VOXEL_SCRATCH_BYTES = size_t(24) << 20;
static __device__ __align__(256) unsigned char g_voxel_scratch[VOXEL_SCRATCH_BYTES];

namespace {
size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

int scratch_address(void** out, char* err, size_t errn) {
    static std::mutex mu;
    static void* addr[64] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        snprintf(err, errn, "device: %s", cudaGetErrorString(e));
        return AEROS_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_voxel_scratch);
        if (e != cudaSuccess || !p) {
            snprintf(err, errn, "scratch symbol: %s", cudaGetErrorString(e));
            return AEROS_ERR_CUDA;
        }
        addr[dev] = p;
    }
    *out = addr[dev];
    return AEROS_OK;
}
}  // namespace

int voxelize_noalloc_impl(const float* tris, int64_t ntri, const aeros_voxel_grid* g, uint8_t* d_mask, char* err,
                          size_t errn) {
    if ((size_t)ntri * sizeof(float) * 9 > VOXEL_SCRATCH_BYTES) {
        snprintf(err, errn, "%lld triangles exceed the %zu-byte voxelizer scratch", (long long)ntri, VOXEL_SCRATCH_BYTES);
        return AEROS_ERR_INVALID;
    }
    std::vector<HTri> tv;
    tv.reserve((size_t)std::max<int64_t>(ntri, 0));
    for (int64_t i = 0; i < ntri; ++i) {
        HTri t;
        if (make_tri(tris + 9 * i, t)) tv.push_back(t);
    }
    const long long total = (long long)g->nx * g->ny * g->nz;
    const cudaStream_t s = nullptr;
    if (tv.empty()) {
        cudaError_t e = cudaMemsetAsync(d_mask, 0, (size_t)total, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { snprintf(err, errn, "memset: %s", cudaGetErrorString(e)); return AEROS_ERR_CUDA; }
        return AEROS_OK;
    }
    Builder b(tv);
    b.nodes.reserve(tv.size() * 2 / 4 + 2);
    b.build(0, (int)tv.size(), 0);
    std::vector<float> flat(tv.size() * 9);
    for (size_t i = 0; i < tv.size(); ++i) memcpy(&flat[9 * i], tv[i].v, 36);
    // layout: overflow flag | nodes | triangles, each 256-byte aligned
    const size_t off_nodes = 256;
    const size_t off_tris = align256(off_nodes + b.nodes.size() * sizeof(DNode));
    const size_t need = off_tris + flat.size() * sizeof(float);
    if (need > VOXEL_SCRATCH_BYTES) {
        snprintf(err, errn, "mesh needs %zu bytes of the %zu-byte voxelizer scratch", need, VOXEL_SCRATCH_BYTES);
        return AEROS_ERR_INVALID;
    }
    void* base = nullptr;
    if (int rc = scratch_address(&base, err, errn)) return rc;
    unsigned char* sc = static_cast<unsigned char*>(base);
    int* dof = reinterpret_cast<int*>(sc);
    DNode* dn = reinterpret_cast<DNode*>(sc + off_nodes);
    float* dt = reinterpret_cast<float*>(sc + off_tris);
    cudaError_t e = cudaMemsetAsync(dof, 0, sizeof(int), s);   // the flag starts at zero
    if (e == cudaSuccess) e = cudaMemcpyAsync(dn, b.nodes.data(), b.nodes.size() * sizeof(DNode), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, flat.data(), flat.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    int overflow = 0;
    if (e == cudaSuccess) {
        int sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        long long blocks = (total + 127) / 128;
        blocks = std::min<long long>(blocks, (long long)std::max(1, sms) * 16);
        k_voxelize<<<(int)std::max<long long>(1, blocks), 128, 0, s>>>(dn, dt, *g, d_mask, dof);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&overflow, dof, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { snprintf(err, errn, "voxelize: %s", cudaGetErrorString(e)); return AEROS_ERR_CUDA; }
    if (overflow) { snprintf(err, errn, "voxelize: BVH traversal stack overflow"); return AEROS_ERR_UNSUPPORTED; }
    return AEROS_OK;
}

}  // namespace aeros
