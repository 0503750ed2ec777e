// samplers.cuh — device samplers shared by the post-processing, distance-field
// and surface-force kernels, each rounding as its reference function (the
// including units compile with --fmad=false):
//   field_trilinear  sampleFieldTrilinear(field, pos, skipSolid = true),
//                    aeros/src/lbm.cpp:1881-1933
//   sdf_sample1      sampleSDFCPU, aeros/src/voxel_grid.cpp:32-81
//   sdf_normal1      sdfNormalCPU, voxel_grid.cpp:83-123
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "lattice.cuh"

namespace aeros {
namespace smp {

// the solver grid in world units and its cell descriptors (D_WALL: solid or ground)
struct FieldView {
    int nx, ny, nz;
    float min[3], cs[3];
    const uint32_t* desc;
};

__device__ __forceinline__ float clamp01f(float t) { return fminf(fmaxf(t, 0.0f), 1.0f); }

// Trilinear over the 8 cells around a world point; solid corners and
// non-finite values are left out and the weights renormalised. false where
// the reference reports no data (outside, too few fluid corners, non-finite).
__device__ inline bool field_trilinear(const FieldView& a, const float* field, float wx, float wy, float wz,
                                       float* out) {
    *out = 0.0f;
    if (!(isfinite(wx) && isfinite(wy) && isfinite(wz))) return false;
    if (a.cs[0] < 1e-9f || a.cs[1] < 1e-9f || a.cs[2] < 1e-9f) return false;
    if (a.nx < 2 || a.ny < 2 || a.nz < 2) return false;
    const float fx = (wx - a.min[0]) / a.cs[0], fy = (wy - a.min[1]) / a.cs[1], fz = (wz - a.min[2]) / a.cs[2];
    const int ix = (int)floorf(fx), iy = (int)floorf(fy), iz = (int)floorf(fz);
    if (ix < 0 || iy < 0 || iz < 0 || ix > a.nx - 2 || iy > a.ny - 2 || iz > a.nz - 2) return false;
    const float tx = clamp01f(fx - (float)ix), ty = clamp01f(fy - (float)iy), tz = clamp01f(fz - (float)iz);
    const float wxs[2] = {1.0f - tx, tx}, wys[2] = {1.0f - ty, ty}, wzs[2] = {1.0f - tz, tz};
    float acc = 0.0f, wsum = 0.0f;
    for (int dz = 0; dz <= 1; ++dz)
        for (int dy = 0; dy <= 1; ++dy)
            for (int dx = 0; dx <= 1; ++dx) {
                const int cell = ((iz + dz) * a.ny + (iy + dy)) * a.nx + (ix + dx);
                if (a.desc[cell] & D_WALL) continue;
                const float v = field[cell];
                if (!isfinite(v)) continue;
                const float w = wxs[dx] * wys[dy] * wzs[dz];
                acc += v * w;
                wsum += w;
            }
    if (wsum < 1e-6f) return false;
    acc /= wsum;
    if (!isfinite(acc)) return false;
    *out = acc;
    return true;
}

struct SdfView {
    const float* d;
    int nx, ny, nz;
    float min[3], cs[3];
};

__device__ __forceinline__ bool valid_f(float v) { return isfinite(v) && fabsf(v) < 1e6f; }

// floorf to int for |v| < 2^30; beyond, +-2^30 (outside every grid)
__device__ __forceinline__ int ifloor(float v) {
    const float f = floorf(v);
    if (!(f > -1073741824.0f)) return -1073741824;
    if (!(f < 1073741824.0f)) return 1073741824;
    return (int)f;
}

__device__ inline float sdf_get(const SdfView& g, int x, int y, int z, float fallback) {
    if (x < 0 || x >= g.nx || y < 0 || y >= g.ny || z < 0 || z >= g.nz) return fallback;
    const float v = g.d[((long long)z * g.ny + y) * g.nx + x];
    return valid_f(v) ? v : fallback;
}

// sampleSDFCPU, voxel_grid.cpp:32-81
__device__ inline float sdf_sample1(const SdfView& g, float px, float py, float pz) {
    if (!valid_f(px) || !valid_f(py) || !valid_f(pz)) return 1000.0f;
    float csx = g.cs[0], csy = g.cs[1], csz = g.cs[2];
    if (!valid_f(csx) || fabsf(csx) < 1e-8f) return 1000.0f;
    if (!valid_f(csy) || fabsf(csy) < 1e-8f) csy = csx;
    if (!valid_f(csz) || fabsf(csz) < 1e-8f) csz = csx;
    const float fx = (px - g.min[0]) / csx - 0.5f;
    const float fy = (py - g.min[1]) / csy - 0.5f;
    const float fz = (pz - g.min[2]) / csz - 0.5f;
    const int ix0 = ifloor(fx), iy0 = ifloor(fy), iz0 = ifloor(fz);
    const int ix1 = ix0 + 1, iy1 = iy0 + 1, iz1 = iz0 + 1;
    float tx = fx - ix0, ty = fy - iy0, tz = fz - iz0;
    tx = fminf(fmaxf(tx, 0.0f), 1.0f);
    ty = fminf(fmaxf(ty, 0.0f), 1.0f);
    tz = fminf(fmaxf(tz, 0.0f), 1.0f);
    if (ix0 < 0 || iy0 < 0 || iz0 < 0 || ix1 >= g.nx || iy1 >= g.ny || iz1 >= g.nz) {
        const int ix = ifloor((px - g.min[0]) / csx);
        const int iy = ifloor((py - g.min[1]) / csy);
        const int iz = ifloor((pz - g.min[2]) / csz);
        if (ix < 0 || ix >= g.nx || iy < 0 || iy >= g.ny || iz < 0 || iz >= g.nz) return 1000.0f;
        return g.d[((long long)iz * g.ny + iy) * g.nx + ix];
    }
    const float c000 = sdf_get(g, ix0, iy0, iz0, 1000.0f), c100 = sdf_get(g, ix1, iy0, iz0, 1000.0f);
    const float c010 = sdf_get(g, ix0, iy1, iz0, 1000.0f), c110 = sdf_get(g, ix1, iy1, iz0, 1000.0f);
    const float c001 = sdf_get(g, ix0, iy0, iz1, 1000.0f), c101 = sdf_get(g, ix1, iy0, iz1, 1000.0f);
    const float c011 = sdf_get(g, ix0, iy1, iz1, 1000.0f), c111 = sdf_get(g, ix1, iy1, iz1, 1000.0f);
    const float c00 = c000 * (1 - tx) + c100 * tx;
    const float c10 = c010 * (1 - tx) + c110 * tx;
    const float c01 = c001 * (1 - tx) + c101 * tx;
    const float c11 = c011 * (1 - tx) + c111 * tx;
    const float c0 = c00 * (1 - ty) + c10 * ty;
    const float c1 = c01 * (1 - ty) + c11 * ty;
    return c0 * (1 - tz) + c1 * tz;
}

// sdfNormalCPU, voxel_grid.cpp:83-123
__device__ inline void sdf_normal1(const SdfView& g, float px, float py, float pz, float* n3) {
    n3[0] = 0.0f; n3[1] = 1.0f; n3[2] = 0.0f;
    if (g.nx <= 1 || g.ny <= 1 || g.nz <= 1) return;
    if (!valid_f(px) || !valid_f(py) || !valid_f(pz)) return;
    float csx = g.cs[0], csy = g.cs[1], csz = g.cs[2];
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
        const int ix = ifloor((px - g.min[0]) / csx);
        const int iy = ifloor((py - g.min[1]) / csy);
        const int iz = ifloor((pz - g.min[2]) / csz);
        if (ix <= 0 || ix >= g.nx - 1 || iy <= 0 || iy >= g.ny - 1 || iz <= 0 || iz >= g.nz - 1) return;
        dx = sdf_get(g, ix + 1, iy, iz, 0.0f) - sdf_get(g, ix - 1, iy, iz, 0.0f);
        dy = sdf_get(g, ix, iy + 1, iz, 0.0f) - sdf_get(g, ix, iy - 1, iz, 0.0f);
        dz = sdf_get(g, ix, iy, iz + 1, 0.0f) - sdf_get(g, ix, iy, iz - 1, 0.0f);
        len = sqrtf(dx * dx + dy * dy + dz * dz);
        if (len < 1e-6f) return;
    }
    n3[0] = dx / len; n3[1] = dy / len; n3[2] = dz / len;
}

}  // namespace smp
}  // namespace aeros
