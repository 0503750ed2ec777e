// setup.cu — per-cell descriptors built on the device at domain creation.
//
// The wall distance only enters the step clamped to 0..6 (Van Driest factor
// for d <= 5, aeros/src/lbm.cpp:1134-1139); six Jacobi sweeps of the
// 6-neighbour min-plus-one relaxation give the exact Manhattan distance up to
// 6, which is what the reference's two-pass chamfer (lbm.cpp:647-675)
// computes there. The full 0..255 field is rebuilt on the host only when a
// caller reads it back.
#include <cuda_runtime.h>

#include "lattice.cuh"
#include "setup.cuh"

namespace aeros {

__global__ void k_wd_init(const uint8_t* mask, uint8_t* wd, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) wd[c] = mask[c] ? 0 : 7;
}

__global__ void k_wd_relax(const uint8_t* in, uint8_t* out, int nx, int ny, int nz) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = nx * ny * nz;
    if (c >= n) return;
    const int x = c % nx, r = c / nx, y = r % ny, z = r / ny;
    int v = in[c];
    if (v) {
        if (x > 0) v = min(v, in[c - 1] + 1);
        if (x < nx - 1) v = min(v, in[c + 1] + 1);
        if (y > 0) v = min(v, in[c - nx] + 1);
        if (y < ny - 1) v = min(v, in[c + nx] + 1);
        if (z > 0) v = min(v, in[c - nx * ny] + 1);
        if (z < nz - 1) v = min(v, in[c + nx * ny] + 1);
    }
    out[c] = (uint8_t)v;
}

__global__ void k_build_desc(const DescArgs a, const uint8_t* mask, const uint8_t* wd, uint32_t* desc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    if (c >= nx * ny * nz) return;
    const int x = c % nx, r = c / nx, y = r % ny, z = r / ny;
    const uint8_t m = mask[c];
    uint32_t d = 0;
    const bool wall = m != 0;
    if (wall) d |= D_WALL;
    if (m == 2) d |= D_GROUND;
    const bool shell = x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 || z == nz - 1;
    if (shell) d |= D_SHELL;
#pragma unroll
    for (int q = 1; q < Q19; ++q) {
        const int sx = x - cx19(q), sy = y - cy19(q), sz = z - cz19(q);
        const bool in = sx >= 0 && sx < nx && sy >= 0 && sy < ny && sz >= 0 && sz < nz;
        if (!in || mask[(sz * ny + sy) * nx + sx] != 0) d |= 1u << q;
    }
    d |= (uint32_t)min((int)wd[c], 6) << D_WD_SHIFT;
    const int pos = a.flow_axis == 0 ? x : (a.flow_axis == 1 ? y : z);
    const bool inl = pos == a.inlet_pos, outl = pos == a.outlet_pos;
    if (inl) d |= D_INLET;
    if (outl) d |= D_OUTLET;
    if (!wall && !inl && !outl && !shell) {
        const int nbs[6] = {c - 1, c + 1, c - nx, c + nx, c - nx * ny, c + nx * ny};
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (mask[nbs[k]] == 1) ok = false;
        if (ok) d |= D_LES;
    }
    if (a.outlet_mode && !wall) {
        uint32_t slot = 0;
        if (pos == a.outlet_pos) slot = 1;
        else if (pos == a.ic) slot = 2;
        else if (pos == a.ic2) slot = 3;
        d |= slot << D_OUT_SHIFT;
    }
    desc[c] = d;
}

cudaError_t build_descriptors(const DescArgs& a, const uint8_t* d_mask, uint8_t* d_tmp0, uint8_t* d_tmp1,
                              uint32_t* d_desc, cudaStream_t s) {
    const int n = a.nx * a.ny * a.nz;
    const int blocks = (n + 255) / 256;
    k_wd_init<<<blocks, 256, 0, s>>>(d_mask, d_tmp0, n);
    uint8_t* in = d_tmp0;
    uint8_t* out = d_tmp1;
    for (int it = 0; it < 6; ++it) {
        k_wd_relax<<<blocks, 256, 0, s>>>(in, out, a.nx, a.ny, a.nz);
        uint8_t* t = in; in = out; out = t;
    }
    k_build_desc<<<blocks, 256, 0, s>>>(a, d_mask, in, d_desc);
    return cudaGetLastError();
}

}  // namespace aeros
