// forces.cu — FP64 reductions over FP32 fields. Compiled with --fmad=false:
// the per-cell term p*n + rho*u*(u.n) rounds exactly as the reference's.
#include "forces.cuh"
#include "lattice.cuh"

namespace aeros {

__device__ __forceinline__ void face_cell(const ForceArgs& a, long long i, int& cell, float& nx, float& ny, float& nz) {
    const int x0 = a.box[0], x1 = a.box[1], y0 = a.box[2], y1 = a.box[3], z0 = a.box[4], z1 = a.box[5];
    const long long nyz = (long long)(z1 - z0 + 1) * (y1 - y0 + 1);
    const long long nzx = (long long)(z1 - z0 + 1) * (x1 - x0 + 1);
    const int NX = a.nx, NY = a.ny;
    nx = ny = nz = 0.0f;
    if (i < 2 * nyz) {   // x faces
        const int side = (int)(i & 1);
        const long long k = i >> 1;
        const int y = y0 + (int)(k % (y1 - y0 + 1)), z = z0 + (int)(k / (y1 - y0 + 1));
        cell = (z * NY + y) * NX + (side ? x1 : x0);
        nx = side ? 1.0f : -1.0f;
        return;
    }
    i -= 2 * nyz;
    if (i < 2 * nzx) {   // y faces
        const int side = (int)(i & 1);
        const long long k = i >> 1;
        const int x = x0 + (int)(k % (x1 - x0 + 1)), z = z0 + (int)(k / (x1 - x0 + 1));
        cell = (z * NY + (side ? y1 : y0)) * NX + x;
        ny = side ? 1.0f : -1.0f;
        return;
    }
    i -= 2 * nzx;        // z faces
    const int side = (int)(i & 1);
    const long long k = i >> 1;
    const int x = x0 + (int)(k % (x1 - x0 + 1)), y = y0 + (int)(k / (x1 - x0 + 1));
    cell = ((side ? z1 : z0) * NY + y) * NX + x;
    nz = side ? 1.0f : -1.0f;
}

__device__ __forceinline__ long long face_total(const ForceArgs& a) {
    const long long dx = a.box[1] - a.box[0] + 1, dy = a.box[3] - a.box[2] + 1, dz = a.box[5] - a.box[4] + 1;
    return 2 * (dz * dy + dz * dx + dy * dx);
}

__global__ void __launch_bounds__(FORCE_BLOCK) k_cv_force(const ForceArgs a) {
    double fx = 0.0, fy = 0.0, fz = 0.0;
    const long long total = face_total(a);
    for (long long i = blockIdx.x * (long long)FORCE_BLOCK + threadIdx.x; i < total;
         i += (long long)gridDim.x * FORCE_BLOCK) {
        int c;
        float nx, ny, nz;
        face_cell(a, i, c, nx, ny, nz);
        const uint32_t d = a.desc[c];
        if ((d & D_WALL) && !(d & D_GROUND)) continue;   // body cells are skipped, ground is not
        const float rho = a.rho[c];
        const float4 uv = a.u[c];
        const float ux = uv.x, uy = uv.y, uz = uv.z;
        const float p = (1.0f / 3.0f) * (rho - 1.0f);
        const float un = ux * nx + uy * ny + uz * nz;
        fx += (double)(p * nx + rho * ux * un);
        fy += (double)(p * ny + rho * uy * un);
        fz += (double)(p * nz + rho * uz * un);
    }
    __shared__ double s[3][FORCE_BLOCK / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        fx += __shfl_down_sync(0xffffffffu, fx, o);
        fy += __shfl_down_sync(0xffffffffu, fy, o);
        fz += __shfl_down_sync(0xffffffffu, fz, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { s[0][wid] = fx; s[1][wid] = fy; s[2][wid] = fz; }
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) {
        double t[3] = {0.0, 0.0, 0.0};
        for (int w = 0; w < FORCE_BLOCK / 32; ++w) { t[0] += s[0][w]; t[1] += s[1][w]; t[2] += s[2][w]; }
        for (int k = 0; k < 3; ++k) a.partials[3 * blockIdx.x + k] = t[k];
        __threadfence();
        last = atomicAdd(a.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    // the last block sums the block partials: strided per thread, then the
    // same shuffle and warp order as above (a fixed order: deterministic)
    __threadfence();
    double t[3] = {0.0, 0.0, 0.0};
    const volatile double* pp = a.partials;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += FORCE_BLOCK)
        for (int k = 0; k < 3; ++k) t[k] += pp[3 * b + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 3; ++k) t[k] += __shfl_down_sync(0xffffffffu, t[k], o);
    __syncthreads();   // s[] is reused
    if (lane == 0) { s[0][wid] = t[0]; s[1][wid] = t[1]; s[2][wid] = t[2]; }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double r[3] = {0.0, 0.0, 0.0};
    for (int w = 0; w < FORCE_BLOCK / 32; ++w) { r[0] += s[0][w]; r[1] += s[1][w]; r[2] += s[2][w]; }
    for (int k = 0; k < 3; ++k) a.out[k] = r[k];
    *a.counter = 0;
}

int cv_force_blocks(const int box[6], int max_blocks) {
    const long long dx = box[1] - box[0] + 1, dy = box[3] - box[2] + 1, dz = box[5] - box[4] + 1;
    const long long total = 2 * (dz * dy + dz * dx + dy * dx);
    long long b = (total + FORCE_BLOCK - 1) / FORCE_BLOCK;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (int)b;
}

cudaError_t launch_cv_force(const ForceArgs& a, int blocks, cudaStream_t s) {
    k_cv_force<<<blocks, FORCE_BLOCK, 0, s>>>(a);
    return cudaGetLastError();
}

__global__ void k_projected_area(int nx, int ny, int nz, const uint32_t* desc, int axis, unsigned long long* count) {
    const int amax = axis == 0 ? ny : nx;
    const int bmax = axis == 2 ? ny : nz;
    const int len = axis == 0 ? nx : (axis == 1 ? ny : nz);
    const long long cols = (long long)amax * bmax;
    unsigned long long local = 0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < cols; k += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(k % amax), b = (int)(k / amax);
        bool hit = false;
        for (int t = 0; t < len && !hit; ++t) {
            int x, y, z;
            if (axis == 0) { x = t; y = a; z = b; }
            else if (axis == 1) { x = a; y = t; z = b; }
            else { x = a; y = b; z = t; }
            const uint32_t d = desc[(z * ny + y) * nx + x];
            hit = (d & D_WALL) && !(d & D_GROUND);
        }
        local += hit ? 1 : 0;
    }
    if (local) atomicAdd(count, local);
}

cudaError_t launch_projected_area(int nx, int ny, int nz, const uint32_t* desc, int axis, unsigned long long* count,
                                  cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    k_projected_area<<<256, 256, 0, s>>>(nx, ny, nz, desc, axis, count);
    return cudaGetLastError();
}

}  // namespace aeros
