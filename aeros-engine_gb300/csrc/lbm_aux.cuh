// lbm_aux.cuh — initialisation, state I/O and divergence-reset kernels, and
// the per-storage launcher table the C ABI dispatches through.
#pragma once

#include <cuda_runtime.h>

#include "lbm_step.cuh"

namespace aeros {

// computeEquilibriumFast, aeros/src/lbm.cpp:146-184 (same expression trees).
__host__ __device__ __forceinline__ float eq_checked(int q, float rho, float ux, float uy, float uz, float usqr) {
    if (!isfinite(rho)) rho = 1.0f;
    if (usqr > 0.09f) {
        const float scale = sqrtf(0.09f / usqr);
        ux *= scale; uy *= scale; uz *= scale;
        usqr = ux * ux + uy * uy + uz * uz;
    }
    float cu = (float)cx19(q) * ux + (float)cy19(q) * uy + (float)cz19(q) * uz;
    if (!isfinite(cu)) cu = 0.0f;
    float feq = w19(q) * rho * (1.0f + cu * 3.0f + cu * cu * 4.5f - usqr * 1.5f);
    if (!isfinite(feq)) feq = w19(q) * rho;
    return feq;
}

struct FillArgs {
    void* f;
    const uint32_t* desc;
    long long qstride;
    int ncell;
    float fluid[19];   // plain values
    float wall[19];
    float dq[19];      // shifted storage: s_q - w_q (stored value = f - w - dq)
};

struct Shift19 {       // s_q - w_q of the shifted storage (zero for FP32)
    float d[Q19];
};

struct ShiftT {        // shifted D3Q7 storage: Tc(y) = tc0 + tc1 * y, the grid's nx, ny
    float tc0, tc1;
    int nx, ny;
};

// Uniform equilibrium (initLBM, aeros/src/lbm.cpp:686-739) in pre-collision layout.
template <class S>
__global__ void k_fill_uniform(const FillArgs a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncell) return;
    const bool wall = (a.desc[c] & D_WALL) != 0;
    typename S::T* f = reinterpret_cast<typename S::T*>(a.f);
#pragma unroll
    for (int q = 0; q < Q19; ++q) {
        const float v = wall ? a.wall[q] : a.fluid[q];
        S::store(f + (long long)q * a.qstride + c, S::shifted ? (v - w19(q)) - a.dq[q] : v);
    }
}

// Equilibrium from per-cell rho/u with the init limiter (lbm.cpp:720-737).
template <class S>
__global__ void k_set_equilibrium(void* fp, const uint32_t* desc, long long qstride, int ncell, const float* rho,
                                  const float* ux, const float* uy, const float* uz, const Shift19 sh) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell || (desc[c] & D_WALL)) return;
    const float r = rho ? rho[c] : 1.0f;
    float vx = ux[c], vy = uy[c], vz = uz[c];
    float usqr = vx * vx + vy * vy + vz * vz;
    if (usqr > 0.09f) {
        const float scale = sqrtf(0.09f / usqr);
        vx *= scale; vy *= scale; vz *= scale;
        usqr = vx * vx + vy * vy + vz * vz;
    }
    typename S::T* f = reinterpret_cast<typename S::T*>(fp);
#pragma unroll
    for (int q = 0; q < Q19; ++q) {
        const float v = eq_checked(q, r, vx, vy, vz, usqr);
        S::store(f + (long long)q * qstride + c, S::shifted ? (v - w19(q)) - sh.d[q] : v);
    }
}

// Pre-collision populations [19][ncell] (plain values) into the slots the
// next even step gathers from. Wall cells are left untouched.
// D3Q7 (nq = 7): the slot of direction i holds g - w_i Tc(y_w), y_w the row
// of the cell the even step's gather takes it as stored by (y - c_iy on a
// regular link, y otherwise; only i = 3, 4 move along y).
template <class S>
__global__ void k_write_pre(void* fp, const uint32_t* desc, long long qstride, int ncell, const float* src, int nq,
                            const ShiftT ts, const Shift19 sh) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell || (desc[c] & D_WALL)) return;
    typename S::T* f = reinterpret_cast<typename S::T*>(fp);
    const int y = (c / ts.nx) % ts.ny;
    for (int q = 0; q < nq; ++q) {
        const float v = src[(long long)q * ncell + c];
        float st = v;
        if (S::shifted) {
            if (nq == Q19) {
                st = (v - w19(q)) - sh.d[q];
            } else {
                const bool regular = !((desc[c] >> q) & 1u);
                const int yw = regular ? y - cy19(q) : y;
                st = v - w7(q) * fmaf(ts.tc1, (float)yw, ts.tc0);
            }
        }
        S::store(f + (long long)q * qstride + c, st);
    }
}

// Re-equilibration after divergence (aeros/src/lbm.cpp:1583-1600): fluid cells
// get f = feq(1, u_in), rho = 1, u = u_in.
template <class S>
__global__ void k_reset(void* fp, const uint32_t* desc, long long qstride, int ncell, FillArgs fa, float* rho, float4* u,
                        float uin0, float uin1, float uin2) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell || (desc[c] & D_WALL)) return;
    typename S::T* f = reinterpret_cast<typename S::T*>(fp);
#pragma unroll
    for (int q = 0; q < Q19; ++q)
        S::store(f + (long long)q * qstride + c, S::shifted ? (fa.fluid[q] - w19(q)) - fa.dq[q] : fa.fluid[q]);
    rho[c] = 1.0f;
    u[c] = make_float4(uin0, uin1, uin2, 0.0f);
}

// D3Q7 populations from a temperature field. The reference's thermal step
// streams before it collides (thermal_lbm.cpp:199-336), so its freshly set
// populations g = geq(T, u = 0) (thermal_lbm.cpp:179-183, 191-194) are a
// post-collision state: they are streamed here once, with the step's own
// boundary rules, into the slots the next (even) step gathers from.
template <class S>
__global__ void k_thermal_prestream(const StepArgs A) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.ncell) return;
    const uint32_t d = A.desc[c];
    if (d & D_WALL) return;
    const int x = c % A.nx, r = c / A.nx, y = r % A.ny, z = r / A.ny;
    typename S::T* g = reinterpret_cast<typename S::T*>(A.g);
#pragma unroll
    for (int i = 0; i < Q7; ++i) {
        const TLink L = th_resolve(A, x, y, z, c, i, false, d);
        float v;
        if (L.bounce == 0) {
            v = w7(i) * A.T[L.idx] * (1.0f + 4.0f * 0.0f);
        } else {
            const float go = w7(opp19(i)) * A.T[c] * (1.0f + 4.0f * 0.0f);
            v = L.bounce == 2 ? (-go + 2.0f * w7(i) * L.Tw) : go;
        }
        S::store(g + (long long)i * A.qstride + c, S::shifted ? v - w7(i) * th_tc(A, L.bounce == 0 ? y - cy19(i) : y) : v);
    }
}

// Launcher table, one instance per storage format (the translation unit of
// each format is compiled with its own floating-point contraction setting).
struct Launchers {
    cudaError_t (*step)(const StepArgs& A, const StepVar& V, const StepOffsets& O, bool odd, bool thermal, bool mat,
                        int grid, cudaStream_t s);
    int (*occupancy)(bool odd, bool thermal);
    cudaError_t (*fill_uniform)(const FillArgs& a, cudaStream_t s);
    cudaError_t (*set_equilibrium)(void* f, const uint32_t* desc, long long qstride, int ncell, const float* rho,
                                   const float* ux, const float* uy, const float* uz, const Shift19& sh,
                                   cudaStream_t s);
    cudaError_t (*write_pre)(void* f, const uint32_t* desc, long long qstride, int ncell, const float* src, int nq,
                             const ShiftT& ts, const Shift19& sh, cudaStream_t s);
    cudaError_t (*reset)(void* f, const uint32_t* desc, long long qstride, int ncell, const FillArgs& fa, float* rho,
                         float4* u, const float* uin, cudaStream_t s);
    cudaError_t (*thermal_fill)(const StepArgs& A, cudaStream_t s);
    cudaError_t (*batch_step)(const BatchArgs& B, bool odd, int kind, int grid, cudaStream_t s);
    int (*batch_occupancy)();
    int (*fused_occupancy)(bool odd, bool thermal);
    int (*warp_occupancy)(bool odd);
    int warp_pad;               // nx must be a multiple of this for warp tiles (16 bytes of storage)
    int warp_tile;              // cells per warp tile
};

const Launchers& launchers_fp32();
const Launchers& launchers_fp16();
const Launchers& launchers_bf16();

#define AEROS_DEFINE_LAUNCHERS(NAME, STORE)                                                                           \
    namespace NAME##_detail {                                                                                         \
    template <bool O, bool T, bool M>                                                                                 \
    cudaError_t launch_one(const StepArgs& A, const StepVar& V, const StepOffsets& OF, int grid, cudaStream_t s) {   \
        if (!M && !T && A.warp) {                                                                                     \
            const int g = (O ? A.warp_grid_odd : A.warp_grid) + A.shell_blocks;                                       \
            if (A.Fx != 0.0f || A.Fy != 0.0f || A.Fz != 0.0f)                                                         \
                k_lbm_warp<STORE, O, true><<<g, STEP_BLOCK, WarpLayout<STORE>::BYTES, s>>>(A, V, OF);                     \
            else                                                                                                      \
                k_lbm_warp<STORE, O, false><<<g, STEP_BLOCK, WarpLayout<STORE>::BYTES, s>>>(A, V, OF);                    \
        } else if (!M && A.fused) {                                                                                   \
            const int g = (O ? A.fused_grid_odd : A.fused_grid) + A.shell_blocks;                                      \
            if (A.shell_blocks > 0) k_lbm_fused<STORE, O, T, false><<<g, STEP_BLOCK, 0, s>>>(A, V, OF);                    \
            else k_lbm_fused<STORE, O, T, true><<<g, STEP_BLOCK, 0, s>>>(A, V, OF);                                        \
        } else if (!M && A.split) {                                                                                   \
            StepArgs B = A;                                                                                           \
            B.shell_part_base = grid;                                                                                 \
            if (B.shell_grid > 0) k_lbm_shell<STORE, O, T><<<B.shell_grid, STEP_BLOCK, 0, s>>>(B, V);                 \
            k_lbm_interior<STORE, O, T><<<grid, STEP_BLOCK, 0, s>>>(B, V);                                            \
        } else {                                                                                                      \
            k_lbm_step<STORE, O, T, M><<<grid, STEP_BLOCK, 0, s>>>(A, V);                                             \
        }                                                                                                             \
        return cudaGetLastError();                                                                                    \
    }                                                                                                                 \
    cudaError_t step_(const StepArgs& A, const StepVar& V, const StepOffsets& OF, bool odd, bool thermal, bool mat,  \
                      int grid, cudaStream_t s) {                                                                     \
        if (mat) {                                                                                                    \
            if (odd) return thermal ? launch_one<true, true, true>(A, V, OF, grid, s) : launch_one<true, false, true>(A, V, OF, grid, s); \
            return thermal ? launch_one<false, true, true>(A, V, OF, grid, s) : launch_one<false, false, true>(A, V, OF, grid, s);  \
        }                                                                                                             \
        if (odd) return thermal ? launch_one<true, true, false>(A, V, OF, grid, s) : launch_one<true, false, false>(A, V, OF, grid, s); \
        return thermal ? launch_one<false, true, false>(A, V, OF, grid, s) : launch_one<false, false, false>(A, V, OF, grid, s);    \
    }                                                                                                                 \
    template <bool O, bool T>                                                                                         \
    int occ_one() {                                                                                                   \
        int n = 0;                                                                                                    \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_lbm_step<STORE, O, T, false>, STEP_BLOCK, 0);             \
        return n > 0 ? n : 1;                                                                                         \
    }                                                                                                                 \
    int occupancy_(bool odd, bool thermal) {                                                                          \
        return odd ? (thermal ? occ_one<true, true>() : occ_one<true, false>())                                       \
                   : (thermal ? occ_one<false, true>() : occ_one<false, false>());                                    \
    }                                                                                                                 \
    cudaError_t fill_(const FillArgs& a, cudaStream_t s) {                                                            \
        k_fill_uniform<STORE><<<(a.ncell + 255) / 256, 256, 0, s>>>(a);                                               \
        return cudaGetLastError();                                                                                    \
    }                                                                                                                 \
    cudaError_t seteq_(void* f, const uint32_t* desc, long long qs, int n, const float* rho, const float* ux,        \
                       const float* uy, const float* uz, const Shift19& sh, cudaStream_t s) {                         \
        k_set_equilibrium<STORE><<<(n + 255) / 256, 256, 0, s>>>(f, desc, qs, n, rho, ux, uy, uz, sh);                \
        return cudaGetLastError();                                                                                    \
    }                                                                                                                 \
    cudaError_t writepre_(void* f, const uint32_t* desc, long long qs, int n, const float* src, int nq,              \
                          const ShiftT& ts, const Shift19& sh, cudaStream_t s) {                                      \
        k_write_pre<STORE><<<(n + 255) / 256, 256, 0, s>>>(f, desc, qs, n, src, nq, ts, sh);                          \
        return cudaGetLastError();                                                                                    \
    }                                                                                                                 \
    cudaError_t reset_(void* f, const uint32_t* desc, long long qs, int n, const FillArgs& fa, float* rho, float4* u,  \
                       const float* uin, cudaStream_t s) {                                                            \
        k_reset<STORE><<<(n + 255) / 256, 256, 0, s>>>(f, desc, qs, n, fa, rho, u, uin[0], uin[1], uin[2]);           \
        return cudaGetLastError();                                                                                    \
    }                                                                                                                 \
    cudaError_t thfill_(const StepArgs& A, cudaStream_t s) {                                                          \
        k_thermal_prestream<STORE><<<(A.ncell + 255) / 256, 256, 0, s>>>(A);                                          \
        return cudaGetLastError();                                                                                    \
    }                                                                                                                 \
    cudaError_t batch_(const BatchArgs& B, bool odd, int kind, int grid, cudaStream_t s) {                          \
        if (kind == 0) {                                                                                              \
            if (odd) k_batch_step<STORE, true, 0><<<grid, BATCH_BLOCK, 0, s>>>(B);                                     \
            else k_batch_step<STORE, false, 0><<<grid, BATCH_BLOCK, 0, s>>>(B);                                        \
        } else {                                                                                                      \
            if (odd) k_batch_step<STORE, true, 1><<<grid, BATCH_BLOCK, 0, s>>>(B);                                     \
            else k_batch_step<STORE, false, 1><<<grid, BATCH_BLOCK, 0, s>>>(B);                                        \
        }                                                                                                             \
        return cudaGetLastError();                                                                                    \
    }                                                                                                                 \
    int fused_occ_(bool odd, bool thermal) {                                                                          \
        int n = 0;                                                                                                    \
        if (thermal) {                                                                                                \
            if (odd) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_lbm_fused<STORE, true, true, false>, STEP_BLOCK, 0); \
            else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_lbm_fused<STORE, false, true, false>, STEP_BLOCK, 0);   \
        } else {                                                                                                      \
            if (odd) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_lbm_fused<STORE, true, false, false>, STEP_BLOCK, 0); \
            else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_lbm_fused<STORE, false, false, false>, STEP_BLOCK, 0);  \
        }                                                                                                             \
        return n > 0 ? n : 1;                                                                                         \
    }                                                                                                                 \
    template <bool O, bool F>                                                                                         \
    int warp_occ_one() {                                                                                              \
        int n = 0;                                                                                                    \
        cudaFuncSetAttribute(k_lbm_warp<STORE, O, F>, cudaFuncAttributeMaxDynamicSharedMemorySize,                    \
                             WarpLayout<STORE>::BYTES);                                                               \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_lbm_warp<STORE, O, F>, STEP_BLOCK,                        \
                                                      WarpLayout<STORE>::BYTES);                                      \
        return n > 0 ? n : 1;                                                                                         \
    }                                                                                                                 \
    int warp_occ_(bool odd) {                                                                                         \
        const int a = odd ? warp_occ_one<true, false>() : warp_occ_one<false, false>();                               \
        const int b = odd ? warp_occ_one<true, true>() : warp_occ_one<false, true>();                                 \
        return a < b ? a : b;                                                                                         \
    }                                                                                                                 \
    int batch_occ_() {                                                                                                \
        int n = 0, m = 0;                                                                                             \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_step<STORE, false, 1>, BATCH_BLOCK, 0);              \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, k_batch_step<STORE, true, 1>, BATCH_BLOCK, 0);               \
        n = n < m ? n : m;                                                                                            \
        return n > 0 ? n : 1;                                                                                         \
    }                                                                                                                 \
    }                                                                                                                 \
    const Launchers& NAME() {                                                                                         \
        using namespace NAME##_detail;                                                                                \
        static const Launchers L = {step_,      occupancy_, fill_,      seteq_,      writepre_,                     \
                                    reset_,     thfill_,    batch_,     batch_occ_,  fused_occ_,                    \
                                    warp_occ_,  WarpLayout<STORE>::PAD, WarpLayout<STORE>::WT};                       \
        return L;                                                                                                     \
    }

}  // namespace aeros
