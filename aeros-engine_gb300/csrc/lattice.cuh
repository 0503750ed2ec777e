// lattice.cuh — D3Q19 / D3Q7 velocity sets, population storage formats and
// integer helpers shared by every kernel of the solver step.
//
// Directions, weights and opposites are the reference's tables
// (aeros/src/lbm.cpp:92-109, aeros/src/thermal_lbm.cpp:31-40), written as
// constexpr functions so fully unrolled loops fold them into immediates.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace aeros {

constexpr int Q19 = 19;
constexpr int Q7 = 7;

__host__ __device__ __forceinline__ constexpr int cx19(int q) {
    return (q == 1 || q == 7 || q == 9 || q == 11 || q == 13) ? 1
         : (q == 2 || q == 8 || q == 10 || q == 12 || q == 14) ? -1 : 0;
}
__host__ __device__ __forceinline__ constexpr int cy19(int q) {
    return (q == 3 || q == 7 || q == 10 || q == 15 || q == 17) ? 1
         : (q == 4 || q == 8 || q == 9 || q == 16 || q == 18) ? -1 : 0;
}
__host__ __device__ __forceinline__ constexpr int cz19(int q) {
    return (q == 5 || q == 11 || q == 14 || q == 15 || q == 18) ? 1
         : (q == 6 || q == 12 || q == 13 || q == 16 || q == 17) ? -1 : 0;
}
__host__ __device__ __forceinline__ constexpr int ca19(int q, int a) {
    return a == 0 ? cx19(q) : (a == 1 ? cy19(q) : cz19(q));
}
// opposite direction: pairs (1,2), (3,4), ..., (17,18)
__host__ __device__ __forceinline__ constexpr int opp19(int q) {
    return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1);
}
// weights 1/3, 1/18, 1/36 rounded to float exactly as 1.0f/3.0f etc.
__host__ __device__ __forceinline__ constexpr float w19(int q) {
    return q == 0 ? 1.0f / 3.0f : (q <= 6 ? 1.0f / 18.0f : 1.0f / 36.0f);
}
__host__ __device__ __forceinline__ constexpr float w7(int q) { return q == 0 ? 0.25f : 0.125f; }
// direction index of a velocity (cx, cy, cz) in {-1,0,1}^3, -1 when absent
__host__ __device__ __forceinline__ int dir19_of(int cx, int cy, int cz) {
#pragma unroll
    for (int q = 0; q < Q19; ++q)
        if (cx19(q) == cx && cy19(q) == cy && cz19(q) == cz) return q;
    return -1;
}

// ---- per-cell descriptor (uint32), built once on the host -----------------
// bits 0..18 : source x - c_q is not an in-domain fluid cell (solid, ground,
//              or outside the domain before periodic wrapping)
constexpr uint32_t D_WALL = 1u << 19;       // solid or ground cell
constexpr uint32_t D_LES = 1u << 20;        // two-pass |S| applies (lbm.cpp:994-1011)
constexpr int D_WD_SHIFT = 21;              // wall distance clamped to 0..6 (3 bits)
constexpr uint32_t D_INLET = 1u << 24;      // on the inlet plane (geometric)
constexpr uint32_t D_OUTLET = 1u << 25;     // on the outlet plane (geometric)
constexpr int D_OUT_SHIFT = 26;             // 2 bits: outlet side-buffer plane + 1
constexpr uint32_t D_SHELL = 1u << 28;      // any coordinate on the domain boundary
constexpr uint32_t D_GROUND = 1u << 29;     // wall cell that is ground, not body (lbm.cpp:624-643)
constexpr uint32_t D_LINKS = (1u << 19) - 2u;

// ---- population storage ---------------------------------------------------
// FP32 stores f_i. FP16 / BF16 store shifted deviations (f_i - s_i for the
// fluid lattice, g_i - w_i Tc for the thermal one) and compute in FP32.
// FP16 keeps them times 2^10 (STORE_SCALE_F16): with the freestream shift the
// far-field deviations are 1e-7 .. 1e-5, below FP16's normal range (6.1e-5),
// where its spacing is absolute; scaled, they keep 11 significant bits, and
// |f - s| up to 64 stays finite (the guards treat f outside [-1, 10] as bad).
// load / store apply the scale; raw_load / raw_store move the stored bits'
// value and kScale / kInv let a caller fold the scale into its own FMA.
constexpr float STORE_SCALE_F16 = 1024.0f;

struct StoreF32 {
    using T = float;
    static constexpr bool shifted = false;
    static constexpr float kScale = 1.0f, kInv = 1.0f;
    __device__ __forceinline__ static float load(const T* p) { return __ldg(p); }
    __device__ __forceinline__ static float load_rw(const T* p) { return *p; }
    __device__ __forceinline__ static void store(T* p, float v) { *p = v; }
    __device__ __forceinline__ static float raw_load(const T* p) { return *p; }
    __device__ __forceinline__ static void raw_store(T* p, float v) { *p = v; }
};
struct StoreF16 {
    using T = __half;
    static constexpr bool shifted = true;
    static constexpr float kScale = STORE_SCALE_F16, kInv = 1.0f / STORE_SCALE_F16;
    __device__ __forceinline__ static float load(const T* p) { return __half2float(*p) * kInv; }
    __device__ __forceinline__ static float load_rw(const T* p) { return __half2float(*p) * kInv; }
    __device__ __forceinline__ static void store(T* p, float v) { *p = __float2half_rn(v * kScale); }
    __device__ __forceinline__ static float raw_load(const T* p) { return __half2float(*p); }
    __device__ __forceinline__ static void raw_store(T* p, float v) { *p = __float2half_rn(v); }
};
struct StoreBF16 {
    using T = __nv_bfloat16;
    static constexpr bool shifted = true;
    static constexpr float kScale = 1.0f, kInv = 1.0f;
    __device__ __forceinline__ static float load(const T* p) { return __bfloat162float(*p); }
    __device__ __forceinline__ static float load_rw(const T* p) { return __bfloat162float(*p); }
    __device__ __forceinline__ static void store(T* p, float v) { *p = __float2bfloat16_rn(v); }
    __device__ __forceinline__ static float raw_load(const T* p) { return __bfloat162float(*p); }
    __device__ __forceinline__ static void raw_store(T* p, float v) { *p = __float2bfloat16_rn(v); }
};

// ---- exact unsigned division by a run-time constant -------------------------
// Granlund & Montgomery, "Division by invariant integers using
// multiplication" (PLDI 1994), Figure 4.1: exact for every 32-bit numerator.
struct FastDiv {
    uint32_t d, m, s1, s2;
    FastDiv() : d(1), m(0), s1(0), s2(0) {}
    explicit FastDiv(uint32_t div) : d(div) {
        uint32_t l = 0;
        while ((1ull << l) < div) ++l;
        m = (uint32_t)(((1ull << 32) * ((1ull << l) - div)) / div + 1);
        s1 = l > 0 ? 1 : 0;
        s2 = l > 0 ? l - 1 : 0;
    }
    __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
        uint32_t t = __umulhi(m, n);
#else
        uint32_t t = (uint32_t)(((uint64_t)m * n) >> 32);
#endif
        return (t + ((n - t) >> s1)) >> s2;
    }
};

}  // namespace aeros
