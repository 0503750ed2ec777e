// lbm_step.cuh — the fused D3Q19 (+D3Q7) solver step on GB300.
//
// One launch = one lattice step (aeros/src/lbm.cpp:957-1580): previous-step
// |S| (LES), collision, stream with the reference's boundary rules, thermal
// step (aeros/src/thermal_lbm.cpp:199-355), per-step statistics.
//
// Layout: structure of arrays, population q of cell c at f[q*qstride + c].
// Streaming is the in-place AA pattern (one population array):
//   even step: gather f_q from slot (c, q); scatter post_q to slot (c, opp q)
//   odd step : gather f_q from slot (c - c_q, opp q); scatter post_q to
//              slot (c + c_q, q)
// so every slot is read and written by exactly one thread per step. Boundary
// links are redirected to slots nobody else owns (bounce-back, copy-own,
// free-slip); rules that read other cells' post-collision values of the same
// step (convective / zero-gradient outlet) go through a parity-double-buffered
// side buffer of the three outlet planes.
//
// Threads: one cell each, over a tile list (interior tiles first, then the
// boundary shell from an explicit cell list); the grid is persistent (SMs x
// resident blocks) and strides over tiles. Per-block partial sums land in
// `partials`; the last block to finish reduces them in a fixed order
// (deterministic) and applies the divergence guard.
#pragma once

#include "lattice.cuh"

namespace aeros {

#ifndef AEROS_STEP_BLOCK
#define AEROS_STEP_BLOCK 128
#endif
constexpr int STEP_BLOCK = AEROS_STEP_BLOCK;   // threads per block = cells per tile (a multiple of 32)
constexpr int BATCH_BLOCK = 256;               // threads per block of the many-domain kernel
#ifndef AEROS_STEP_MIN_BLOCKS
#define AEROS_STEP_MIN_BLOCKS 6
#endif
constexpr int STEP_MIN_BLOCKS = AEROS_STEP_MIN_BLOCKS;   // resident blocks per SM the register budget targets

struct Partial {            // 80 bytes, one per block
    double rho, ke, tke, nu, tsum;
    float maxu;
    int nan, neg, bad, rout, rnf, ulim, nun;
    int pad[2];
};

struct Control {
    unsigned int blocks_done;
    unsigned int tile_next;     // dynamic tile scheduler, reset by the finisher
    int halt;               // divergence guard tripped: later steps return at once
    int halt_kind;          // 1: NaN count before streaming, 2: mean density
    int th_valid;           // Nusselt updated at least once
    int pad0;
    long long steps;        // counted steps (lbmCurrentStep)
    long long kexec;        // step bodies executed
    float prev_kinetic;
    int converged;
    double sum_rho, sum_ke, sum_tke;
    float avg_rho, avg_ke, avg_tke, max_u, convergence;
    float nusselt, mean_t;
    int pad;
    long long nan, neg, bad, rout, rnf, ulim;
    // fused launch (dynamic warp work items): exact fixed-point sums of the
    // step, zeroed by the finisher
    unsigned int shell_next, warps_done;
    unsigned long long fx_drho, fx_ke, fx_tke;
    unsigned long long fx_cnt[7];   // NaN, negative, bad, rho range, rho finite, u limited, cells
    unsigned long long fx_nu, fx_tsum, fx_nun;   // thermal: Nusselt row sum, sum of T, Nusselt row cells
    unsigned int fx_maxu2, pad2;
};

struct StepArgs {
    int nx, ny, nz, nxny, ncell;
    long long qstride;
    int n_interior, ntiles_interior, n_shell, ntiles;
    int shell_stride;           // tile sequence position stride of shell tiles
    FastDiv div_ix, div_iy;     // interior decode: (nx-2), (ny-2)
    FastDiv div_x, div_y;       // shell decode: nx, ny
    void* f;
    void* fq[Q19];              // start of population plane q (f + q * qstride)
    int nbq[Q19];               // linear offset of c_q: cx + cy * nx + cz * nx * ny
    const uint32_t* desc;
    const int* shell;
    const uint32_t* shell_gth;  // odd steps: element offset (plane * qstride + cell) of the source of
                                // population q of shell cell si, at [q * n_shell + si]; NULL: resolve
    const uint32_t* shell_sct;  // odd steps: element offset that post-collision population j goes to
    const unsigned long long* shell_kind;   // 2 bits per D3Q19 direction (LinkKind),
                                            // 2 bits per D3Q7 direction from bit 40
    float *rho, *strain, *tke;
    int out_plane;
    void* g;
    float* T;
    Partial* partials;
    Control* ctl;
    float* mat_f;
    float* mat_g;
    float tau0, Cs, velScale2;
    float Fx, Fy, Fz;
    float uin[3];
    float feq_in[19];           // inlet equilibrium in register form (h = f - w when shifted)
    float dq[19];               // shifted storage: s_q - w_q, s = f_eq(1, u_shift) (stored value = f - s_r)
    float dqs[19];              // dq times the storage scale (2^10 for FP16, 1 for BF16)
    float conv;
    int flow_axis, flow_sign;
    int periodic_x, periodic_z;
    int use_trt, use_les;
    int freeslip, outlet_mode;  // outlet_mode: 0 none, 1 convective, 2 zero-gradient
    int fast_ok;                // forces bounded: clean states need no non-finite checks
    int shifted_fast;           // shifted storage, no body force, no thermal: collide19_shifted_fast
    int split;                  // shell and interior as two launches
    int fused;                  // one launch: shell blocks beside dynamic interior blocks (non-thermal)
    int shell_blocks;           // fused: blocks given to the boundary shell
    int fused_grid;             // fused even steps: interior blocks (resident blocks per SM x SMs)
    int fused_grid_odd;         // fused odd steps (own register budget, own occupancy)
    int warp;                   // interior through warp tiles (k_lbm_warp)
    int wt_first, wt_last;      // warp tiles: first and last linear tile (WarpLayout::WT cells) holding interior cells
    int warp_grid, warp_grid_odd;   // warp tiles: interior blocks of even / odd steps (resident blocks per SM x SMs)
    int inlet_pos;              // inlet plane coordinate along the flow axis
    const int* zg_src;          // zero-gradient outlet: plane index each unknown q of outlet-plane
                                // cell pi reads, at [q * out_plane + pi] (NULL: computed)
    int shell_part_base, shell_grid;   // split: first partial slot and grid of the shell launch
    int total_div10, fluid_cells;
    float conv_threshold;
    int th_on, th_fixed, th_ylo;
    float th_invtau, th_hot, th_cold, th_tref, th_glb, th_H;
    float th_tc0, th_tc1;       // shifted D3Q7 storage: Tc(y) = th_tc0 + th_tc1 * y (conduction profile or Tref)
    int th_buoy_mode;           // 0: from the previous step's T, 1: zero (fresh
                                // field, thermal_lbm.cpp:132), 2: from T_buoy
    const float* T_buoy;
    double th_rows_n;           // Nx*Nz*(yhi-ylo+1), thermal_lbm.cpp:76
};

// The many-domain kernel copies a member's StepArgs into shared memory, one
// 32-bit word per thread. Three configurations in which that copy took a
// second pass (StepArgs of 1080 or 1232 bytes with blocks of 256 threads,
// 928 bytes with blocks of 128) read a mix of two members' arguments: a hang,
// and illegal addresses on the 16- and 64-domain sweeps. Every configuration
// with a single pass (928 bytes, 256 threads) runs clean. The cause was not
// found: keep StepArgs at its size and the copy in one pass, pass additions
// as kernel parameters of their own (StepOffsets), and run any change to
// either on the full sweep.
static_assert(sizeof(StepArgs) <= 928, "StepArgs is copied by the many-domain kernel: see above");
static_assert(sizeof(StepArgs) / 4 <= BATCH_BLOCK, "the many-domain kernel copies StepArgs in one pass: see above");

// What changes from one step to the next (AA parity of the double-buffered
// velocity and outlet side buffers, first-step and last-step flags).
struct StepVar {
    const float4* up;           // previous-step velocity (ux, uy, uz, 0) per cell
    float4* uc;                 // this step's velocity
    float* out_w;               // outlet side buffer written this step
    const float* out_r;         // ... and the one the previous step wrote
    int apply_overrides;        // inlet / outlet overrides (off right after (re)initialisation)
    int write_obs;              // write rho, strain, TKE (last step of a call)
    int write_u;                // write the velocity (every step with LES, else the last)
};

// Van Driest factor table, aeros/src/lbm.cpp:112-120
__device__ __forceinline__ float van_driest(int d) {
    return d == 1 ? 0.3934693403f : d == 2 ? 0.6321205588f : d == 3 ? 0.7768698399f
         : d == 4 ? 0.8646647168f : d == 5 ? 0.9179150014f : 0.0f;
}

// Per-thread accumulators. A thread sums its own cells (a fixed set: tiles
// are assigned statically) in FP32 — the density as the deviation rho - 1 —
// and the block and global sums are FP64 in a fixed order, so the statistics
// are deterministic.
struct Acc {
    float drho, ke, tke, tsum;
    double nu;     // Nusselt row sum (few cells per thread), FP64 as the reference
    float maxu2;   // max |u|^2; the reference's max |u| is its square root
    int nan, neg, bad, rout, rnf, ulim, nun, cells;
    __device__ void zero() {
        drho = ke = tke = tsum = 0.0f;
        nu = 0.0;
        maxu2 = 0.0f;
        nan = neg = bad = rout = rnf = ulim = nun = cells = 0;
    }
};

template <class S>
__device__ __forceinline__ typename S::T* fplane(const StepArgs& A, int q) {
    return reinterpret_cast<typename S::T*>(A.fq[q]);
}
template <class S>
__device__ __forceinline__ typename S::T* gplane(const StepArgs& A, int q) {
    return reinterpret_cast<typename S::T*>(A.g) + (long long)q * A.qstride;
}

__device__ __forceinline__ int nb19(const StepArgs& A, int q) { return A.nbq[q]; }

// ---- shifted storage ---------------------------------------------------------
// FP16 / BF16 slots hold f - s_r, s = f_eq(rho = 1, u_shift) (the freestream
// equilibrium; s = w when u_shift = 0), for the direction r that the next
// gather reads the value as. Registers hold h = f - w. A load of direction q
// adds dq[q] = s_q - w_q; a store subtracts dq of its reader's direction, which
// differs from the value's own direction on links that turn a population
// (bounce-back, copy-own, free slip): s is not symmetric under c -> -c.
// One FMA each way (an add of the parameter constant and a separate
// power-of-two scale gives the same bits but measured 20 % slower on even
// steps).
template <class S>
__device__ __forceinline__ float ld_shift(const StepArgs& A, int q, float raw) {
    return fmaf(raw, S::kInv, A.dq[q]);
}
template <class S>
__device__ __forceinline__ float st_shift(const StepArgs& A, int r, float v) {
    return fmaf(v, S::kScale, -A.dqs[r]);
}
template <class S>
__device__ __forceinline__ float ldp(const StepArgs& A, int q, const typename S::T* p) {
    if constexpr (S::shifted) return ld_shift<S>(A, q, S::raw_load(p));
    else return S::load_rw(p);
}
template <class S>
__device__ __forceinline__ void stp(const StepArgs& A, int r, typename S::T* p, float v) {
    if constexpr (S::shifted) S::raw_store(p, st_shift<S>(A, r, v));
    else S::store(p, v);
}

__device__ __forceinline__ bool is_wall(const StepArgs& A, int c) { return (A.desc[c] & D_WALL) != 0; }

// ---- boundary-shell link resolution (reference rules, lbm.cpp:1376-1406) ----
enum LinkKind { L_REGULAR = 0, L_BOUNCE = 1, L_COPYOWN = 2, L_FREESLIP = 3 };
struct Link {
    int idx, slot, kind;
};

// Where pre-collision population q of cell (x,y,z) comes from.
__device__ __forceinline__ Link resolve_src(const StepArgs& A, int x, int y, int z, int cell, int q) {
    int s0 = x - cx19(q), s1 = y - cy19(q), s2 = z - cz19(q);
    if (A.periodic_x) { s0 = s0 < 0 ? s0 + A.nx : (s0 >= A.nx ? s0 - A.nx : s0); }
    if (A.periodic_z) { s2 = s2 < 0 ? s2 + A.nz : (s2 >= A.nz ? s2 - A.nz : s2); }
    const int o0 = (s0 < 0 || s0 >= A.nx), o1 = (s1 < 0 || s1 >= A.ny), o2 = (s2 < 0 || s2 >= A.nz);
    const int outm = o0 | (o1 << 1) | (o2 << 2);
    if (!outm) {
        const int sc = (s2 * A.ny + s1) * A.nx + s0;
        if (is_wall(A, sc)) return {cell, q, L_BOUNCE};
        return {sc, opp19(q), L_REGULAR};
    }
    if (A.freeslip && !((outm >> A.flow_axis) & 1)) {
        const int r0 = o0 ? x : s0, r1 = o1 ? y : s1, r2 = o2 ? z : s2;
        const int rq = dir19_of(o0 ? -cx19(q) : cx19(q), o1 ? -cy19(q) : cy19(q), o2 ? -cz19(q) : cz19(q));
        const int rc = (r2 * A.ny + r1) * A.nx + r0;
        if (is_wall(A, rc)) return {cell, q, L_BOUNCE};
        return {rc, opp19(rq), L_FREESLIP};
    }
    return {cell, q, L_COPYOWN};
}

// Same resolution with the link kind precomputed on the host: only index
// arithmetic on the device (no loads of neighbour descriptors).
__device__ __forceinline__ Link resolve_kind(const StepArgs& A, int x, int y, int z, int cell, int q, int kind) {
    if (kind == L_BOUNCE || kind == L_COPYOWN) return {cell, q, kind};
    int s0 = x - cx19(q), s1 = y - cy19(q), s2 = z - cz19(q);
    if (A.periodic_x) { s0 = s0 < 0 ? s0 + A.nx : (s0 >= A.nx ? s0 - A.nx : s0); }
    if (A.periodic_z) { s2 = s2 < 0 ? s2 + A.nz : (s2 >= A.nz ? s2 - A.nz : s2); }
    if (kind == L_REGULAR) return {(s2 * A.ny + s1) * A.nx + s0, opp19(q), L_REGULAR};
    const bool o0 = (s0 < 0 || s0 >= A.nx), o1 = (s1 < 0 || s1 >= A.ny), o2 = (s2 < 0 || s2 >= A.nz);
    const int r0 = o0 ? x : s0, r1 = o1 ? y : s1, r2 = o2 ? z : s2;
    const int rq = dir19_of(o0 ? -cx19(q) : cx19(q), o1 ? -cy19(q) : cy19(q), o2 ? -cz19(q) : cz19(q));
    return {(r2 * A.ny + r1) * A.nx + r0, opp19(rq), L_FREESLIP};
}

// Direction the next gather reads post-collision population j of cell
// (x,y,z) as, given the kind of the cell's link of direction opp(j): j on a
// regular link, opp(j) when it comes back to the cell (bounce-back, copy-own
// of population opp(j)), c_j reflected on the axes where x + c_j leaves the
// domain on a free-slip link.
__device__ __forceinline__ int reader_of(const StepArgs& A, int kind, int x, int y, int z, int j) {
    if (kind == L_REGULAR) return j;
    if (kind != L_FREESLIP) return opp19(j);
    int s0 = x + cx19(j), s1 = y + cy19(j), s2 = z + cz19(j);
    if (A.periodic_x) { s0 = s0 < 0 ? s0 + A.nx : (s0 >= A.nx ? s0 - A.nx : s0); }
    if (A.periodic_z) { s2 = s2 < 0 ? s2 + A.nz : (s2 >= A.nz ? s2 - A.nz : s2); }
    const bool o0 = (s0 < 0 || s0 >= A.nx), o1 = (s1 < 0 || s1 >= A.ny), o2 = (s2 < 0 || s2 >= A.nz);
    return dir19_of(o0 ? -cx19(j) : cx19(j), o1 ? -cy19(j) : cy19(j), o2 ? -cz19(j) : cz19(j));
}

// ---- collision of one fluid cell, plain form ---------------------------------
// Same expression trees as aeros/src/lbm.cpp:1061-1299 (compiled without
// contraction, this is bitwise the reference's float arithmetic).
struct CellResult {
    float rho, ux, uy, uz, usqr, strain, tke;
};

__device__ __forceinline__ float eq19(int q, float rho, float cu, float usqr) {
    return w19(q) * rho * (1.0f + cu * 3.0f + cu * cu * 4.5f - usqr * 1.5f);
}
__device__ __forceinline__ float cu19(int q, float ux, float uy, float uz) {
    // (cx*ux + cy*uy) + cz*uz with the zero terms dropped (exact)
    float a = 0.0f;
    bool first = true;
    if (cx19(q) != 0) { a = cx19(q) > 0 ? ux : -ux; first = false; }
    if (cy19(q) != 0) { a = first ? (cy19(q) > 0 ? uy : -uy) : (cy19(q) > 0 ? a + uy : a - uy); first = false; }
    if (cz19(q) != 0) { a = first ? (cz19(q) > 0 ? uz : -uz) : (cz19(q) > 0 ? a + uz : a - uz); }
    return a;
}
__device__ __forceinline__ float src19(int q, float ueX, float ueY, float ueZ, float Fx, float Fy, float Fz) {
    const float cx = (float)cx19(q), cy = (float)cy19(q), cz = (float)cz19(q);
    const float cu = cu19(q, ueX, ueY, ueZ);
    return 3.0f * w19(q) * ((cx - ueX + 3.0f * cu * cx) * Fx + (cy - ueY + 3.0f * cu * cy) * Fy + (cz - ueZ + 3.0f * cu * cz) * Fz);
}

// BGK / TRT relaxation with the Guo source (aeros/src/lbm.cpp:1204-1264).
// CHECKS: the reference's non-finite replacements; without them the code is
// the same arithmetic for states where they cannot trigger (finite, in-range
// populations and bounded forces: every intermediate is finite). FORCE: with
// the source terms; without a force they add exact zeros and are dropped.
template <bool SHIFTED, bool CHECKS, bool FORCE>
__device__ __forceinline__ void relax19(float f[Q19], float rho, float drho, float ueX, float ueY, float ueZ,
                                        float ueSqr, float invTau, float sMinus, float Fx, float Fy, float Fz) {
    const float kP = 1.0f - 0.5f * invTau;
    const float kM = 1.0f - 0.5f * sMinus;
    {
        const float feq = SHIFTED ? w19(0) * drho + w19(0) * rho * (0.0f - ueSqr * 1.5f) : eq19(0, rho, 0.0f, ueSqr);
        float fi = f[0];
        if (CHECKS && !isfinite(fi)) fi = feq;
        float fNew = fi - (fi - feq) * invTau;
        if (FORCE) fNew = fNew + kP * src19(0, ueX, ueY, ueZ, Fx, Fy, Fz);
        if (CHECKS && !isfinite(fNew)) fNew = feq;
        f[0] = fNew;
    }
#pragma unroll
    for (int qi = 1; qi < Q19; qi += 2) {
        const int qo = qi + 1;
        const float cu = cu19(qi, ueX, ueY, ueZ);
        float feq, feqO;
        if (SHIFTED) {
            const float wr = w19(qi) * rho;
            feq = w19(qi) * drho + wr * (cu * 3.0f + cu * cu * 4.5f - ueSqr * 1.5f);
            feqO = w19(qo) * drho + wr * (-cu * 3.0f + cu * cu * 4.5f - ueSqr * 1.5f);
        } else {
            feq = eq19(qi, rho, cu, ueSqr);
            feqO = eq19(qo, rho, -cu, ueSqr);
        }
        float fi = f[qi];
        float fo = f[qo];
        if (CHECKS) {
            if (!isfinite(fi)) fi = feq;
            if (!isfinite(fo)) fo = feqO;
        }
        const float fp = 0.5f * (fi + fo), fm = 0.5f * (fi - fo);
        const float ep = 0.5f * (feq + feqO), em = 0.5f * (feq - feqO);
        const float fpN = fp - invTau * (fp - ep);
        const float fmN = fm - sMinus * (fm - em);
        float newI, newO;
        if (FORCE) {
            const float srcI = src19(qi, ueX, ueY, ueZ, Fx, Fy, Fz);
            const float srcO = src19(qo, ueX, ueY, ueZ, Fx, Fy, Fz);
            const float srcP = 0.5f * (srcI + srcO);
            const float srcM = 0.5f * (srcI - srcO);
            newI = fpN + fmN + kP * srcP + kM * srcM;
            newO = fpN - fmN + kP * srcP - kM * srcM;
        } else {
            newI = fpN + fmN;
            newO = fpN - fmN;
        }
        if (CHECKS) {
            if (!isfinite(newI)) newI = feq;
            if (!isfinite(newO)) newO = feqO;
        }
        f[qi] = newI;
        f[qo] = newO;
    }
}

// Shifted-storage relaxation without a body force: the same TRT update as
// relax19, arranged around the symmetric and antisymmetric equilibrium parts
//   e+ = w (drho + 4.5 rho cu^2 - 1.5 rho u^2),  e- = 3 w rho cu
// with per-cell coefficients folded in (the FP16/BF16 form is measured against
// the FP64 run, not bit-matched, so contraction and reassociation are free).
__device__ __forceinline__ void relax19_shifted_fast(float f[Q19], float rho, float drho, float ueX, float ueY,
                                                     float ueZ, float ueSqr, float invTau, float sMinus) {
    const float P = drho - 1.5f * rho * ueSqr;
    const float R45 = 4.5f * rho;
    const float A1 = 0.5f * (1.0f - invTau), A2 = 0.5f * (1.0f - sMinus);
    f[0] = f[0] - invTau * (f[0] - w19(0) * P);
    const float W1 = invTau * w19(1), W2 = invTau * w19(7);
    const float M1 = 3.0f * rho * sMinus * w19(1), M2 = 3.0f * rho * sMinus * w19(7);
#pragma unroll
    for (int qi = 1; qi < Q19; qi += 2) {
        const int qo = qi + 1;
        const float cu = cu19(qi, ueX, ueY, ueZ);
        const float ep = fmaf(R45, cu * cu, P);
        const float fp = fmaf(A1, f[qi] + f[qo], (qi <= 6 ? W1 : W2) * ep);
        const float fm = fmaf(A2, f[qi] - f[qo], (qi <= 6 ? M1 : M2) * cu);
        f[qi] = fp + fm;
        f[qo] = fp - fm;
    }
}

// f: pre-collision populations in -> post-collision out (the plain values f_i,
// or the deviations f_i - w_i when SHIFTED). Moments, guards, limiter, inlet
// override, LES tau, Guo force and TRT rate: aeros/src/lbm.cpp:1061-1299, same
// expression trees (compiled without contraction the plain form is bitwise
// the reference's float arithmetic).
// Shifted storage, no body force, a cell off the inlet/outlet planes: the
// same model in fewer instructions. The sums and differences of opposite
// populations are formed once (in place) and serve both the moments and the
// TRT update; reciprocals are single-instruction approximations (the shifted
// form is measured against the FP64 oracle, not bitwise the reference); the
// density guard and the velocity limiter are applied as in the full path.
// Returns false, with f untouched, when a population may be outside the clean
// range (the full path then replays the reference's per-population checks).
__device__ __forceinline__ bool collide19_shifted_fast(float f[Q19], const StepArgs& A, uint32_t d, float strainPre,
                                                       CellResult& o, Acc& acc) {
    float ss = 0.0f;
#pragma unroll
    for (int q = 0; q < Q19; ++q) ss = fmaf(f[q], f[q], ss);
    if (!(ss <= 1.0f)) return false;
    // f[qi] <- h_qi + h_qo, f[qo] <- h_qi - h_qo for the opposite pairs
    float drho = f[0], jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int qi = 2 * k + 1;
        const float p = f[qi] + f[qi + 1], m = f[qi] - f[qi + 1];
        f[qi] = p;
        f[qi + 1] = m;
        drho += p;
        if (cx19(qi) != 0) jx = cx19(qi) > 0 ? jx + m : jx - m;
        if (cy19(qi) != 0) jy = cy19(qi) > 0 ? jy + m : jy - m;
        if (cz19(qi) != 0) jz = cz19(qi) > 0 ? jz + m : jz - m;
    }
    float rho = 1.0f + drho;
    if (rho < 0.5f || rho > 1.5f) {   // density guard, lbm.cpp:1078-1080
        acc.rout++;
        acc.nan++;
        rho = 1.0f;
        drho = 0.0f;
    }
    const float invRho = __fdividef(1.0f, rho);
    float ux = jx * invRho, uy = jy * invRho, uz = jz * invRho;
    float usqr = ux * ux + uy * uy + uz * uz;
    if (usqr > 0.09f) {   // both limiters of the full path (lbm.cpp:1086-1090, 1148-1153)
        const float sc = sqrtf(0.09f / usqr);
        ux *= sc; uy *= sc; uz *= sc;
        usqr = ux * ux + uy * uy + uz * uz;
        if (usqr > 0.09f) {
            acc.ulim++;
            const float sc2 = sqrtf(0.09f / usqr);
            ux *= sc2; uy *= sc2; uz *= sc2;
            usqr = ux * ux + uy * uy + uz * uz;
        }
    }
    float tauEff = A.tau0, strainMag = 0.0f;
    if (A.use_les) {
        strainMag = strainPre;
        if (strainMag < 10.0f && strainMag > 1e-6f) {
            float cs = A.Cs;
            const int wd = (int)((d >> D_WD_SHIFT) & 7u);
            if (wd <= 5) cs *= van_driest(wd);
            tauEff = fminf(fmaxf(fmaf(cs * cs, strainMag * 3.0f, A.tau0), 0.51f), 1.5f);
        }
    }
    const float invTau = __fdividef(1.0f, tauEff);
    float sMinus = invTau;
    if (A.use_trt) {
        const float m = invTau - 0.5f;
        const float denom = (fabsf(m) > 1e-6f) ? (__fdividef(0.1875f, m) + 0.5f) : 1.0f;
        sMinus = __fdividef(1.0f, fmaxf(0.05f, denom));
    }
    // TRT on the deviations h = f - w: f^eq - w = w (P + 3 rho cu + 4.5 rho cu^2)
    // with P = rho - 1 - 1.5 rho |u|^2 (the symmetric part relaxes with 1/tau,
    // the antisymmetric with s-)
    const float P = drho - 1.5f * rho * usqr;
    const float R45 = 4.5f * rho;
    const float A1 = 0.5f * (1.0f - invTau), A2 = 0.5f * (1.0f - sMinus);
    const float W1 = invTau * w19(1), W2 = invTau * w19(7);
    const float M1 = 3.0f * rho * sMinus * w19(1), M2 = 3.0f * rho * sMinus * w19(7);
    f[0] = f[0] - invTau * (f[0] - w19(0) * P);
    float post = f[0] * f[0];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int qi = 2 * k + 1;
        const float cu = cu19(qi, ux, uy, uz);
        const float ep = fmaf(R45, cu * cu, P);
        const float fp = fmaf(A1, f[qi], (qi <= 6 ? W1 : W2) * ep);
        const float fm = fmaf(A2, f[qi + 1], (qi <= 6 ? M1 : M2) * cu);
        f[qi] = fp + fm;
        f[qi + 1] = fp - fm;
        post = fmaf(f[qi], f[qi], post);
        post = fmaf(f[qi + 1], f[qi + 1], post);
    }
    // negative post-collision populations: sum h^2 below the smallest weight
    // squared proves every f = h + w >= 0; otherwise count exactly
    if (!(post < (1.0f / 36.0f) * (1.0f / 36.0f))) {
#pragma unroll
        for (int q = 0; q < Q19; ++q) acc.neg += (f[q] + w19(q) < 0.0f) ? 1 : 0;
    }
    o.rho = rho;
    o.ux = ux; o.uy = uy; o.uz = uz;
    o.strain = strainMag;
    const float cS = A.Cs * strainMag;
    float tke = cS * cS * A.velScale2;
    if (!isfinite(tke) || tke < 0.0f) tke = 0.0f;
    if (tke > 1.0e6f) tke = 1.0e6f;
    o.tke = tke;
    o.usqr = usqr;
    acc.maxu2 = fmaxf(acc.maxu2, usqr);
    acc.drho += drho;
    acc.ke += usqr;
    acc.tke += tke;
    acc.cells++;
    return true;
}

// NOFORCE: the domain has no body force and no buoyancy (the force terms are
// compiled out; the results are the same as with zero forces).
template <bool SHIFTED, bool NOFORCE = false>
__device__ __forceinline__ void collide19(float f[Q19], const StepArgs& A, uint32_t d, bool isInlet, bool isOutlet,
                                          float strainPre, float buoy, CellResult& o, Acc& acc) {
    if (SHIFTED && A.shifted_fast && !isInlet && !isOutlet && collide19_shifted_fast(f, A, d, strainPre, o, acc)) return;
    // moments and the sum of squares of the populations in one pass
    float rho = 0.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f, ss = 0.0f;
#pragma unroll
    for (int q = 0; q < Q19; ++q) {
        const float m = f[q];
        rho += m;
        if (cx19(q) != 0) ux = cx19(q) > 0 ? ux + m : ux - m;
        if (cy19(q) != 0) uy = cy19(q) > 0 ? uy + m : uy - m;
        if (cz19(q) != 0) uz = cz19(q) > 0 ? uz + m : uz - m;
        ss = fmaf(m, m, ss);
    }
    // Only a non-finite population or one outside [-1, 10] lets the
    // reference's per-population replacement (lbm.cpp:1061-1074) change
    // anything; then it is replayed exactly. A rounded sum of squares <= 1
    // bounds every |f| by 1 (each rounded partial sum is >= every rounded
    // square so far) and is false for NaN / inf: the common case costs 19
    // FMAs. Otherwise the range is taken exactly. Shifted form: bounds on
    // h = f - w that imply f in [-1, 10].
    bool clean = ss <= 1.0f;
    if (!clean) {
        float fmn = f[0], fmx = f[0];
#pragma unroll
        for (int q = 1; q < Q19; ++q) { fmn = fminf(fmn, f[q]); fmx = fmaxf(fmx, f[q]); }
        clean = isfinite(rho) && fmn >= -1.0f && fmx <= (SHIFTED ? 9.6f : 10.0f);
    }
    if (!clean) {
        rho = 0.0f; ux = 0.0f; uy = 0.0f; uz = 0.0f;
#pragma unroll
        for (int q = 0; q < Q19; ++q) {
            float m = f[q];
            const float fi = SHIFTED ? m + w19(q) : m;
            if (!isfinite(fi)) { m = SHIFTED ? 0.0f : w19(q); acc.nan++; acc.bad++; }
            else if (fi < -1.0f || fi > 10.0f) { m = SHIFTED ? 0.0f : w19(q); acc.bad++; }
            rho += m;
            if (cx19(q) != 0) ux = cx19(q) > 0 ? ux + m : ux - m;
            if (cy19(q) != 0) uy = cy19(q) > 0 ? uy + m : uy - m;
            if (cz19(q) != 0) uz = cz19(q) > 0 ? uz + m : uz - m;
        }
    }
    if (SHIFTED) rho = 1.0f + rho;
    if (!isfinite(rho)) { acc.rnf++; acc.nan++; rho = 1.0f; }
    else if (rho < 0.5f || rho > 1.5f) { acc.rout++; acc.nan++; rho = 1.0f; }
    const float invRho = __frcp_rn(rho);   // correctly rounded: equals 1.0f / rho
    ux *= invRho; uy *= invRho; uz *= invRho;
    if (!isfinite(ux)) { ux = 0.0f; uy = 0.0f; uz = 0.0f; acc.nan++; }
    const float usqrTmp = ux * ux + uy * uy + uz * uz;
    if (usqrTmp > 0.09f) {
        const float sc = sqrtf(0.09f / usqrTmp);
        ux *= sc; uy *= sc; uz *= sc;
    }
    if (isInlet && !A.periodic_x) { rho = 1.0f; ux = A.uin[0]; uy = A.uin[1]; uz = A.uin[2]; }

    const float tau0 = A.tau0;
    float tauEff = tau0;
    float strainMag = 0.0f;
    if (A.use_les && !isInlet && !isOutlet) {
        strainMag = strainPre;
        if (isfinite(strainMag) && strainMag < 10.0f && strainMag > 1e-6f) {
            float cs = A.Cs;
            const int wd = (int)((d >> D_WD_SHIFT) & 7u);
            if (wd <= 5) cs *= van_driest(wd);
            const float nu_t = cs * cs * strainMag;
            tauEff = tau0 + nu_t / (1.0f / 3.0f);
            if (tauEff > 1.5f) tauEff = 1.5f;
            if (tauEff < 0.51f) tauEff = 0.51f;
        }
    }
    float usqr = ux * ux + uy * uy + uz * uz;
    if (usqr > 0.09f) {
        acc.ulim++;
        const float sc = sqrtf(0.09f / usqr);
        ux *= sc; uy *= sc; uz *= sc;
        usqr = ux * ux + uy * uy + uz * uz;
    }
    const float invTau = __frcp_rn(tauEff);
    const float Fx = A.Fx, Fz = A.Fz;
    const float Fy = A.th_on ? A.Fy + buoy : A.Fy;
    const bool hasForce = !NOFORCE && (Fx != 0.0f || Fy != 0.0f || Fz != 0.0f);
    float ueX = ux, ueY = uy, ueZ = uz, ueSqr = usqr;
    float halfInvRho = 0.0f;
    if (hasForce) {
        halfInvRho = __frcp_rn(rho) * 0.5f;   // equals 0.5f / rho (power-of-two scaling)
        ueX += Fx * halfInvRho; ueY += Fy * halfInvRho; ueZ += Fz * halfInvRho;
        ueSqr = ueX * ueX + ueY * ueY + ueZ * ueZ;
    }
    float sMinus = invTau;
    if (A.use_trt) {
        const float m = invTau - 0.5f;
        const float denom = (fabsf(m) > 1e-6f) ? (0.1875f / m + 0.5f) : 1.0f;
        sMinus = __frcp_rn(fmaxf(0.05f, denom));
    }
    const float drho = rho - 1.0f;
    if (SHIFTED && clean && A.fast_ok && !hasForce) {
        relax19_shifted_fast(f, rho, drho, ueX, ueY, ueZ, ueSqr, invTau, sMinus);
    } else if (clean && A.fast_ok) {
        if (hasForce) relax19<SHIFTED, false, true>(f, rho, drho, ueX, ueY, ueZ, ueSqr, invTau, sMinus, Fx, Fy, Fz);
        else relax19<SHIFTED, false, false>(f, rho, drho, ueX, ueY, ueZ, ueSqr, invTau, sMinus, Fx, Fy, Fz);
    } else {
        if (hasForce) relax19<SHIFTED, true, true>(f, rho, drho, ueX, ueY, ueZ, ueSqr, invTau, sMinus, Fx, Fy, Fz);
        else relax19<SHIFTED, true, false>(f, rho, drho, ueX, ueY, ueZ, ueSqr, invTau, sMinus, Fx, Fy, Fz);
    }
    // negative post-collision populations (lbmNegativePops): one minimum per
    // weight class, exact count only when one is negative
    {
        bool anyneg;
        if (SHIFTED) {
            float m0 = f[0], m1 = f[1], m2 = f[7];
#pragma unroll
            for (int q = 2; q <= 6; ++q) m1 = fminf(m1, f[q]);
#pragma unroll
            for (int q = 8; q < Q19; ++q) m2 = fminf(m2, f[q]);
            anyneg = m0 < -w19(0) || m1 < -w19(1) || m2 < -w19(7);
        } else {   // any sign bit (a -0.0 only triggers the exact count below)
            uint32_t sb = 0;
#pragma unroll
            for (int q = 0; q < Q19; ++q) sb |= __float_as_uint(f[q]);
            anyneg = (sb >> 31) != 0;
        }
        if (anyneg || !clean) {
#pragma unroll
            for (int q = 0; q < Q19; ++q) acc.neg += ((SHIFTED ? f[q] + w19(q) : f[q]) < 0.0f) ? 1 : 0;
        }
    }
    o.rho = rho;
    if (hasForce) {
        o.ux = ux + Fx * halfInvRho;
        o.uy = uy + Fy * halfInvRho;
        o.uz = uz + Fz * halfInvRho;
    } else {
        o.ux = ux; o.uy = uy; o.uz = uz;
    }
    o.strain = strainMag;
    const float tkeLb = (A.Cs * strainMag) * (A.Cs * strainMag);
    float tke = tkeLb * A.velScale2;
    if (!isfinite(tke) || tke < 0.0f) tke = 0.0f;
    if (tke > 1.0e6f) tke = 1.0e6f;
    o.tke = tke;
    o.usqr = usqr;
    acc.maxu2 = fmaxf(acc.maxu2, usqr);
    acc.drho += drho;
    acc.ke += usqr;
    acc.tke += tke;
    acc.cells++;
}

// Two-pass |S| from previous-step velocity (aeros/src/lbm.cpp:1012-1031).
__device__ __forceinline__ float strain_prev(const StepArgs& A, const StepVar& V, int c) {
    const float4 xm = __ldg(V.up + c - 1), xp = __ldg(V.up + c + 1);
    const float4 ym = __ldg(V.up + c - A.nx), yp = __ldg(V.up + c + A.nx);
    const float4 zm = __ldg(V.up + c - A.nxny), zp = __ldg(V.up + c + A.nxny);
    const float dux_dx = (xp.x - xm.x) * 0.5f;
    const float duy_dy = (yp.y - ym.y) * 0.5f;
    const float duz_dz = (zp.z - zm.z) * 0.5f;
    const float dux_dy = (yp.x - ym.x) * 0.5f;
    const float dux_dz = (zp.x - zm.x) * 0.5f;
    const float duy_dx = (xp.y - xm.y) * 0.5f;
    const float duy_dz = (zp.y - zm.y) * 0.5f;
    const float duz_dx = (xp.z - xm.z) * 0.5f;
    const float duz_dy = (yp.z - ym.z) * 0.5f;
    const float Sxx = dux_dx, Syy = duy_dy, Szz = duz_dz;
    const float Sxy = 0.5f * (dux_dy + duy_dx);
    const float Sxz = 0.5f * (dux_dz + duz_dx);
    const float Syz = 0.5f * (duy_dz + duz_dy);
    const float S2 = Sxx * Sxx + Syy * Syy + Szz * Szz + 2.0f * (Sxy * Sxy + Sxz * Sxz + Syz * Syz);
    return sqrtf(2.0f * S2);
}

__device__ __forceinline__ int plane_index(const StepArgs& A, int x, int y, int z) {
    return A.flow_axis == 0 ? y + A.ny * z : (A.flow_axis == 1 ? x + A.nx * z : x + A.nx * y);
}

// ---- thermal lattice (D3Q7), fused into the same thread -------------------------
// Dirichlet wall temperature seen from source row sy (thermal_lbm.cpp:60-65,283-286).
__device__ __forceinline__ bool th_dirichlet(const StepArgs& A, int sy, float& Tw) {
    if (!A.th_fixed) return false;
    if (sy <= 0) { Tw = A.th_hot; return true; }
    if (sy >= A.ny - 1) { Tw = A.th_cold; return true; }
    return false;
}

// Thermal link of population i at (x,y,z): X/Z always periodic, Y-out and
// solid sources bounce (anti-bounce-back at fixed-temperature walls).
struct TLink {
    int idx;       // source cell (regular) or own cell
    int bounce;    // 0 regular, 1 bounce, 2 Dirichlet
    float Tw;
};
__device__ __forceinline__ TLink th_resolve(const StepArgs& A, int x, int y, int z, int cell, int i, bool interior,
                                            uint32_t d, int kind = -1) {
    if (kind >= 0) {   // shell cell with the kind precomputed: 0 regular, 1 bounce, 2 Dirichlet
        if (kind == 0) {
            int sx = x - cx19(i), sz = z - cz19(i);
            if (sx < 0) sx = A.nx - 1; else if (sx >= A.nx) sx = 0;
            if (sz < 0) sz = A.nz - 1; else if (sz >= A.nz) sz = 0;
            return {(sz * A.ny + (y - cy19(i))) * A.nx + sx, 0, 0.0f};
        }
        const int sy = y - cy19(i);
        return {cell, kind, kind == 2 ? (sy <= 0 ? A.th_hot : A.th_cold) : 0.0f};
    }
    if (interior) {
        if (!((d >> i) & 1u)) return {cell - nb19(A, i), 0, 0.0f};
        float Tw = 0.0f;
        const bool dir = th_dirichlet(A, y - cy19(i), Tw) && (y - cy19(i) <= 0 || y - cy19(i) >= A.ny - 1);
        return {cell, dir ? 2 : 1, Tw};
    }
    int sx = x - cx19(i), sy = y - cy19(i), sz = z - cz19(i);
    if (sx < 0) sx = A.nx - 1; else if (sx >= A.nx) sx = 0;
    if (sz < 0) sz = A.nz - 1; else if (sz >= A.nz) sz = 0;
    float Tw = 0.0f;
    if (sy < 0 || sy >= A.ny) {
        const bool dir = th_dirichlet(A, sy < 0 ? 0 : A.ny - 1, Tw);
        return {cell, dir ? 2 : 1, Tw};
    }
    const int sc = (sz * A.ny + sy) * A.nx + sx;
    if (is_wall(A, sc)) {
        const bool dir = th_dirichlet(A, sy, Tw) && (sy <= 0 || sy >= A.ny - 1);
        return {cell, dir ? 2 : 1, Tw};
    }
    return {sc, 0, 0.0f};
}

// ---- the step ------------------------------------------------------------------
// MAT: materialize (write the gathered pre-collision populations, no step).
// ---- thermal sub-step (D3Q7), aeros/src/thermal_lbm.cpp:199-336 ----------------
// Gather (stream, with Dirichlet / adiabatic walls), BGK with this cell's new
// velocity, scatter. INTERIOR: links from the descriptor, unrolled;
// otherwise the shell's precomputed kinds, rolled loops.
// Shifted D3Q7 storage: a slot holds g_i - w_i Tc(y_w), Tc the conduction
// profile between fixed wall temperatures (Tref without fixed walls) and y_w
// the row of the cell that stored the value: the reader's own row on links
// that come back to it, its row - c_iy on a regular link. Far from the
// conduction state only the perturbation is stored, which 16 bits resolve.
// Writer and reader evaluate Tc of the same integer row: the same bits.
__device__ __forceinline__ float th_tc(const StepArgs& A, int yw) { return fmaf(A.th_tc1, (float)yw, A.th_tc0); }

template <class S, bool ODD, bool MAT, bool INTERIOR>
__device__ __forceinline__ void thermal_substep(const StepArgs& A, int cell, int x, int y, int z, uint32_t d,
                                                unsigned long long skind, const CellResult& r, Acc& acc) {
    constexpr bool SH = S::shifted;
    // shift of a value read as direction i: the storing row is y - c_iy on a
    // regular link (only i = 3, 4 have c_iy != 0; for them the descriptor's
    // link bit is exactly "not regular", y never wraps)
    auto rd_shift = [&](int i, bool regular) -> float {
        return SH ? w7(i) * th_tc(A, regular ? y - cy19(i) : y) : 0.0f;
    };
    const float tc_own = SH ? th_tc(A, y) : 0.0f;   // stored by this cell: g - w Tc(y)
    float g[Q7];
#pragma unroll
    for (int i = 0; i < Q7; ++i) {
        if (!ODD) {
            g[i] = S::load_rw(gplane<S>(A, i) + cell) + rd_shift(i, !((d >> i) & 1u));
        } else {
            const TLink L = th_resolve(A, x, y, z, cell, i, INTERIOR, d,
                                       INTERIOR ? -1 : (int)((skind >> (40 + 2 * i)) & 3ull));
            if (L.bounce == 0) {
                g[i] = S::load_rw(gplane<S>(A, opp19(i)) + L.idx) + rd_shift(i, true);
            } else {
                const float v = S::load_rw(gplane<S>(A, i) + cell) + rd_shift(i, false);   // post_{opp i}
                g[i] = L.bounce == 2 ? (-v + 2.0f * w7(i) * L.Tw) : v;
            }
        }
    }
    if (MAT) {
#pragma unroll
        for (int i = 0; i < Q7; ++i) A.mat_g[(long long)i * A.ncell + cell] = g[i];
        return;
    }
    float T = 0.0f;
#pragma unroll
    for (int i = 0; i < Q7; ++i) T += g[i];
    if (!isfinite(T)) T = A.th_tref;
    {
        const float lo = A.th_cold - 1.0f, hi = A.th_hot + 1.0f;
        const float m = (lo < T) ? T : lo;
        T = (m < hi) ? m : hi;
    }
    const float v[3] = {r.ux, r.uy, r.uz};
#pragma unroll
    for (int i = 0; i < Q7; ++i) {
        const float cu = i == 0 ? 0.0f : ((i & 1) ? v[(i - 1) >> 1] : -v[(i - 1) >> 1]);
        const float eq = w7(i) * T * (1.0f + 4.0f * cu);
        g[i] = g[i] - (g[i] - eq) * A.th_invtau;
    }
    A.T[cell] = T;
    acc.tsum += T;
    if (y == A.th_ylo) { acc.nu += (double)(A.th_hot - T) / 0.5; acc.nun++; }
#pragma unroll
    for (int j = 0; j < Q7; ++j) {
        if (!ODD) {
            S::store(gplane<S>(A, opp19(j)) + cell, g[j] - w7(j) * tc_own);
        } else {
            const TLink L = th_resolve(A, x, y, z, cell, opp19(j), INTERIOR, d,
                                       INTERIOR ? -1 : (int)((skind >> (40 + 2 * opp19(j))) & 3ull));
            if (L.bounce == 0) {
                S::store(gplane<S>(A, j) + L.idx, g[j] - w7(j) * tc_own);
            } else {
                // becomes pre-collision population opp j of this cell
                const float val = L.bounce == 2 ? (-g[j] + 2.0f * w7(j) * L.Tw) : g[j];
                S::store(gplane<S>(A, opp19(j)) + cell, val - w7(j) * tc_own);
            }
        }
    }
}

// Odd-step addressing by byte offsets, a kernel parameter of its own beside
// StepArgs (the many-domain kernel copies StepArgs into shared memory and
// keeps that copy unchanged): from a cell's slot in plane 0 to the slot
// population q is gathered from, ((opp q) * qstride - nb_q) * element size,
// and to the slot post-collision population j goes to, (j * qstride + nb_j)
// * element size.
struct StepOffsets {
    long long goff[Q19];
    long long soff[Q19];
};

// ---- interior cell (1 <= x,y,z <= N-2): flat neighbour offsets ---------------
// OFFS: odd-step gathers and scatters as one cell address plus the byte
// offsets O; otherwise plane pointer plus neighbour offset.
template <class S, bool ODD, bool THERMAL, bool MAT, bool OFFS = false>
__device__ __forceinline__ void process_interior(const StepArgs& A, const StepVar& V, int cell, int x, int y, int z,
                                                 Acc& acc, const uint32_t* dpre = nullptr,
                                                 const StepOffsets* O = nullptr) {
    const uint32_t d = dpre ? *dpre : A.desc[cell];
    constexpr bool SH = S::shifted;
    float f[Q19];
    float strainPre = 0.0f;
    if (!ODD) {
        // even step: every load is of the cell itself, in bounds whatever
        // the descriptor says, so all are issued before the descriptor
        // arrives (one memory round trip less on the critical path)
        const float strainAll = (!MAT && A.use_les) ? strain_prev(A, V, cell) : 0.0f;
#pragma unroll
        for (int q = 0; q < Q19; ++q) f[q] = ldp<S>(A, q, fplane<S>(A, q) + cell);
        if (d & D_WALL) return;
        if (d & D_LES) strainPre = strainAll;
    } else {
        // odd step: the descriptor first (the gather differs next to walls;
        // issuing both forms costs more registers than the round trip saves)
        if (d & D_WALL) return;
        if (!MAT && A.use_les && (d & D_LES)) strainPre = strain_prev(A, V, cell);
        // one address per cell; every gather is a constant byte offset from it
        const char* pc = static_cast<const char*>(A.f) + (long long)cell * (long long)sizeof(typename S::T);
        auto src = [&](int q) -> const typename S::T* {
            if constexpr (OFFS) return reinterpret_cast<const typename S::T*>(pc + O->goff[q]);
            else return fplane<S>(A, opp19(q)) + (cell - nb19(A, q));
        };
        if ((d & D_LINKS) == 0) {
#pragma unroll
            for (int q = 0; q < Q19; ++q) f[q] = ldp<S>(A, q, src(q));
        } else {
#pragma unroll
            for (int q = 0; q < Q19; ++q) {
                const bool special = (d >> q) & 1u;
                f[q] = ldp<S>(A, q, special ? fplane<S>(A, q) + cell : src(q));
            }
        }
    }
    const bool plain = (d & D_LINKS) == 0;   // no wall next to the cell
    float buoy = 0.0f;
    if (!MAT && THERMAL && A.th_buoy_mode != 1)
        buoy = A.th_glb * ((A.th_buoy_mode == 0 ? A.T[cell] : A.T_buoy[cell]) - A.th_tref);
    if (MAT) {
#pragma unroll
        for (int q = 0; q < Q19; ++q) A.mat_f[(long long)q * A.ncell + cell] = SH ? f[q] + w19(q) : f[q];
    }
    CellResult r;
    if (!MAT) {
        collide19<SH>(f, A, d, false, false, strainPre, buoy, r, acc);
        const uint32_t os = (d >> D_OUT_SHIFT) & 3u;   // planes Nx-2 / Nx-3 feed the outlet
        if (os) {
            const int P = A.out_plane;
            const int pi = plane_index(A, x, y, z);
#pragma unroll
            for (int q = 0; q < Q19; ++q) V.out_w[((int)(os - 1) * Q19 + q) * P + pi] = f[q];
        }
        if (!ODD) {
            if (!S::shifted || plain) {
#pragma unroll
                for (int j = 0; j < Q19; ++j) stp<S>(A, j, fplane<S>(A, opp19(j)) + cell, f[j]);
            } else {
#pragma unroll
                for (int j = 0; j < Q19; ++j) {
                    const bool solid = (d >> opp19(j)) & 1u;   // c + c_j is a wall: read back as opp j
                    stp<S>(A, solid ? opp19(j) : j, fplane<S>(A, opp19(j)) + cell, f[j]);
                }
            }
        } else {
            char* pc = static_cast<char*>(A.f) + (long long)cell * (long long)sizeof(typename S::T);
            auto dst = [&](int j) -> typename S::T* {
                if constexpr (OFFS) return reinterpret_cast<typename S::T*>(pc + O->soff[j]);
                else return fplane<S>(A, j) + (cell + nb19(A, j));
            };
            if (plain) {
#pragma unroll
                for (int j = 0; j < Q19; ++j) stp<S>(A, j, dst(j), f[j]);
            } else {
#pragma unroll
                for (int j = 0; j < Q19; ++j) {
                    const bool solid = (d >> opp19(j)) & 1u;   // target c + c_j is a wall
                    if (solid) stp<S>(A, opp19(j), fplane<S>(A, opp19(j)) + cell, f[j]);
                    else stp<S>(A, j, dst(j), f[j]);
                }
            }
        }
        if (V.write_u) V.uc[cell] = make_float4(r.ux, r.uy, r.uz, 0.0f);
        if (V.write_obs) { A.rho[cell] = r.rho; A.strain[cell] = r.strain; A.tke[cell] = r.tke; }
    }
    if (THERMAL) thermal_substep<S, ODD, MAT, true>(A, cell, x, y, z, d, 0ull, r, acc);
}

// ---- boundary-shell cell: precomputed link kinds -----------------------------
template <class S, bool ODD, bool THERMAL, bool MAT>
__device__ __forceinline__ void process_shell_body(const StepArgs& A, const StepVar& V, int si, int cell, int x, int y,
                                                   int z, unsigned long long skind, Acc& acc) {
    // the link kinds give in-domain sources for every shell cell: the
    // populations are loaded before the descriptor arrives
    const uint32_t d = A.desc[cell];
    constexpr bool SH = S::shifted;
    float f[Q19];
    const bool tables = ODD && A.shell_gth != nullptr;
    // the inlet override replaces every population of an inlet-plane cell
    // (lbm.cpp:1411-1429): nothing to load there
    const int apos = A.flow_axis == 0 ? x : (A.flow_axis == 1 ? y : z);
    const bool inlet_override = V.apply_overrides && !A.periodic_x && apos == A.inlet_pos;
    if (inlet_override) {
#pragma unroll
        for (int q = 0; q < Q19; ++q) f[q] = A.feq_in[q];
    } else if (tables) {   // precomputed sources: coalesced table loads instead of per-link index arithmetic
        const typename S::T* fb = reinterpret_cast<const typename S::T*>(A.f);
        uint32_t off[Q19];
#pragma unroll
        for (int q = 0; q < Q19; ++q) off[q] = __ldg(A.shell_gth + (size_t)q * A.n_shell + si);
#pragma unroll
        for (int q = 0; q < Q19; ++q) f[q] = ldp<S>(A, q, fb + off[q]);
    } else {
#pragma unroll
        for (int q = 0; q < Q19; ++q) {
            if (!ODD) {
                f[q] = ldp<S>(A, q, fplane<S>(A, q) + cell);
            } else {
                const Link L = resolve_kind(A, x, y, z, cell, q, (int)((skind >> (2 * q)) & 3ull));
                f[q] = ldp<S>(A, q, fplane<S>(A, L.slot) + L.idx);
            }
        }
    }
    if (d & D_WALL) return;
    float buoy = 0.0f;
    if (!MAT && THERMAL && A.th_buoy_mode != 1)
        buoy = A.th_glb * ((A.th_buoy_mode == 0 ? A.T[cell] : A.T_buoy[cell]) - A.th_tref);
    const bool isInlet = (d & D_INLET) != 0, isOutlet = (d & D_OUTLET) != 0;
    if (V.apply_overrides && !A.periodic_x) {
        if (isInlet) {
#pragma unroll
            for (int q = 0; q < Q19; ++q) f[q] = A.feq_in[q];
        } else if (isOutlet && A.outlet_mode) {
            const int P = A.out_plane;
            const int pi = plane_index(A, x, y, z);
            if (A.outlet_mode == 1) {
                // convective outlet, aeros/src/lbm.cpp:1465-1496
#pragma unroll
                for (int q = 0; q < Q19; ++q) {
                    const float fOut = V.out_r[(0 * Q19 + q) * P + pi];
                    const float fIn = V.out_r[(1 * Q19 + q) * P + pi];
                    const float fIn2 = V.out_r[(2 * Q19 + q) * P + pi];
                    const float df = fIn - fOut;
                    const float df2 = fIn - fIn2;
                    f[q] = fOut + A.conv * df + 0.15f * A.conv * df2;
                }
            } else {
                // zero-gradient: unknowns take the outlet plane's post value
                // pulled by the plane upstream (tangential shift)
                const int pos[3] = {x, y, z};
                const int n3[3] = {A.nx, A.ny, A.nz};
                const int per[3] = {A.periodic_x, 0, A.periodic_z};
#pragma unroll
                for (int q = 0; q < Q19; ++q) {
                    if (ca19(q, A.flow_axis) * A.flow_sign >= 0) continue;
                    int tpi;
                    if (A.zg_src) {   // precomputed at creation
                        tpi = __ldg(A.zg_src + q * P + pi);
                    } else {
                        int t[3] = {x - cx19(q), y - cy19(q), z - cz19(q)};
                        t[A.flow_axis] = pos[A.flow_axis];
                        for (int a = 0; a < 3; ++a) {
                            if (a == A.flow_axis) continue;
                            if (t[a] < 0 || t[a] >= n3[a]) t[a] = per[a] ? (t[a] + n3[a]) % n3[a] : pos[a];
                        }
                        const int tc = (t[2] * A.ny + t[1]) * A.nx + t[0];
                        tpi = is_wall(A, tc) ? pi : plane_index(A, t[0], t[1], t[2]);
                    }
                    f[q] = V.out_r[(0 * Q19 + q) * P + tpi];
                }
            }
        }
    }
    if (MAT) {
#pragma unroll
        for (int q = 0; q < Q19; ++q) A.mat_f[(long long)q * A.ncell + cell] = SH ? f[q] + w19(q) : f[q];
    }
    CellResult r;
    if (!MAT) {
        collide19<SH>(f, A, d, isInlet, isOutlet, 0.0f, buoy, r, acc);
        const uint32_t os = (d >> D_OUT_SHIFT) & 3u;
        if (os) {
            const int P = A.out_plane;
            const int pi = plane_index(A, x, y, z);
#pragma unroll
            for (int q = 0; q < Q19; ++q) V.out_w[((int)(os - 1) * Q19 + q) * P + pi] = f[q];
        }
        if (tables) {
            typename S::T* fb = reinterpret_cast<typename S::T*>(A.f);
            uint32_t off[Q19];
#pragma unroll
            for (int j = 0; j < Q19; ++j) off[j] = __ldg(A.shell_sct + (size_t)j * A.n_shell + si);
#pragma unroll
            for (int j = 0; j < Q19; ++j) {
                const int oj = opp19(j);
                const int kind = (int)((skind >> (2 * oj)) & 3ull);
                const int r = S::shifted ? reader_of(A, kind, x, y, z, j) : j;
                stp<S>(A, r, fb + off[j], kind == L_COPYOWN ? f[oj] : f[j]);
            }
        } else {
#pragma unroll
            for (int j = 0; j < Q19; ++j) {
                const int oj = opp19(j);
                const int kind = (int)((skind >> (2 * oj)) & 3ull);
                if (!ODD) {
                    const int r = S::shifted ? reader_of(A, kind, x, y, z, j) : j;
                    stp<S>(A, r, fplane<S>(A, oj) + cell, kind == L_COPYOWN ? f[oj] : f[j]);
                } else {
                    const Link L = resolve_kind(A, x, y, z, cell, oj, kind);
                    if (L.kind == L_REGULAR || L.kind == L_FREESLIP) stp<S>(A, L.slot, fplane<S>(A, L.slot) + L.idx, f[j]);
                    else if (L.kind == L_BOUNCE) stp<S>(A, oj, fplane<S>(A, oj) + cell, f[j]);
                    else stp<S>(A, oj, fplane<S>(A, oj) + cell, f[oj]);
                }
            }
        }
        if (V.write_u) V.uc[cell] = make_float4(r.ux, r.uy, r.uz, 0.0f);
        if (V.write_obs) { A.rho[cell] = r.rho; A.strain[cell] = r.strain; A.tke[cell] = r.tke; }
    }
    if (THERMAL) thermal_substep<S, ODD, MAT, false>(A, cell, x, y, z, d, skind, r, acc);
}

template <class S, bool ODD, bool THERMAL, bool MAT>
__device__ __noinline__ void process_shell_call(const StepArgs& A, const StepVar& V, int si, int cell, int x, int y,
                                                int z, unsigned long long skind, Acc& acc) {
    process_shell_body<S, ODD, THERMAL, MAT>(A, V, si, cell, x, y, z, skind, acc);
}

// 16-bit storage without the thermal lattice: the shell cell inline (measured
// on the 3.3 M-cell sphere, one box: FP16 step 0.1297 -> 0.1231 ms, 16-domain
// batch step 0.322 -> 0.308 ms). FP32 storage and the thermal lattice call it
// out of line (FP32 inline: 0.1521 -> 0.1533 ms).
template <class S, bool ODD, bool THERMAL, bool MAT>
__device__ __forceinline__ void process_shell(const StepArgs& A, const StepVar& V, int si, int cell, int x, int y, int z,
                                              unsigned long long skind, Acc& acc) {
    if constexpr (sizeof(typename S::T) == 2 && !THERMAL)
        process_shell_body<S, ODD, THERMAL, MAT>(A, V, si, cell, x, y, z, skind, acc);
    else
        process_shell_call<S, ODD, THERMAL, MAT>(A, V, si, cell, x, y, z, skind, acc);
}

// Block reduction of the per-thread accumulators into one partial (FP64),
// fixed shape: the result does not depend on warp scheduling.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int BLOCK>
__device__ __forceinline__ void block_reduce_store(const Acc& a, Partial* out) {
    __shared__ double sd[5][BLOCK / 32];
    __shared__ float sf[BLOCK / 32];
    __shared__ int si[8][BLOCK / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const double d0 = warp_sum((double)a.drho), d1 = warp_sum((double)a.ke), d2 = warp_sum((double)a.tke);
    const double d3 = warp_sum(a.nu), d4 = warp_sum((double)a.tsum);
    float mx = a.maxu2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    const int i0 = warp_sum(a.nan), i1 = warp_sum(a.neg), i2 = warp_sum(a.bad), i3 = warp_sum(a.rout);
    const int i4 = warp_sum(a.rnf), i5 = warp_sum(a.ulim), i6 = warp_sum(a.nun), i7 = warp_sum(a.cells);
    if (lane == 0) {
        sd[0][wid] = d0; sd[1][wid] = d1; sd[2][wid] = d2; sd[3][wid] = d3; sd[4][wid] = d4;
        sf[wid] = mx;
        si[0][wid] = i0; si[1][wid] = i1; si[2][wid] = i2; si[3][wid] = i3;
        si[4][wid] = i4; si[5][wid] = i5; si[6][wid] = i6; si[7][wid] = i7;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        Partial p;
        p.rho = p.ke = p.tke = p.nu = p.tsum = 0.0;
        p.maxu = 0.0f;
        p.nan = p.neg = p.bad = p.rout = p.rnf = p.ulim = p.nun = 0;
        p.pad[0] = 0;
        for (int w = 0; w < BLOCK / 32; ++w) {
            p.rho += sd[0][w]; p.ke += sd[1][w]; p.tke += sd[2][w]; p.nu += sd[3][w]; p.tsum += sd[4][w];
            p.maxu = fmaxf(p.maxu, sf[w]);
            p.nan += si[0][w]; p.neg += si[1][w]; p.bad += si[2][w]; p.rout += si[3][w];
            p.rnf += si[4][w]; p.ulim += si[5][w]; p.nun += si[6][w]; p.pad[0] += si[7][w];
        }
        *out = p;
    }
}

// Last block: sums the partials in block order and updates the control block
// (aeros/src/lbm.cpp:1313-1319 and 1554-1580).
static __device__ __noinline__ void apply_totals(const StepArgs& A, const double t[5], float m, const long long c[8]);
template <int BLOCK>
__device__ void finish_totals(const StepArgs& A, const Partial* parts, int nparts);

template <int BLOCK>
__device__ void finish_step(const StepArgs& A, int nparts) {
    __shared__ bool last;
    __threadfence();
    if (threadIdx.x == 0) last = (atomicAdd(&A.ctl->blocks_done, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    finish_totals<BLOCK>(A, A.partials, nparts);
}

// All threads of one block: sums nparts partials in a fixed order (FP64) and
// updates the domain's control block.
template <int BLOCK>
__device__ void finish_totals(const StepArgs& A, const Partial* parts, int nparts) {
    double t[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    float m = 0.0f;
    long long c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < nparts; b += BLOCK) {
        const volatile Partial* p = parts + b;
        t[0] += p->rho; t[1] += p->ke; t[2] += p->tke; t[3] += p->nu; t[4] += p->tsum;
        m = fmaxf(m, p->maxu);
        c[0] += p->nan; c[1] += p->neg; c[2] += p->bad; c[3] += p->rout;
        c[4] += p->rnf; c[5] += p->ulim; c[6] += p->nun; c[7] += p->pad[0];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        for (int k = 0; k < 5; ++k) t[k] += __shfl_down_sync(0xffffffffu, t[k], o);
        m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
        for (int k = 0; k < 8; ++k) c[k] += __shfl_down_sync(0xffffffffu, c[k], o);
    }
    __shared__ double s_d[5][BLOCK / 32];
    __shared__ float s_m[BLOCK / 32];
    __shared__ long long s_i[8][BLOCK / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        for (int k = 0; k < 5; ++k) s_d[k][wid] = t[k];
        s_m[wid] = m;
        for (int k = 0; k < 8; ++k) s_i[k][wid] = c[k];
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int j = 1; j < BLOCK / 32; ++j) {
        for (int k = 0; k < 5; ++k) t[k] += s_d[k][j];
        m = fmaxf(m, s_m[j]);
        for (int k = 0; k < 8; ++k) c[k] += s_i[k][j];
    }
    apply_totals(A, t, m, c);
}

// Updates the domain's control block from the step's totals: t = sums of
// (rho - 1), |u|^2, TKE, Nusselt rows, T; m = max |u|^2; c = counters (NaN,
// negative, bad, rho out of range, rho non-finite, u limited, Nusselt cells,
// fluid cells). One thread.
static __device__ __noinline__ void apply_totals(const StepArgs& A, const double t[5], float m, const long long c[8]) {
    Control* ctl = A.ctl;
    ctl->blocks_done = 0;
    ctl->tile_next = 0;
    ctl->kexec += 1;
    ctl->nan = c[0];
    if (c[0] > A.total_div10) {   // diverged before streaming: step not counted
        ctl->halt = 1;
        ctl->halt_kind = 1;
        return;
    }
    ctl->steps += 1;
    const double sum_rho = (double)c[7] + t[0];   // cells + sum of (rho - 1)
    ctl->sum_rho = sum_rho; ctl->sum_ke = t[1]; ctl->sum_tke = t[2];
    const float avg_rho = (float)(sum_rho / A.fluid_cells);
    const float avg_ke = (float)(t[1] / A.fluid_cells);
    ctl->avg_rho = avg_rho;
    ctl->avg_ke = avg_ke;
    ctl->avg_tke = (float)(t[2] / A.fluid_cells);
    ctl->max_u = sqrtf(m);
    ctl->neg = c[1]; ctl->bad = c[2]; ctl->rout = c[3]; ctl->rnf = c[4]; ctl->ulim = c[5];
    ctl->convergence = fabsf(avg_ke - ctl->prev_kinetic);
    ctl->prev_kinetic = avg_ke;
    ctl->converged = ctl->convergence < A.conv_threshold;
    if (A.th_on) {
        if (c[6] > 0) {
            float dT = fabsf(A.th_hot - A.th_cold);
            if (dT < 1e-6f) dT = 1e-6f;
            ctl->nusselt = (float)(t[3] / (double)c[6]) * A.th_H / dT;
            ctl->th_valid = 1;
        }
        ctl->mean_t = A.th_rows_n > 0.0 ? (float)(t[4] / A.th_rows_n) : 0.5f;
    }
    if (!isfinite(avg_rho) || avg_rho > 1.2f || avg_rho < 0.8f) {
        ctl->halt = 1;
        ctl->halt_kind = 2;
    }
}

// Shell cell si (shell cells are listed in increasing cell order).
template <class S, bool ODD, bool THERMAL, bool MAT>
__device__ __forceinline__ void shell_cell(const StepArgs& A, const StepVar& V, int si, Acc& acc) {
    if (si < A.n_shell) {
        const int cell = A.shell[si];
        const uint32_t r = A.div_x.div((uint32_t)cell);
        const int x = cell - (int)r * A.nx;
        const uint32_t z = A.div_y.div(r);
        const int y = (int)(r - z * (uint32_t)A.ny);
        process_shell<S, ODD, THERMAL, MAT>(A, V, si, cell, x, y, (int)z, A.shell_kind[si], acc);
    }
}

// Interior cell li: the interior (x, y, z in 1 .. n-2) in x-fastest order.
// dpre: its descriptor, already loaded (NULL: load it here).
template <class S, bool ODD, bool THERMAL, bool MAT, bool OFFS = false>
__device__ __forceinline__ void interior_cell(const StepArgs& A, const StepVar& V, int li, Acc& acc,
                                              const uint32_t* dpre = nullptr, const StepOffsets* O = nullptr) {
    if (li < A.n_interior) {
        const uint32_t r = A.div_ix.div((uint32_t)li);
        const int x = li - (int)r * (A.nx - 2) + 1;
        const uint32_t zq = A.div_iy.div(r);
        const int y = (int)(r - zq * (uint32_t)(A.ny - 2)) + 1;
        const int z = (int)zq + 1;
        process_interior<S, ODD, THERMAL, MAT, OFFS>(A, V, (z * A.ny + y) * A.nx + x, x, y, z, acc, dpre, O);
    }
}

template <class S, bool ODD, bool THERMAL, bool MAT>
__device__ __forceinline__ void shell_tile(const StepArgs& A, const StepVar& V, int st, Acc& acc) {
    shell_cell<S, ODD, THERMAL, MAT>(A, V, st * STEP_BLOCK + (int)threadIdx.x, acc);
}

template <class S, bool ODD, bool THERMAL, bool MAT, bool OFFS = false>
__device__ __forceinline__ void interior_tile(const StepArgs& A, const StepVar& V, int it, Acc& acc,
                                              const StepOffsets* O = nullptr) {
    interior_cell<S, ODD, THERMAL, MAT, OFFS>(A, V, it * STEP_BLOCK + (int)threadIdx.x, acc, nullptr, O);
}

template <class S, bool ODD, bool THERMAL, bool MAT>
__device__ __forceinline__ void process_tile(const StepArgs& A, const StepVar& V, int tile, Acc& acc) {
    // Shell tiles (costlier: per-link index arithmetic) are spread evenly
    // through the tile sequence: tile t is shell tile t / k when t % k == 0.
    const int nsh = A.ntiles - A.ntiles_interior;
    const int k = A.shell_stride;
    const bool is_shell = nsh > 0 && (tile % k) == 0 && tile / k < nsh;
    if (is_shell) shell_tile<S, ODD, THERMAL, MAT>(A, V, tile / k, acc);
    else interior_tile<S, ODD, THERMAL, MAT>(A, V, tile - min(nsh, tile / k + 1), acc);
}

// One lattice step. Tiles of STEP_BLOCK cells are assigned round-robin to a
// persistent grid (a fixed assignment, so the statistics are deterministic).
template <class S, bool ODD, bool THERMAL, bool MAT>
__global__ void __launch_bounds__(STEP_BLOCK, STEP_MIN_BLOCKS) k_lbm_step(const StepArgs A, const StepVar V) {
    if (!MAT && A.ctl->halt) return;   // uniform: every thread reads the same flag
    Acc acc;
    acc.zero();
    for (int tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) process_tile<S, ODD, THERMAL, MAT>(A, V, tile, acc);
    if (MAT) return;
    block_reduce_store<STEP_BLOCK>(acc, A.partials + blockIdx.x);
    finish_step<STEP_BLOCK>(A, (int)gridDim.x);
}

// The same step as two launches on one stream: the boundary shell first, then
// the interior, whose code then runs without the shell path beside it in the
// instruction cache. The shell grid stores its partials after the interior
// grid's (slots A.shell_part_base ...); the interior grid's last block sums both.
template <class S, bool ODD, bool THERMAL>
__global__ void __launch_bounds__(STEP_BLOCK, STEP_MIN_BLOCKS) k_lbm_shell(const StepArgs A, const StepVar V) {
    if (A.ctl->halt) return;
    Acc acc;
    acc.zero();
    const int nsh = A.ntiles - A.ntiles_interior;
    for (int st = blockIdx.x; st < nsh; st += gridDim.x) shell_tile<S, ODD, THERMAL, false>(A, V, st, acc);
    block_reduce_store<STEP_BLOCK>(acc, A.partials + A.shell_part_base + blockIdx.x);
}

template <class S, bool ODD, bool THERMAL>
__global__ void __launch_bounds__(STEP_BLOCK, STEP_MIN_BLOCKS) k_lbm_interior(const StepArgs A, const StepVar V) {
    if (A.ctl->halt) return;
    Acc acc;
    acc.zero();
    for (int it = blockIdx.x; it < A.ntiles_interior; it += gridDim.x) interior_tile<S, ODD, THERMAL, false>(A, V, it, acc);
    block_reduce_store<STEP_BLOCK>(acc, A.partials + blockIdx.x);
    finish_step<STEP_BLOCK>(A, A.shell_part_base + A.shell_grid);
}

struct WarpSums {               // one warp's sums over the slices of a work item
    long long drho, ke, tke;    // fixed point
    long long cnt[7];           // NaN, negative, bad, rho range, rho finite, u limited, cells
    long long nu, tsum, nun;    // thermal: fixed point, fixed point, count
};

// Fixed-point units of the per-cell statistics. Each cell's value is rounded
// to its unit once and the integers are summed exactly (warp redux, then
// 64-bit atomics), so the totals do not depend on how cells are grouped into
// slices, blocks or launches.
constexpr float FX_DRHO = 16777216.0f;         // 2^24: rho - 1 (|rho - 1| <= 0.5; exact for the plain form)
constexpr float FX_KE = 1099511627776.0f;      // 2^40: |u|^2 (<= 0.09 after the limiter)
constexpr float FX_TKE = 1073741824.0f;        // 2^30: TKE (0 .. 1e6)
constexpr double FX_NU = 4294967296.0;       // 2^32: Nusselt row terms per slice (|term| <= 4)
constexpr float FX_T = 16777216.0f;          // 2^24: temperatures per slice (|T| <= 1.5)

// Exact warp sum of a non-negative value in units of 1/scale (x * scale <
// 2^50): high and low 24-bit parts are summed by redux separately.
__device__ __forceinline__ long long warp_fixed_sum(float x, float scale) {
    const float y = x * scale;
    const float hi = floorf(y * 0x1p-24f);
    const unsigned h = (unsigned)hi;
    const unsigned l = (unsigned)(y - hi * 0x1p24f);
    return ((long long)__reduce_add_sync(0xffffffffu, h) << 24) + (long long)__reduce_add_sync(0xffffffffu, l);
}

__device__ __forceinline__ float warp_allsum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_allsum(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---- one launch per step: shell blocks beside dynamic interior blocks -------------
// The grid is A.shell_blocks + the persistent interior grid. The first
// A.shell_blocks blocks (dispatched first: about one per SM) take the
// boundary-shell tiles, whose cost is latency, while the co-resident interior
// blocks stream the interior; interior blocks take 256-cell tiles from a
// global counter, so the blocks dispatched once the shell blocks retire share
// the remaining tiles. Each 32-cell slice's sums are converted to 64-bit fixed
// point and accumulated exactly, so the statistics do not depend on which
// block took which tile.
#ifndef AEROS_FUSED_MIN_BLOCKS
#define AEROS_FUSED_MIN_BLOCKS 8
#endif
#ifndef AEROS_BATCH_MIN_BLOCKS
#define AEROS_BATCH_MIN_BLOCKS 4
#endif

#ifndef AEROS_FUSED_ODD_MIN_BLOCKS
#define AEROS_FUSED_ODD_MIN_BLOCKS AEROS_FUSED_MIN_BLOCKS
#endif

// Linear cell index of interior cell li (x-fastest over x, y, z in 1 .. n-2).
__device__ __forceinline__ int interior_cell_index(const StepArgs& A, int li) {
    const uint32_t r = A.div_ix.div((uint32_t)li);
    const int x = li - (int)r * (A.nx - 2) + 1;
    const uint32_t zq = A.div_iy.div(r);
    const int y = (int)(r - zq * (uint32_t)(A.ny - 2)) + 1;
    return (((int)zq + 1) * A.ny + y) * A.nx + x;
}

#ifndef AEROS_FUSED_TH_MIN_BLOCKS
#define AEROS_FUSED_TH_MIN_BLOCKS 6
#endif

// One 32-cell slice's statistics into the warp's running sums: FP32 warp sums
// (a fixed shuffle tree over a fixed set of cells) converted to 64-bit fixed
// point, so that the totals do not depend on which block took which slice.
template <bool THERMAL>
__device__ __forceinline__ void add_slice_sums(WarpSums& W, const Acc& acc, float& mx, int lane) {
    const long long sd = (int)__reduce_add_sync(0xffffffffu, (unsigned)__float2int_rn(acc.drho * FX_DRHO));
    const long long sk = warp_fixed_sum(acc.ke, FX_KE), st = warp_fixed_sum(acc.tke, FX_TKE);
    mx = fmaxf(mx, acc.maxu2);
    const int cells = __popc(__ballot_sync(0xffffffffu, acc.cells != 0));
    const bool rare = __any_sync(0xffffffffu, (acc.nan | acc.neg | acc.bad | acc.rout | acc.rnf | acc.ulim) != 0);
    int c6[6] = {0, 0, 0, 0, 0, 0};
    if (rare) {
        c6[0] = warp_allsum(acc.nan); c6[1] = warp_allsum(acc.neg); c6[2] = warp_allsum(acc.bad);
        c6[3] = warp_allsum(acc.rout); c6[4] = warp_allsum(acc.rnf); c6[5] = warp_allsum(acc.ulim);
    }
    if (lane == 0) {
        W.drho += sd;
        W.ke += sk;
        W.tke += st;
        W.cnt[6] += cells;
        if (rare)
            for (int j = 0; j < 6; ++j) W.cnt[j] += c6[j];
    }
    if constexpr (THERMAL) {
        double nu = acc.nu;   // a fixed shuffle tree over the slice's cells
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nu += __shfl_xor_sync(0xffffffffu, nu, o);
        const float ts = warp_allsum(acc.tsum);
        const int nun = (int)__reduce_add_sync(0xffffffffu, (unsigned)acc.nun);
        if (lane == 0) {
            W.nu += __double2ll_rn(nu * FX_NU);
            W.tsum += __float2ll_rn(ts * FX_T);
            W.nun += nun;
        }
    }
}

// A warp's sums of the step into the domain's fixed-point accumulators; the
// last of the step's `nwarps` callers (warps, or blocks when one warp per
// block calls for its block) applies the totals (statistics, divergence
// guard, Nusselt number) and rewinds the accumulators for the next step.
template <bool THERMAL>
__device__ __forceinline__ void finish_warp_sums(const StepArgs& A, const WarpSums& W, float mx, int lane,
                                                 unsigned int nwarps) {
    Control* ctl = A.ctl;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __syncwarp();
    if (lane == 0) atomicAdd(&ctl->fx_drho, (unsigned long long)W.drho);
    else if (lane == 1) atomicAdd(&ctl->fx_ke, (unsigned long long)W.ke);
    else if (lane == 2) atomicAdd(&ctl->fx_tke, (unsigned long long)W.tke);
    else if (lane >= 3 && lane < 10 && W.cnt[lane - 3]) atomicAdd(&ctl->fx_cnt[lane - 3], (unsigned long long)W.cnt[lane - 3]);
    else if (lane == 10 && mx > 0.0f) atomicMax(&ctl->fx_maxu2, __float_as_uint(mx));
    else if (THERMAL && lane == 11) atomicAdd(&ctl->fx_nu, (unsigned long long)W.nu);
    else if (THERMAL && lane == 12) atomicAdd(&ctl->fx_tsum, (unsigned long long)W.tsum);
    else if (THERMAL && lane == 13) atomicAdd(&ctl->fx_nun, (unsigned long long)W.nun);
    __threadfence();
    __syncwarp();
    int last = 0;
    if (lane == 0) last = atomicAdd(&ctl->warps_done, 1u) == nwarps - 1;
    if (__shfl_sync(0xffffffffu, last, 0) && lane == 0) {
        __threadfence();
        volatile Control* vc = ctl;
        const double t[5] = {(double)(long long)vc->fx_drho / (double)FX_DRHO, (double)(long long)vc->fx_ke / (double)FX_KE,
                             (double)(long long)vc->fx_tke / (double)FX_TKE,
                             THERMAL ? (double)(long long)vc->fx_nu / FX_NU : 0.0,
                             THERMAL ? (double)(long long)vc->fx_tsum / (double)FX_T : 0.0};
        const long long c[8] = {(long long)vc->fx_cnt[0], (long long)vc->fx_cnt[1], (long long)vc->fx_cnt[2],
                                (long long)vc->fx_cnt[3], (long long)vc->fx_cnt[4], (long long)vc->fx_cnt[5],
                                THERMAL ? (long long)vc->fx_nun : 0, (long long)vc->fx_cnt[6]};
        const float m = __uint_as_float(vc->fx_maxu2);
        vc->fx_drho = 0; vc->fx_ke = 0; vc->fx_tke = 0;
        for (int j = 0; j < 7; ++j) vc->fx_cnt[j] = 0;
        vc->fx_nu = 0; vc->fx_tsum = 0; vc->fx_nun = 0;
        vc->fx_maxu2 = 0;
        vc->warps_done = 0;
        apply_totals(A, t, m, c);   // also rewinds tile_next
    }
}

// The block's warp sums into the step's accumulators, by its first warp: one
// fence per block instead of one per warp (a fence waits for the fencing
// thread's own outstanding stores; the finisher reads only the accumulators,
// which the first warp writes, so the other warps' stores need no ordering).
// The last block to arrive applies the totals.
template <bool THERMAL>
__device__ __forceinline__ void finish_block_sums(const StepArgs& A, const WarpSums* s_sums, float* s_mx, float mx,
                                                  int lane, int wid) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s_mx[wid] = mx;
    __syncthreads();
    if (wid != 0) return;
    WarpSums W = s_sums[0];
    float m = s_mx[0];
#pragma unroll
    for (int w = 1; w < STEP_BLOCK / 32; ++w) {
        const WarpSums& o = s_sums[w];
        W.drho += o.drho; W.ke += o.ke; W.tke += o.tke;
        for (int j = 0; j < 7; ++j) W.cnt[j] += o.cnt[j];
        W.nu += o.nu; W.tsum += o.tsum; W.nun += o.nun;
        m = fmaxf(m, s_mx[w]);
    }
    finish_warp_sums<THERMAL>(A, W, m, lane, gridDim.x);
}

// The single-launch step: the first shell_blocks blocks take the boundary
// shell's tiles, the others take interior tiles from a counter (QUEUE: no
// shell blocks, the counter hands out the shell's tiles first). THERMAL: the
// D3Q7 lattice stepped in the same thread (its Nusselt row sum and mean
// temperature summed like the other statistics, in fixed point).
template <class S, bool ODD, bool THERMAL, bool QUEUE>
__global__ void __launch_bounds__(STEP_BLOCK, THERMAL ? AEROS_FUSED_TH_MIN_BLOCKS
                                                      : (ODD ? AEROS_FUSED_ODD_MIN_BLOCKS : AEROS_FUSED_MIN_BLOCKS))
    k_lbm_fused(const StepArgs A, const StepVar V, const StepOffsets O) {
    if (A.ctl->halt) return;   // uniform: every thread reads the same flag
    __shared__ WarpSums s_sums[STEP_BLOCK / 32];
    __shared__ int s_tile[2];
    const int lane = (int)(threadIdx.x & 31u), wid = (int)(threadIdx.x >> 5);
    WarpSums& W = s_sums[wid];
    if (lane == 0) {
        W.drho = W.ke = W.tke = 0;
        for (int j = 0; j < 7; ++j) W.cnt[j] = 0;
        W.nu = W.tsum = W.nun = 0;
    }
    __syncwarp();
    float mx = 0.0f;
    Control* ctl = A.ctl;
    auto add_slice = [&](const Acc& acc) { add_slice_sums<THERMAL>(W, acc, mx, lane); };
    const int nsh = A.ntiles - A.ntiles_interior;
    const int nq = QUEUE ? nsh : 0;   // shell tiles handed out by the counter
    const int nall = nq + A.ntiles_interior;
    int par = 0;
    int it = 0;
    if (!QUEUE && (int)blockIdx.x < A.shell_blocks) {
        for (int st = blockIdx.x; st < nsh; st += A.shell_blocks) {
            Acc acc;
            acc.zero();
            shell_tile<S, ODD, THERMAL, false>(A, V, st, acc);
            add_slice(acc);
        }
        it = nall;
    } else if (QUEUE) {
        // The counter only grows: a block that has drawn an interior tile
        // never draws a shell tile again, and the interior loops below hold
        // no shell code.
        for (;;) {
            if (threadIdx.x == 0) s_tile[par] = (int)atomicAdd(&ctl->tile_next, 1u);
            __syncthreads();
            it = s_tile[par];
            par ^= 1;
            if (it >= nq) break;
            Acc acc;
            acc.zero();
            shell_tile<S, ODD, THERMAL, false>(A, V, it, acc);
            add_slice(acc);
        }
    } else {
        if (threadIdx.x == 0) s_tile[par] = (int)atomicAdd(&ctl->tile_next, 1u);
        __syncthreads();
        it = s_tile[par];
        par ^= 1;
    }
    if (ODD) {
        // Odd steps read the descriptor before the gathers; the next tile's
        // index is taken a tile ahead so that each thread's next interior
        // descriptor is in flight while the current cell is processed.
        uint32_t dnext = D_WALL;
        int cnext = 0;
        if (it < nall) {
            const int li = (it - nq) * STEP_BLOCK + (int)threadIdx.x;
            if (li < A.n_interior) {
                cnext = interior_cell_index(A, li);
                dnext = __ldg(A.desc + cnext);
            }
        }
        while (it < nall) {
            if (threadIdx.x == 0) s_tile[par] = (int)atomicAdd(&ctl->tile_next, 1u);
            __syncthreads();
            const int itn = s_tile[par];
            par ^= 1;
            const uint32_t dcur = dnext;
            const int ccur = cnext;
            if (itn < nall) {
                const int li = (itn - nq) * STEP_BLOCK + (int)threadIdx.x;
                if (li < A.n_interior) {
                    cnext = interior_cell_index(A, li);
                    dnext = __ldg(A.desc + cnext);
                }
            }
            Acc acc;
            acc.zero();
            if ((it - nq) * STEP_BLOCK + (int)threadIdx.x < A.n_interior) {
                // x, y, z from the cell index: only the outlet planes and the
                // thermal sub-step use them
                const uint32_t r = A.div_x.div((uint32_t)ccur);
                const int x = ccur - (int)r * A.nx;
                const uint32_t z = A.div_y.div(r);
                const int y = (int)(r - z * (uint32_t)A.ny);
                process_interior<S, ODD, THERMAL, false, true>(A, V, ccur, x, y, (int)z, acc, &dcur, &O);
            }
            add_slice(acc);
            it = itn;
        }
    } else {
        while (it < nall) {
            Acc acc;
            acc.zero();
            interior_tile<S, ODD, THERMAL, false, true>(A, V, it - nq, acc, &O);
            add_slice(acc);
            if (threadIdx.x == 0) s_tile[par] = (int)atomicAdd(&ctl->tile_next, 1u);
            __syncthreads();
            it = s_tile[par];
            par ^= 1;
        }
    }
    __shared__ float s_mx[STEP_BLOCK / 32];
    finish_block_sums<THERMAL>(A, s_sums, s_mx, mx, lane, wid);
}

// ---- warp-tiled interior: 16-byte async copies into per-warp shared memory ------
// Each warp of an interior block steps tiles of WT = 32 * M consecutive cells
// (tile t holds cells t*WT .. t*WT + WT - 1, lane l the cells l + 32 m; lanes
// of shell and wall cells idle) from wt_first to wt_last, taken from a global
// counter two tiles ahead. What a tile reads reaches the warp's shared
// memory by cp.async 16-byte copies, which hold no registers while in flight,
// and no barrier wider than the warp is taken:
//   populations and descriptors, double buffered: the next tile's copies fly
//   while the warp steps the current one. Rows:
//     even step: plane q at cells c0 .. c0 + WT - 1 (the slots the cells read);
//     odd step : the plane direction q gathers from (opp q) at c0 - nb_q,
//                moved back to a 16-byte boundary (moff(q)), WT + PAD long;
//   the previous step's velocity rows for the |S| stencil (LES), one buffer:
//     the x-row c0 - 16 .. c0 + WT + 15 and the rows at -nx, +nx, -nx*ny,
//     +nx*ny. The strains of a tile are taken first, then the next tile's rows
//     are requested, so they arrive while this tile collides.
// A cell reads exactly the slots it writes (AA pattern), so results go back
// into the rows in place. Even steps then write the rows out as 16-byte
// stores (a chunk holding a shell cell, whose slots the shell blocks write,
// goes out element by element); odd steps scatter from registers. Wall cells
// of an even tile are written back unchanged: no thread writes a wall slot.
// Requires nx a multiple of PAD (every row starts on a 16-byte boundary at a
// fixed offset per direction), nx*ny >= WT (tiles stay inside the domain),
// the population array below 2 GiB (32-bit chunk offsets) and velocity
// buffers with VEL_GUARD cells of slack on both sides.
#ifndef AEROS_WARP_M16
#define AEROS_WARP_M16 1   // cells per lane of a tile, 16-bit storage
#endif
#ifndef AEROS_WARP_M32
#define AEROS_WARP_M32 1   // cells per lane of a tile, FP32 storage
#endif
constexpr int VEL_GUARD = 512;   // velocity cells of slack before and after each buffer

// Per-lane exact sums of a warp's cells, in the warp's shared memory (no
// registers held across tiles).
struct LaneSums {
    long long drho[32], ke[32], tke[32];
    int cells[32];
};

template <class S>
struct WarpLayout {
    using T = typename S::T;
    static constexpr int ESZ = (int)sizeof(T);
    static constexpr int M = ESZ == 4 ? AEROS_WARP_M32 : AEROS_WARP_M16;
    static constexpr int PAD = 16 / ESZ;                 // elements per 16-byte chunk
    static constexpr int WT = 32 * M;                    // cells per tile
    static constexpr int CH_E = WT / PAD, CH_O = CH_E + 1;   // chunks per row (even / odd step)
    static constexpr int ROW_E = CH_E * 16, ROW_O = CH_O * 16;
    static constexpr int NCH_E = Q19 * CH_E, NCH_O = Q19 * CH_O;
    static constexpr int K_E = (NCH_E + 31) / 32, K_O = (NCH_O + 31) / 32;   // chunks per lane
    static constexpr int DESC = WT * 4;                  // descriptor bytes of a tile
    static constexpr int OFF_DESC = NCH_O * 16;          // descriptors after the rows
    static constexpr int BUF = OFF_DESC + DESC;          // one tile's populations and descriptors
    static constexpr int VX = WT + 32;                   // x-row of velocities: c0 - 16 .. c0 + WT + 15
    static constexpr int VEL = (VX + 4 * WT) * 16;       // velocity rows of a tile (float4)
    static constexpr int TAB = K_O * 32 * 4;             // per-lane chunk offsets
    static constexpr int SUMS = (int)((sizeof(LaneSums) + 15) / 16 * 16);
    static constexpr int OFF_VEL = 2 * BUF, OFF_TAB = OFF_VEL + VEL, OFF_SUMS = OFF_TAB + TAB;
    static constexpr int WARP = OFF_SUMS + SUMS;         // shared memory of one warp
    static constexpr int BYTES = (STEP_BLOCK / 32) * WARP;   // dynamic shared memory of a block
    // blocks that fit an SM's 228 KB of shared memory (1 KB reserved per
    // block): the register budget of the launch bounds follows
    static constexpr int MIN_BLOCKS = 233472 / (BYTES + 1024) < 8 ? 233472 / (BYTES + 1024) : 8;
    static_assert(M >= 1 && M <= 4 && DESC / 16 <= 32, "tile shape");
    static_assert(BUF % 16 == 0 && WARP % 16 == 0, "16-byte chunks");
    static_assert(WT + 32 <= VEL_GUARD, "velocity guard: rows reach WT + 16 cells past the domain");
    // odd-step element offset of a cell in the row of direction q: the row
    // starts at c0 - nb_q - moff(q), and nb_q = c_x modulo PAD when nx is a
    // multiple of PAD
    __host__ __device__ static constexpr int moff(int q) {
        return cx19(q) > 0 ? PAD - 1 : (cx19(q) < 0 ? 1 : 0);
    }
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// 16-byte global -> shared copy, cached in L2 only (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Exact statistics of the lanes' cells (LaneSums): each cell's values are
// rounded once to the fixed-point units of WarpSums and added as integers,
// the same integers the slice sums of the other kernels add, so the totals do
// not depend on which warp stepped which cell.
// x * scale (non-negative, < 2^50) as the integer warp_fixed_sum adds for it
__device__ __forceinline__ long long fixed_units(float x, float scale) {
    const float y = x * scale;
    const float hi = floorf(y * 0x1p-24f);
    return ((long long)(unsigned)hi << 24) + (long long)(unsigned)(y - hi * 0x1p24f);
}
__device__ __forceinline__ void lane_zero(LaneSums& L, int lane) {
    L.drho[lane] = L.ke[lane] = L.tke[lane] = 0;
    L.cells[lane] = 0;
}
// The rare counters (NaN, negative, bad, rho range, rho finite, u limited)
// go straight to the step's integer accumulators.
__device__ __forceinline__ void lane_add(const StepArgs& A, LaneSums& L, int lane, const Acc& a, float& mx) {
    if (!a.cells) return;
    L.drho[lane] += __float2int_rn(a.drho * FX_DRHO);
    L.ke[lane] += fixed_units(a.ke, FX_KE);
    L.tke[lane] += fixed_units(a.tke, FX_TKE);
    L.cells[lane] += 1;
    if (a.nan | a.neg | a.bad | a.rout | a.rnf | a.ulim) {
        const int c[6] = {a.nan, a.neg, a.bad, a.rout, a.rnf, a.ulim};
        for (int j = 0; j < 6; ++j)
            if (c[j]) atomicAdd(&A.ctl->fx_cnt[j], (unsigned long long)c[j]);
    }
    mx = fmaxf(mx, a.maxu2);
}
__device__ __forceinline__ long long warp_allsum64(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// The warp's totals into the step's accumulators (finish_warp_sums).
__device__ __forceinline__ void finish_lane_sums(const StepArgs& A, const LaneSums& L, float mx, int lane,
                                                 unsigned int nwarps) {
    __syncwarp();
    WarpSums W;
    W.drho = warp_allsum64(L.drho[lane]);
    W.ke = warp_allsum64(L.ke[lane]);
    W.tke = warp_allsum64(L.tke[lane]);
#pragma unroll
    for (int j = 0; j < 6; ++j) W.cnt[j] = 0;
    W.cnt[6] = warp_allsum(L.cells[lane]);
    W.nu = W.tsum = W.nun = 0;
    finish_warp_sums<false>(A, W, mx, lane, nwarps);
}

// Shared-memory population slot of a tile cell, in register form.
template <class S>
__device__ __forceinline__ float lds_pop(const StepArgs& A, int q, const typename S::T* p) {
    if constexpr (S::shifted) return ld_shift<S>(A, q, S::raw_load(p));
    else return *p;
}

// Two-pass |S| (aeros/src/lbm.cpp:1012-1031) of tile cell t from the staged
// previous-step velocity rows: the expression tree of strain_prev.
template <int WT>
__device__ __forceinline__ float strain_rows(const float4* vel, int t) {
    constexpr int VX = WT + 32;
    const float4 xm = vel[t + 15], xp = vel[t + 17];
    const float4 ym = vel[VX + t], yp = vel[VX + WT + t];
    const float4 zm = vel[VX + 2 * WT + t], zp = vel[VX + 3 * WT + t];
    const float dux_dx = (xp.x - xm.x) * 0.5f;
    const float duy_dy = (yp.y - ym.y) * 0.5f;
    const float duz_dz = (zp.z - zm.z) * 0.5f;
    const float dux_dy = (yp.x - ym.x) * 0.5f;
    const float dux_dz = (zp.x - zm.x) * 0.5f;
    const float duy_dx = (xp.y - xm.y) * 0.5f;
    const float duy_dz = (zp.y - zm.y) * 0.5f;
    const float duz_dx = (xp.z - xm.z) * 0.5f;
    const float duz_dy = (yp.z - ym.z) * 0.5f;
    const float Sxx = dux_dx, Syy = duy_dy, Szz = duz_dz;
    const float Sxy = 0.5f * (dux_dy + duy_dx);
    const float Sxz = 0.5f * (dux_dz + duz_dx);
    const float Syz = 0.5f * (duy_dz + duz_dy);
    const float S2 = Sxx * Sxx + Syy * Syy + Szz * Szz + 2.0f * (Sxy * Sxy + Sxz * Sxz + Syz * Syz);
    return sqrtf(2.0f * S2);
}

// One interior cell of a warp tile (non-thermal). buf: the tile's buffer;
// t: the cell's position in the tile; strainPre: its previous-step |S|.
template <class S, bool ODD, bool FORCE>
__device__ __forceinline__ void warp_cell(const StepArgs& A, const StepVar& V, const StepOffsets& O, int cell,
                                          uint32_t d, unsigned char* buf, int t, float strainPre, Acc& acc) {
    using L = WarpLayout<S>;
    using T = typename S::T;
    constexpr bool SH = S::shifted;
    constexpr int ROW = ODD ? L::ROW_O : L::ROW_E;
    auto slot = [&](int q) -> T* {
        return reinterpret_cast<T*>(buf + q * ROW) + t + (ODD ? L::moff(q) : 0);
    };
    float f[Q19];
    if (!ODD || (d & D_LINKS) == 0) {
#pragma unroll
        for (int q = 0; q < Q19; ++q) f[q] = lds_pop<S>(A, q, slot(q));
    } else {
        // a link to a wall or out of the domain: the population comes back to
        // the cell's own slot (bounce-back), which is not in the row
#pragma unroll
        for (int q = 0; q < Q19; ++q)
            f[q] = ((d >> q) & 1u) ? ldp<S>(A, q, fplane<S>(A, q) + cell) : lds_pop<S>(A, q, slot(q));
    }
    CellResult r;
    collide19<SH, !FORCE>(f, A, d, false, false, strainPre, 0.0f, r, acc);
    const uint32_t os = (d >> D_OUT_SHIFT) & 3u;   // planes Nx-2 / Nx-3 feed the outlet
    if (os) {
        const uint32_t rr = A.div_x.div((uint32_t)cell);
        const int x = cell - (int)rr * A.nx;
        const uint32_t z = A.div_y.div(rr);
        const int y = (int)(rr - z * (uint32_t)A.ny);
        const int P = A.out_plane;
        const int pi = plane_index(A, x, y, (int)z);
#pragma unroll
        for (int q = 0; q < Q19; ++q) V.out_w[((int)(os - 1) * Q19 + q) * P + pi] = f[q];
    }
    if (!ODD) {
        // post_j goes to the slot (cell, opp j): row opp j, in place; read back
        // as opp j when c + c_j is a wall (the shift of the reader)
#pragma unroll
        for (int j = 0; j < Q19; ++j) {
            const int rd = (SH && ((d >> opp19(j)) & 1u)) ? opp19(j) : j;
            if constexpr (SH) S::raw_store(slot(opp19(j)), st_shift<S>(A, rd, f[j]));
            else *slot(opp19(j)) = f[j];
        }
    } else {
        char* pc = static_cast<char*>(A.f) + (long long)cell * (long long)sizeof(T);
        if ((d & D_LINKS) == 0) {
#pragma unroll
            for (int j = 0; j < Q19; ++j) stp<S>(A, j, reinterpret_cast<T*>(pc + O.soff[j]), f[j]);
        } else {
#pragma unroll
            for (int j = 0; j < Q19; ++j) {
                const bool solid = (d >> opp19(j)) & 1u;   // target c + c_j is a wall
                if (solid) stp<S>(A, opp19(j), fplane<S>(A, opp19(j)) + cell, f[j]);
                else stp<S>(A, j, reinterpret_cast<T*>(pc + O.soff[j]), f[j]);
            }
        }
    }
    if (V.write_u) V.uc[cell] = make_float4(r.ux, r.uy, r.uz, 0.0f);
    if (V.write_obs) { A.rho[cell] = r.rho; A.strain[cell] = r.strain; A.tke[cell] = r.tke; }
}

// Issues a tile's population and descriptor copies into buf: population
// chunks from the lane's offset table (bytes from A.f before the tile's own
// offset), then the descriptors.
template <class S, bool ODD>
__device__ __forceinline__ void warp_issue_pops(const StepArgs& A, int c0, uint32_t buf, const int* tab, int lane) {
    using L = WarpLayout<S>;
    constexpr int NCH = ODD ? L::NCH_O : L::NCH_E;
    constexpr int K = ODD ? L::K_O : L::K_E;
    const char* fb = static_cast<const char*>(A.f) + (long long)c0 * L::ESZ;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = lane + 32 * k;
        if (k < K - 1 || i < NCH) cp_async16(buf + (uint32_t)i * 16u, fb + tab[k * 32 + lane]);
    }
    if (lane < L::DESC / 16)
        cp_async16(buf + (uint32_t)(L::OFF_DESC + lane * 16), reinterpret_cast<const char*>(A.desc + c0) + lane * 16);
}
// ... and the tile's previous-step velocity rows into vbuf.
template <class S>
__device__ __forceinline__ void warp_issue_vel(const StepArgs& A, const StepVar& V, int c0, uint32_t vbuf, int lane) {
    using L = WarpLayout<S>;
    const float4* u = V.up + c0 + lane;
#pragma unroll
    for (int k = 0; k <= L::M; ++k) cp_async16(vbuf + (uint32_t)((lane + 32 * k) * 16), u - 16 + 32 * k);
    const int off[4] = {-A.nx, A.nx, -A.nxny, A.nxny};
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int k = 0; k < L::M; ++k)
            cp_async16(vbuf + (uint32_t)((L::VX + r * L::WT + lane + 32 * k) * 16), u + off[r] + 32 * k);
}

// One lattice step (non-thermal) in one launch: shell blocks as in
// k_lbm_fused, interior warps over warp tiles.
template <class S, bool ODD, bool FORCE>
__global__ void __launch_bounds__(STEP_BLOCK, WarpLayout<S>::MIN_BLOCKS) k_lbm_warp(const StepArgs A, const StepVar V, const StepOffsets O) {
    using L = WarpLayout<S>;
    using T = typename S::T;
    if (A.ctl->halt) return;   // uniform: every thread reads the same flag
    extern __shared__ __align__(128) unsigned char wsm[];
    const int lane = (int)(threadIdx.x & 31u), wid = (int)(threadIdx.x >> 5);
    unsigned char* ws = wsm + wid * L::WARP;
    LaneSums& sums = *reinterpret_cast<LaneSums*>(ws + L::OFF_SUMS);
    lane_zero(sums, lane);
    float mx = 0.0f;
    if ((int)blockIdx.x < A.shell_blocks) {
        const int nsh = A.ntiles - A.ntiles_interior;
        for (int st = blockIdx.x; st < nsh; st += A.shell_blocks) {
            Acc acc;
            acc.zero();
            shell_tile<S, ODD, false, false>(A, V, st, acc);
            lane_add(A, sums, lane, acc, mx);
        }
    } else {
        constexpr int NCH = ODD ? L::NCH_O : L::NCH_E;
        constexpr int CH = ODD ? L::CH_O : L::CH_E;
        constexpr int K = ODD ? L::K_O : L::K_E;
        int* tab = reinterpret_cast<int*>(ws + L::OFF_TAB);
        const float4* vel = reinterpret_cast<const float4*>(ws + L::OFF_VEL);
        // chunk i = lane + 32 k of a tile: row i / CH, chunk i % CH of the row
        for (int k = 0; k < K; ++k) {
            const int i = lane + 32 * k;
            long long e = 0;
            if (i < NCH) {
                const int q = i / CH, ch = i - q * CH;
                e = ODD ? (long long)opp19(q) * A.qstride - A.nbq[q] - L::moff(q) : (long long)q * A.qstride;
                e += (long long)ch * L::PAD;
            }
            tab[k * 32 + lane] = (int)(e * L::ESZ);
        }
        __syncwarp();
        const bool les = A.use_les != 0;
        const int ntiles = A.wt_last - A.wt_first + 1;
        const uint32_t b0 = smem_u32(ws), vb = b0 + (uint32_t)L::OFF_VEL;
        int cur = 0, nxt = 0;
        if (lane == 0) {
            cur = (int)atomicAdd(&A.ctl->tile_next, 1u);
            nxt = (int)atomicAdd(&A.ctl->tile_next, 1u);
        }
        cur = __shfl_sync(0xffffffffu, cur, 0);
        nxt = __shfl_sync(0xffffffffu, nxt, 0);
        if (cur < ntiles) warp_issue_pops<S, ODD>(A, (A.wt_first + cur) * L::WT, b0, tab, lane);
        cp_async_commit();
        if (les && cur < ntiles) warp_issue_vel<S>(A, V, (A.wt_first + cur) * L::WT, vb, lane);
        cp_async_commit();
        int b = 0;
        while (cur < ntiles) {
            const int cn = (A.wt_first + nxt) * L::WT;
            if (nxt < ntiles) warp_issue_pops<S, ODD>(A, cn, b0 + (uint32_t)((b ^ 1) * L::BUF), tab, lane);
            cp_async_commit();
            int nn = 0;   // the tile after next: its index arrives while this one is stepped
            if (lane == 0 && nxt < ntiles) nn = (int)atomicAdd(&A.ctl->tile_next, 1u);
            cp_async_wait<1>();   // this tile's rows (only the newest group may still be in flight)
            __syncwarp();
            unsigned char* buf = ws + b * L::BUF;
            const uint32_t* dsc = reinterpret_cast<const uint32_t*>(buf + L::OFF_DESC);
            const int c0 = (A.wt_first + cur) * L::WT;
            // the tile's strains first: the velocity rows are then free for the
            // next tile's, which arrive while this tile collides
            float sp[L::M];
            uint32_t own[L::M];   // even step: cells whose slots this warp writes back
#pragma unroll
            for (int m = 0; m < L::M; ++m) {
                const int t = lane + 32 * m;
                const uint32_t d = dsc[t];
                const bool in = c0 + t < A.ncell;
                sp[m] = (les && in && !(d & (D_WALL | D_SHELL)) && (d & D_LES)) ? strain_rows<L::WT>(vel, t) : 0.0f;
                own[m] = ODD ? 0u : __ballot_sync(0xffffffffu, in && !(d & D_SHELL));
            }
            __syncwarp();
            if (les && nxt < ntiles) warp_issue_vel<S>(A, V, cn, vb, lane);
            cp_async_commit();
#pragma unroll 1
            for (int m = 0; m < L::M; ++m) {
                const int t = lane + 32 * m;
                const int cell = c0 + t;
                const uint32_t d = dsc[t];
                float s = sp[0];
#pragma unroll
                for (int k = 1; k < L::M; ++k)
                    if (m == k) s = sp[k];
                Acc acc;
                acc.zero();
                if (cell < A.ncell && !(d & (D_WALL | D_SHELL))) warp_cell<S, ODD, FORCE>(A, V, O, cell, d, buf, t, s, acc);
                lane_add(A, sums, lane, acc, mx);
            }
            __syncwarp();
            if (!ODD) {
                // the rows back to their planes: whole 16-byte chunks where every
                // cell is the warp's, element by element where a shell cell is in
                char* fb = static_cast<char*>(A.f) + (long long)c0 * L::ESZ;
#pragma unroll
                for (int k = 0; k < L::K_E; ++k) {
                    const int i = lane + 32 * k;
                    if (k < L::K_E - 1 || i < L::NCH_E) {
                        const int e0 = (i % L::CH_E) * L::PAD;   // first cell of the chunk
                        uint32_t word = own[0];
#pragma unroll
                        for (int m = 1; m < L::M; ++m)
                            if ((e0 >> 5) == m) word = own[m];
                        const uint32_t bits = (word >> (e0 & 31)) & ((1u << L::PAD) - 1u);
                        char* g = fb + tab[k * 32 + lane];
                        const unsigned char* sp16 = buf + i * 16;
                        if (bits == (1u << L::PAD) - 1u) {
                            *reinterpret_cast<uint4*>(g) = *reinterpret_cast<const uint4*>(sp16);
                        } else if (bits) {
                            for (int e = 0; e < L::PAD; ++e)
                                if ((bits >> e) & 1u)
                                    reinterpret_cast<T*>(g)[e] = reinterpret_cast<const T*>(sp16)[e];
                        }
                    }
                }
                __syncwarp();
            }
            cur = nxt;
            nxt = __shfl_sync(0xffffffffu, nn, 0);
            if (cur >= ntiles) nxt = ntiles;
            b ^= 1;
        }
        cp_async_wait<0>();
    }
    finish_lane_sums(A, sums, mx, lane, gridDim.x * (STEP_BLOCK / 32));
}

// ---- many domains in one persistent kernel -----------------------------------
// Warps take work items from a global counter; an item is a run of 32-cell
// slices of one domain's shell or interior (shell items of every domain
// first). A warp sums each slice in FP32 (a fixed shuffle tree over a fixed
// set of 32 cells), converts the slice sums to 64-bit fixed point and adds
// them into the domain's accumulators with integer atomics. Integer addition
// is exact and associative, so a domain's statistics do not depend on the
// order of the slices: not on the schedule, the tuning or the other domains.
// The warp that finishes a domain's last slice of the step updates its control
// block. No block-wide barrier is involved.
struct BatchDomain {
    StepArgs A;                 // the domain's arguments (A.ctl: its control block)
    float4* u[2];               // velocity double buffer
    float* out[2];              // outlet side buffers
    int ubuf0, outpar0;         // buffer parities at the first step of the call
    int overrides0;             // overrides on at the first step of the call
    int les;                    // velocity written every step
    int nslices;                // shell + interior slices of 32 cells
    int pad[3];
};

struct BatchWork {
    int dom, kind, slice0, nslices;   // kind 0: shell slices, 1: interior slices
};

struct BatchAcc {               // per domain, zero between steps
    unsigned long long drho, ke, tke;   // fixed point, two's complement
    unsigned long long cnt[7];          // NaN, negative, bad, rho range, rho finite, u limited, cells
    unsigned int maxu2;                 // float bits (values >= 0 order as integers)
    unsigned int done;                  // slices finished this step
};

struct BatchCtl {
    unsigned int work_next[2];  // next work item of the shell / interior launch (reset by its last block)
    unsigned int warps_done[2]; // blocks of the launch that have finished
    int k;                      // step of the call being executed
    int k_last;                 // last step of the call (writes rho, |S|, TKE)
};

struct BatchArgs {
    const BatchDomain* doms;
    const BatchWork* work;      // shell items of every domain, then interior items
    int item_begin, item_end;   // this launch's items
    BatchAcc* acc;
    BatchCtl* ctl;
};

// KIND 0: the shell slices of every domain; KIND 1: the interior slices (one
// launch each per step, so each launch's code is only its own path).
template <class S, bool ODD, int KIND>
__global__ void __launch_bounds__(BATCH_BLOCK, AEROS_BATCH_MIN_BLOCKS) k_batch_step(const BatchArgs B) {
    // Blocks take items; warp w of the block takes slice w of every group of
    // eight, so a block covers 256 consecutive cells at a time (the rows the
    // velocity stencil shares stay in L1). The current domain's arguments are
    // copied to shared memory once per domain change. Each warp keeps its
    // fixed-point sums for the current domain and adds them (then its slice
    // count) to the domain's accumulators when the block moves to another
    // domain or runs out of items.
    __shared__ __align__(16) unsigned char s_args[sizeof(StepArgs)];
    __shared__ WarpSums s_sums[BATCH_BLOCK / 32];
    __shared__ float s_mx[BATCH_BLOCK / 32];
    __shared__ int s_ws[BATCH_BLOCK / 32];
    __shared__ int s_item[2];
    const int lane = (int)(threadIdx.x & 31u), wid = (int)(threadIdx.x >> 5);
    StepArgs& A = *reinterpret_cast<StepArgs*>(s_args);   // StepArgs is not trivially constructible
    WarpSums& W = s_sums[wid];
    const int k = B.ctl->k;
    const bool write_obs = k == B.ctl->k_last;
    if (lane == 0) {
        W.drho = W.ke = W.tke = 0;
        for (int j = 0; j < 7; ++j) W.cnt[j] = 0;
    }
    __syncwarp();
    float mx = 0.0f;
    int w_slices = 0;
    // The block's sums for `dom` into the domain's accumulators, by its
    // first warp: one fence per block instead of one per warp (the finisher
    // reads only the accumulators). Called by the whole block.
    auto flush = [&](int dom) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) {
            s_mx[wid] = mx;
            s_ws[wid] = w_slices;
        }
        __syncthreads();
        if (wid == 0) {
            WarpSums T = s_sums[0];
            float m = s_mx[0];
            int ns = s_ws[0];
            for (int w = 1; w < BATCH_BLOCK / 32; ++w) {
                T.drho += s_sums[w].drho; T.ke += s_sums[w].ke; T.tke += s_sums[w].tke;
                for (int j = 0; j < 7; ++j) T.cnt[j] += s_sums[w].cnt[j];
                m = fmaxf(m, s_mx[w]);
                ns += s_ws[w];
            }
            if (ns > 0) {
                BatchAcc* ac = B.acc + dom;
                if (lane == 0) atomicAdd(&ac->drho, (unsigned long long)T.drho);
                else if (lane == 1) atomicAdd(&ac->ke, (unsigned long long)T.ke);
                else if (lane == 2) atomicAdd(&ac->tke, (unsigned long long)T.tke);
                else if (lane >= 3 && lane < 10 && T.cnt[lane - 3]) atomicAdd(&ac->cnt[lane - 3], (unsigned long long)T.cnt[lane - 3]);
                else if (lane == 10 && m > 0.0f) atomicMax(&ac->maxu2, __float_as_uint(m));
                __threadfence();
                __syncwarp();
                int last = 0;
                if (lane == 0)
                    last = atomicAdd(&ac->done, (unsigned int)ns) + (unsigned int)ns == (unsigned int)B.doms[dom].nslices;
                if (__shfl_sync(0xffffffffu, last, 0) && lane == 0) {
                    __threadfence();
                    volatile BatchAcc* va = ac;
                    const double t[5] = {(double)(long long)va->drho / (double)FX_DRHO,
                                         (double)(long long)va->ke / (double)FX_KE,
                                         (double)(long long)va->tke / (double)FX_TKE, 0.0, 0.0};
                    const long long c[8] = {(long long)va->cnt[0], (long long)va->cnt[1], (long long)va->cnt[2],
                                            (long long)va->cnt[3], (long long)va->cnt[4], (long long)va->cnt[5], 0,
                                            (long long)va->cnt[6]};
                    apply_totals(A, t, __uint_as_float(va->maxu2), c);
                    va->drho = 0; va->ke = 0; va->tke = 0;
                    for (int j = 0; j < 7; ++j) va->cnt[j] = 0;
                    va->maxu2 = 0;
                    va->done = 0;
                }
            }
        }
        __syncthreads();
        if (lane == 0) {
            W.drho = W.ke = W.tke = 0;
            for (int j = 0; j < 7; ++j) W.cnt[j] = 0;
        }
        __syncwarp();
        mx = 0.0f;
        w_slices = 0;
    };
    int cur = -1, par = 0;
    for (;;) {
        if (threadIdx.x == 0) s_item[par] = B.item_begin + (int)atomicAdd(&B.ctl->work_next[KIND], 1u);
        __syncthreads();
        const int item = s_item[par];
        par ^= 1;
        const bool end = item >= B.item_end;
        const int dom = end ? -1 : B.work[item].dom;
        if (cur >= 0 && dom != cur) flush(cur);   // block-uniform
        if (end) break;
        const BatchWork wk = B.work[item];
        const BatchDomain& D = B.doms[dom];
        if (dom != cur) {
            __syncthreads();   // every warp is done with the previous arguments
            const int* src = reinterpret_cast<const int*>(&D.A);
            int* dst = reinterpret_cast<int*>(s_args);
            for (int i = threadIdx.x; i < (int)(sizeof(StepArgs) / 4); i += BATCH_BLOCK) dst[i] = src[i];
            __syncthreads();
            // The arguments are written as ints and read as StepArgs fields:
            // no load of a field may be kept from before the copy.
            asm volatile("" ::: "memory");
            cur = dom;
        }
        // a halted domain stays halted for the rest of the call (its flag is
        // only set by its own finisher, after its last slice of a step)
        if (*(volatile int*)&A.ctl->halt) continue;
        StepVar V;
        V.up = D.u[(D.ubuf0 ^ k) & 1];
        V.uc = D.u[(D.ubuf0 ^ k ^ 1) & 1];
        V.out_w = D.out[(D.outpar0 ^ k) & 1];
        V.out_r = D.out[(D.outpar0 ^ k ^ 1) & 1];
        V.apply_overrides = D.overrides0 || k > 0;
        V.write_obs = write_obs;
        V.write_u = D.les || write_obs;
        for (int base = 0; base < wk.nslices; base += BATCH_BLOCK / 32) {
            const int sl = base + wid;
            if (sl >= wk.nslices) break;   // warp-uniform
            Acc acc;
            acc.zero();
            const int idx = (wk.slice0 + sl) * 32 + lane;
            if (KIND == 0) shell_cell<S, ODD, false, false>(A, V, idx, acc);
            else interior_cell<S, ODD, false, false>(A, V, idx, acc);
            add_slice_sums<false>(W, acc, mx, lane);
            ++w_slices;
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&B.ctl->warps_done[KIND], 1u) == gridDim.x - 1) {   // counts blocks
            B.ctl->work_next[KIND] = 0;
            B.ctl->warps_done[KIND] = 0;
            if (KIND == 1) B.ctl->k = k + 1;
        }
    }
}

}  // namespace aeros
