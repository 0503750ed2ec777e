// surface.cu — surface-pressure lift and drag (computeLiftDrag,
// aeros/src/forces.cpp:401-688, LBM branch) with the device doing the
// per-triangle pass.
//
// Per call, on the handle's stream:
//   k_surface_extent  leading / trailing edge: min and max of dot(v0, flowDir)
//                     over the triangles (ordered-key atomics, exact)
//   k_surface_tri     one thread per triangle: wall sample point
//                     (forces.cpp:75-90), trilinear pressure
//                     (lbm.cpp:1881-1933), Cp with Karman-Tsien, pressure
//                     force, skin friction, moment about the quarter chord,
//                     pressure weight; plus the projected area of
//                     computeLBMRefArea (lbm.cpp:2128-2139). FP32 in the
//                     reference's operation order (--fmad=false); the 15
//                     per-triangle terms are summed over the warp in FP32
//                     (a fixed xor tree over 32 triangles), then over the
//                     block's warps in FP64
//   k_surface_fold    the block partials summed in a fixed tree (16 lanes per
//                     term, each in block order, then the lanes in order):
//                     the result does not depend on scheduling
// then one small device-to-host copy, and the closing formulas on the host
// in FP32 as the reference's (forces.cpp:615-687).
//
// The reference sums the terms in FP32 in triangle order (in thread order
// under OpenMP); the tree here (FP32 over 32 triangles, FP64 above) differs
// from that order by the rounding of the reference's long FP32 running sums.
// The skin-friction power law calls CUDA's log10f / powf where the reference
// calls the host library's (a few units in the last place apart); every
// other operation is a correctly rounded FP32 operation, so the per-triangle
// Cp is the reference's bit for bit. (FP64 log10 / pow and FP64 per-thread
// sums kept the FP64 pipe 72 % busy on GB300 and took 68 us for 81,920
// triangles.)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "../../include/aeros_lbm.h"
#include "handle.cuh"
#include "samplers.cuh"

using namespace aeros;

struct aeros_surface_mesh {
    float* tri = nullptr;        // 9 floats per triangle
    float* nrm = nullptr;        // the first vertex's normal, 3 floats per triangle
    int64_t ntri = 0;
    char* scratch = nullptr;     // leading-edge keys | sums | block partials (sized at creation)
    unsigned char* host = nullptr;   // pinned copy of keys and sums
};

namespace {

constexpr int SB = 256;          // threads per block
constexpr int MAX_BLOCKS = 1024; // fixed cap: the reduction tree does not depend on the device
constexpr int NT = 15;           // per-triangle terms
constexpr int NS = 16;           // terms + the non-finite Cp count

enum { S_FX, S_FY, S_FZ, S_CX, S_CY, S_CZ, S_MX, S_MY, S_MZ, S_AREA, S_PRESS, S_FRONT, S_BASEA, S_BASEF, S_PROJ };

struct V3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ V3 operator*(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ V3 operator/(V3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
// glm: dot = (x x' + y y') + z z', length = sqrt(dot), cross component order
__host__ __device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ float length(V3 a) { return sqrtf(dot(a, a)); }
__host__ __device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
// glm::min / max / clamp comparison forms (NaN passes through as glm's)
__host__ __device__ __forceinline__ float gmax(float a, float b) { return (a < b) ? b : a; }
__host__ __device__ __forceinline__ float gmin(float a, float b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

// Order-preserving keys of floats (larger float, larger key); slot value 0
// means "no triangle", so the slots start from a memset.
__device__ __forceinline__ uint32_t fkey(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__host__ __device__ __forceinline__ float fkey_value(uint32_t k) {
    const uint32_t b = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

// min(1e9, min along) and max(-1e9, max along), as the reference's scan
// that starts from those bounds (forces.cpp:445-452); then the chord and the
// quarter-chord point (forces.cpp:453-461).
struct Chord {
    float min_al, chord;
    V3 ac;
};
__host__ __device__ inline Chord quarter_chord(uint32_t kmin_inv, uint32_t kmax, V3 fd, V3 ctr, float max_dim) {
    float mn = 1e9f, mx = -1e9f;
    if (kmin_inv) {
        const float v = fkey_value(~kmin_inv);
        if (v < mn) mn = v;
    }
    if (kmax) {
        const float v = fkey_value(kmax);
        if (v > mx) mx = v;
    }
    if (!isfinite(mn)) { mn = 0.0f; mx = max_dim; }
    float chord = mx - mn;
    if (chord < 1e-6f) chord = max_dim;
    const V3 perp = ctr - fd * dot(ctr, fd);
    Chord c;
    c.min_al = mn;
    c.chord = chord;
    c.ac = fd * (mn + chord * 0.25f) + perp;
    return c;
}

struct TriArgs {
    smp::FieldView fv;
    const float* pressure;
    smp::SdfView sdf;
    int has_sdf;
    float lbm_cell;
    V3 fd, adir, ctr;
    float vinf, mu, rho, q, mach, beta, max_dim;
    int comp;
    const float* tri;
    const float* nrm;
    long long ntri;
    const uint32_t* ext;   // [0] ~key(min), [1] key(max)
    double* part;          // gridDim.x * NS
    float* cp;             // optional, one per triangle
};

__global__ void __launch_bounds__(SB) k_surface_extent(const float* __restrict__ tri, long long ntri, V3 fd,
                                                       uint32_t* ext) {
    uint32_t kmin_inv = 0, kmax = 0;
    for (long long t = blockIdx.x * (long long)SB + threadIdx.x; t < ntri; t += (long long)gridDim.x * SB) {
        const float al = dot(mk(tri[9 * t], tri[9 * t + 1], tri[9 * t + 2]), fd);
        if (al == al) {   // NaN never compares below or above the bounds
            const uint32_t k = fkey(al);
            kmin_inv = max(kmin_inv, ~k);
            kmax = max(kmax, k);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        kmin_inv = max(kmin_inv, __shfl_xor_sync(0xffffffffu, kmin_inv, o));
        kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (kmin_inv) atomicMax(&ext[0], kmin_inv);
        if (kmax) atomicMax(&ext[1], kmax);
    }
}

// wallSamplePoint, forces.cpp:75-90
__device__ inline V3 wall_sample_point(const TriArgs& a, V3 p, V3 n) {
    const float nl = length(n);
    if (!(nl > 1e-6f) || !isfinite(nl)) return p;
    const V3 nn = n / nl;
    float cs = a.lbm_cell;
    if (!isfinite(cs) || cs <= 1e-9f) cs = 0.01f;
    const float off = 0.6f * cs;
    const V3 s = p + nn * off;
    if (a.has_sdf && smp::sdf_sample1(a.sdf, s.x, s.y, s.z) <= 0.0f) return p;
    return s;
}

__global__ void __launch_bounds__(SB) k_surface_tri(const TriArgs a) {
    __shared__ double red[SB / 32][NS];
    float acc[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) acc[k] = 0.0f;
    const Chord ch = quarter_chord(a.ext[0], a.ext[1], a.fd, a.ctr, a.max_dim);
    for (long long t = blockIdx.x * (long long)SB + threadIdx.x; t < a.ntri; t += (long long)gridDim.x * SB) {
        const float* p = a.tri + 9 * t;
        const V3 v0 = mk(p[0], p[1], p[2]), v1 = mk(p[3], p[4], p[5]), v2 = mk(p[6], p[7], p[8]);
        // computeLBMRefArea's projected area, lbm.cpp:2128-2139
        {
            const V3 cr = cross(v1 - v0, v2 - v0);
            const float area = 0.5f * length(cr);
            if (isfinite(area) && !(area < 1e-12f)) {
                const V3 n = cr * (1.0f / sqrtf(dot(cr, cr)));
                acc[S_PROJ] += area * fabsf(dot(n, a.adir));
            }
        }
        // computeTri, forces.cpp:486-582
        float cp = 0.0f;
        V3 n = mk(a.nrm[3 * t], a.nrm[3 * t + 1], a.nrm[3 * t + 2]);
        const float nl = length(n);
        if (isfinite(v0.x) && isfinite(n.x) && !(nl < 1e-6f || !isfinite(nl))) {
            n = n / nl;
            const V3 tc = ((v0 + v1) + v2) * (1.0f / 3.0f);
            const float area = 0.5f * length(cross(v1 - v0, v2 - v0));
            if (!(!isfinite(area) || area < 1e-9f || area > 1e6f)) {
                const V3 ps = wall_sample_point(a, tc, n);
                float pres = 0.0f;
                if (!smp::field_trilinear(a.fv, a.pressure, ps.x, ps.y, ps.z, &pres)) pres = 0.0f;
                cp = pres / a.q;
                if (a.comp) {
                    const float den = a.beta + (a.mach * a.mach / (1.0f + a.beta)) * cp * 0.5f;
                    if (fabsf(den) > 1e-6f) cp = cp / den;
                    else cp /= a.beta;
                }
                if (!isfinite(cp)) {
                    acc[NT] += 1.0f;
                    cp = 0.0f;
                }
                const V3 pf = n * (-cp * a.q) * area;
                const float fdn = dot(a.fd, n);
                acc[S_FRONT] += area * fabsf(fdn);
                if (fdn > 0.7f) {
                    acc[S_BASEA] += area;
                    acc[S_BASEF] += cp * a.q * area;
                }
                float xa = dot(tc, a.fd) - ch.min_al;
                if (xa < 0.001f) xa = 0.001f;
                if (xa > ch.chord * 1.5f) xa = ch.chord * 1.5f;
                float re = a.rho * a.vinf * xa / a.mu;
                re = gclamp(re, 1.0f, 1e9f);
                float cf;
                if (re < 5e5f) {
                    cf = 0.664f / sqrtf(re);
                } else {
                    float lr = log10f(re);
                    if (lr < 1.0f) lr = 1.0f;
                    cf = 0.455f / powf(lr, 2.58f);
                    if (re < 1e9f) {
                        cf -= 1700.0f / re;
                        if (cf < 0.0005f) cf = 0.0005f;
                    }
                }
                cf *= 1.12f;
                cf = gclamp(cf, 0.0002f, 0.015f);
                float ff = 1.0f - fabsf(fdn);
                if (fdn > 0) ff *= 0.55f;
                const float skin = cf * a.q * area * ff;
                const V3 force = pf + mk(-a.fd.x, -a.fd.y, -a.fd.z) * skin;
                float pw = fabsf(cp) * area;
                if (cp < 0) pw *= 0.8f;
                const V3 cw = tc * pw;
                const V3 m = cross(tc - ch.ac, force);
                acc[S_FX] += force.x; acc[S_FY] += force.y; acc[S_FZ] += force.z;
                acc[S_CX] += cw.x; acc[S_CY] += cw.y; acc[S_CZ] += cw.z;
                acc[S_MX] += m.x; acc[S_MY] += m.y; acc[S_MZ] += m.z;
                acc[S_AREA] += area;
                acc[S_PRESS] += pw;
            }
        }
        if (a.cp) a.cp[t] = cp;
    }
    // block sum: xor tree in each warp (FP32: 32 triangles), then the warps
    // in order in FP64
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        float v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = (double)v;
    }
    __syncthreads();
    if (threadIdx.x < NS) {
        double s = 0.0;
        for (int w = 0; w < SB / 32; ++w) s += red[w][threadIdx.x];
        a.part[(long long)blockIdx.x * NS + threadIdx.x] = s;
    }
}

// FOLD_LANES threads per term, each summing the partials of blocks
// j, j + FOLD_LANES, ... in order, then the lanes' sums in lane order: a
// fixed tree whose dependent chains are FOLD_LANES times shorter than a
// single running sum.
constexpr int FOLD_LANES = 16;
__global__ void __launch_bounds__(NS * FOLD_LANES) k_surface_fold(const double* __restrict__ part, int nblk,
                                                                  double* out) {
    __shared__ double lane_sum[FOLD_LANES][NS];
    const int k = threadIdx.x % NS, j = threadIdx.x / NS;
    double s = 0.0;
    for (int b = j; b < nblk; b += FOLD_LANES) s += part[(long long)b * NS + k];
    lane_sum[j][k] = s;
    __syncthreads();
    if (threadIdx.x < NS) {
        double t = 0.0;
        for (int l = 0; l < FOLD_LANES; ++l) t += lane_sum[l][threadIdx.x];
        out[threadIdx.x] = t;
    }
}

constexpr size_t RES_OFF = 16;                              // after the two keys (padded)
constexpr size_t PART_OFF = RES_OFF + NS * sizeof(double);  // then the block partials
constexpr size_t HOST_BYTES = PART_OFF;                     // what comes back per call

int blocks_for(int64_t ntri) { return (int)std::min<long long>(MAX_BLOCKS, (ntri + SB - 1) / SB); }

// computeLBMRefArea's direction (lbm.cpp:2114-2121), on the host with the
// host's cosf / sinf as the reference's
V3 angle_dir(float az_deg, float el_deg) {
    const float az = az_deg * 0.01745329251994329576923690768489f;
    const float el = el_deg * 0.01745329251994329576923690768489f;
    const float ce = cosf(el), se = sinf(el), ca = cosf(az), sa = sinf(az);
    V3 d = mk(ce * ca, se, ce * sa);
    const float l = length(d);
    if (l > 1e-6f) d = d / l;
    else d = mk(1.0f, 0.0f, 0.0f);
    return d;
}

// computeLBMRefArea's bounding-box fallback (lbm.cpp:2146-2156)
float bbox_area(const aeros_surface_params* sp, V3 fd) {
    float sy = sp->bb_max[1] - sp->bb_min[1], sz = sp->bb_max[2] - sp->bb_min[2], sx = sp->bb_max[0] - sp->bb_min[0];
    if (!std::isfinite(sy) || sy < 0.01f) sy = sp->max_dim;
    if (!std::isfinite(sz) || sz < 0.01f) sz = sp->max_dim;
    if (!std::isfinite(sx) || sx < 0.01f) sx = sp->max_dim;
    float a = (fabsf(fd.x) * sy * sz + fabsf(fd.y) * sx * sz + fabsf(fd.z) * sx * sy);
    if (!std::isfinite(a) || a < 1e-6f) a = sp->max_dim * sp->max_dim * 0.5f;
    return a;
}

// the closing formulas of computeLiftDrag, forces.cpp:615-687
void close_forces(const aeros_surface_params* sp, const float* tot, float q, V3 fd, V3 adir, float mach, V3 ac,
                  aeros_surface_forces* out) {
    float ref_global = sp->ref_area;
    if (sp->auto_ref_area) {   // aeroRefArea = computeLBMRefArea() (lbm.cpp:2140-2145)
        const float fr = tot[S_PROJ] * 0.5f;
        ref_global = (std::isfinite(fr) && fr > 1e-6f && fr < 1e6f) ? fr : bbox_area(sp, adir);
    }
    float ref = ref_global;
    if (!std::isfinite(ref) || ref < 1e-6f) ref = 1.0f;
    ref = gclamp(ref, 1e-6f, 1e6f);

    V3 F = mk(tot[S_FX], tot[S_FY], tot[S_FZ]);
    if (!std::isfinite(F.x)) F = mk(0.0f, 0.0f, 0.0f);
    if (sp->auto_ref_area && tot[S_FRONT] > 1e-6f) {
        const float fr = tot[S_FRONT] * 0.5f;
        if (fr > 1e-6f) ref_global = fr;
    }
    float base = 0.0f;
    if (tot[S_BASEA] > 1e-6f) {
        const float avg = tot[S_BASEF] / (q * tot[S_BASEA] + 1e-9f);
        if (avg > -0.05f) {   // an open base: the empirical base pressure
            float cpb = -0.14f;
            if (sp->reynolds > 1e6f) cpb = -0.12f;
            base = -cpb * q * tot[S_BASEA] * 0.6f;
        }
    }
    float drag = dot(F, fd) + base;
    if (!std::isfinite(drag)) drag = base;
    V3 up = mk(0.0f, 1.0f, 0.0f);
    V3 ldir = up - fd * dot(up, fd);
    float ldl = length(ldir);
    if (ldl < 1e-6f || !std::isfinite(ldl)) {
        up = mk(0.0f, 0.0f, 1.0f);
        ldir = up - fd * dot(up, fd);
        ldl = length(ldir);
    }
    float lift;
    V3 lvec;
    if (ldl < 1e-6f || !std::isfinite(ldl)) {
        lift = 0.0f;
        lvec = mk(0.0f, 0.0f, 0.0f);
    } else {
        ldir = ldir / ldl;
        lift = dot(F, ldir);
        if (!std::isfinite(lift)) lift = 0.0f;
        if (sp->ground_effect) {
            const float gy = sp->vox_min_y + sp->ground_height;
            const float h = sp->center[1] - gy;
            if (h > 0.01f && h < sp->max_dim * 1.0f) {
                const float ge = 1.0f + 0.35f * expf(-h / (sp->max_dim * 0.3f));
                if (lift < 0) lift *= ge;
            }
        }
        lvec = ldir * lift;
        if (!std::isfinite(lvec.x)) lvec = mk(0.0f, 0.0f, 0.0f);
    }
    float ar = 1.0f;
    const float span = sp->bb_max[2] - sp->bb_min[2];
    const float chest = sp->bb_max[0] - sp->bb_min[0];
    if (span > 1e-6f && ref > 1e-6f) ar = (span * span) / ref;
    else if (span > 1e-6f && chest > 1e-6f) ar = span / chest;
    ar = gclamp(ar, 0.3f, 20.0f);
    float eo = 0.8f;
    if (ar < 1.5f) eo = 0.65f;
    float cl = lift / (q * ref + 1e-9f);
    cl = gclamp(cl, -3.0f, 3.0f);
    const float cdi = cl * cl / (3.14159265f * ar * eo + 1e-6f);
    const float induced = cdi * q * ref;
    if (fabsf(cl) > 0.05f) drag += induced;
    if (sp->mach_effects && mach > 0.7f) {
        float cw = 0.0f;
        if (mach < 0.9f) cw = 20.0f * powf(mach - 0.7f, 4.0f);
        else cw = 0.1f + 0.2f * (mach - 0.9f);
        cw = gclamp(cw, 0.0f, 0.5f);
        drag += cw * q * ref;
    }
    V3 dvec = fd * drag;
    if (!std::isfinite(dvec.x)) dvec = mk(0.0f, 0.0f, 0.0f);
    const float l2d = fabsf(drag) > 1e-9f ? lift / drag : 0.0f;
    V3 mom = mk(tot[S_MX], tot[S_MY], tot[S_MZ]);
    float mm = length(mom);
    if (!std::isfinite(mm)) {
        mm = 0.0f;
        mom = mk(0.0f, 0.0f, 0.0f);
    }
    const V3 cps = mk(tot[S_CX], tot[S_CY], tot[S_CZ]);
    V3 cop;
    if (tot[S_PRESS] > 1e-9f && std::isfinite(cps.x)) cop = cps / tot[S_PRESS];
    else if (tot[S_AREA] > 1e-9f) cop = cps / tot[S_AREA];
    else cop = ac;
    if (!std::isfinite(cop.x)) cop = ac;

    out->status = AEROS_SURFACE_DONE;
    out->drag = drag;
    out->lift = lift;
    out->lift_to_drag = l2d;
    out->moment_magnitude = mm;
    const V3* vs[4] = {&dvec, &lvec, &mom, &cop};
    float* ds[4] = {out->drag_vector, out->lift_vector, out->moment, out->center_of_pressure};
    for (int i = 0; i < 4; ++i) {
        ds[i][0] = vs[i]->x;
        ds[i][1] = vs[i]->y;
        ds[i][2] = vs[i]->z;
    }
    out->ref_area = ref_global;
    out->ref_area_used = ref;
}

}  // namespace

extern "C" int aeros_surface_mesh_create(const float* vertices, const float* normals, int64_t ntri,
                                         aeros_surface_mesh** out) {
    if (!out || (ntri > 0 && (!vertices || !normals))) return set_error(AEROS_ERR_INVALID, "NULL argument");
    *out = nullptr;
    if (ntri < 0 || ntri > ((int64_t)1 << 27)) return set_error(AEROS_ERR_INVALID, "%lld triangles", (long long)ntri);
    aeros_surface_mesh* m = new (std::nothrow) aeros_surface_mesh();
    if (!m) return set_error(AEROS_ERR_ALLOC, "mesh");
    m->ntri = ntri;
    if (ntri == 0) {   // no triangles: the pass returns before writing, as the reference without a model
        *out = m;
        return AEROS_OK;
    }
    float* first = new (std::nothrow) float[(size_t)ntri * 3];
    cudaError_t e = first ? cudaSuccess : cudaErrorMemoryAllocation;
    if (first)
        for (int64_t t = 0; t < ntri; ++t) std::memcpy(first + 3 * t, normals + 9 * t, 12);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->tri, (size_t)ntri * 36);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->nrm, (size_t)ntri * 12);
    if (e == cudaSuccess) e = cudaMalloc((void**)&m->scratch, PART_OFF + (size_t)blocks_for(ntri) * NS * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&m->host, HOST_BYTES);
    if (e == cudaSuccess) e = cudaMemcpy(m->tri, vertices, (size_t)ntri * 36, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(m->nrm, first, (size_t)ntri * 12, cudaMemcpyHostToDevice);
    delete[] first;
    if (e != cudaSuccess) {
        aeros_surface_mesh_destroy(m);
        return set_error(AEROS_ERR_ALLOC, "surface mesh: %s", cudaGetErrorString(e));
    }
    *out = m;
    return AEROS_OK;
}

extern "C" int aeros_surface_mesh_destroy(aeros_surface_mesh* mesh) {
    if (!mesh) return AEROS_OK;
    if (mesh->tri) cudaFree(mesh->tri);
    if (mesh->nrm) cudaFree(mesh->nrm);
    if (mesh->scratch) cudaFree(mesh->scratch);
    if (mesh->host) cudaFreeHost(mesh->host);
    delete mesh;
    return AEROS_OK;
}

extern "C" int aeros_lbm_surface_forces(aeros_lbm* h, const aeros_world_params* wp, const aeros_surface_params* sp,
                                        const aeros_surface_mesh* mesh, const float* d_sdf,
                                        const aeros_voxel_grid* sdf_grid, aeros_surface_forces* out, float* cp) {
    if (!h || !wp || !sp || !mesh || !out) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if ((d_sdf == nullptr) != (sdf_grid == nullptr))
        return set_error(AEROS_ERR_INVALID, "distance field and its grid go together");
    if (sdf_grid && (sdf_grid->nx <= 0 || sdf_grid->ny <= 0 || sdf_grid->nz <= 0))
        return set_error(AEROS_ERR_INVALID, "distance-field grid %dx%dx%d", sdf_grid->nx, sdf_grid->ny, sdf_grid->nz);
    std::memset(out, 0, sizeof(*out));
    const int64_t ntri = mesh->ntri;
    if (cp)
        for (int64_t t = 0; t < ntri; ++t) cp[t] = 0.0f;
    out->status = AEROS_SURFACE_NOT_RUN;
    out->ref_area = sp->ref_area;   // aeroRefArea stays as it was on the early returns
    if (ntri <= 0) return AEROS_OK;
    if (int rc = finish_batch(h)) return rc;
    if (!h->uxw) return set_error(AEROS_ERR_STATE, "no world fields yet: call aeros_lbm_world_fields first");

    // scalar set-up, forces.cpp:408-474
    const V3 vel = mk(sp->velocity[0], sp->velocity[1], sp->velocity[2]);
    float vinf = sqrtf(vel.x * vel.x + vel.y * vel.y + vel.z * vel.z);
    if (!std::isfinite(vinf) || vinf < 1e-4f) vinf = 1e-4f;
    const float fdl = length(vel);
    if (fdl < 1e-6f || !std::isfinite(fdl)) {
        out->status = AEROS_SURFACE_NO_FLOW;
        return AEROS_OK;
    }
    TriArgs a;
    a.fd = vel / fdl;
    const float T = sp->air_temperature;
    const float T0s = 273.15f, S = 110.4f, mu0 = 1.716e-5f;   // Sutherland
    float mu = mu0 * powf(T / T0s, 1.5f) * (T0s + S) / (T + S);
    if (!std::isfinite(mu) || mu < 1e-6f) mu = 1.81e-5f;
    float rho = sp->use_real_density ? sp->air_density : 1.225f;
    rho = gclamp(rho, 0.0001f, 10.0f);
    float q = 0.5f * rho * vinf * vinf;
    if (q < 1e-9f) q = 1e-6f;
    const float mach = vinf / (sp->speed_of_sound + 1e-6f);
    a.comp = sp->mach_effects && mach > 0.3f && mach < 0.85f;
    a.beta = a.comp ? gmax(0.2f, sqrtf(1.0f - mach * mach)) : 1.0f;
    a.vinf = vinf;
    a.mu = mu;
    a.rho = rho;
    a.q = q;
    a.mach = mach;
    a.adir = angle_dir(sp->flow_azimuth_deg, sp->flow_elevation_deg);
    a.ctr = mk(sp->center[0], sp->center[1], sp->center[2]);
    a.max_dim = sp->max_dim;
    a.fv = smp::FieldView{h->nx, h->ny, h->nz, {wp->min[0], wp->min[1], wp->min[2]},
                          {wp->cell[0], wp->cell[1], wp->cell[2]}, h->desc};
    a.pressure = h->pressure;
    a.has_sdf = d_sdf != nullptr;
    a.sdf = smp::SdfView{};
    if (d_sdf) {
        a.sdf.d = d_sdf;
        a.sdf.nx = sdf_grid->nx; a.sdf.ny = sdf_grid->ny; a.sdf.nz = sdf_grid->nz;
        for (int i = 0; i < 3; ++i) {
            a.sdf.min[i] = sdf_grid->min[i];
            a.sdf.cs[i] = sdf_grid->cell[i];
        }
    }
    a.lbm_cell = wp->cell[0];
    a.tri = mesh->tri;
    a.nrm = mesh->nrm;
    a.ntri = ntri;

    const int nblk = blocks_for(ntri);
    char* scratch = mesh->scratch;   // the mesh's own: one pass per mesh at a time
    float* dcp = nullptr;
    cudaError_t e = cudaSuccess;
    if (cp) e = cudaMallocAsync((void**)&dcp, (size_t)ntri * 4, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, 8, h->stream);
    if (e == cudaSuccess) {
        a.ext = reinterpret_cast<uint32_t*>(scratch);
        a.part = reinterpret_cast<double*>(scratch + PART_OFF);
        a.cp = dcp;
        k_surface_extent<<<nblk, SB, 0, h->stream>>>(a.tri, ntri, a.fd, reinterpret_cast<uint32_t*>(scratch));
        k_surface_tri<<<nblk, SB, 0, h->stream>>>(a);
        k_surface_fold<<<1, NS * FOLD_LANES, 0, h->stream>>>(a.part, nblk, reinterpret_cast<double*>(scratch + RES_OFF));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(mesh->host, scratch, HOST_BYTES, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && cp) e = cudaMemcpyAsync(cp, dcp, (size_t)ntri * 4, cudaMemcpyDeviceToHost, h->stream);
    if (dcp) cudaFreeAsync(dcp, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return set_error(AEROS_ERR_CUDA, "surface forces: %s", cudaGetErrorString(e));

    uint32_t ext[2];
    double sums[NS];
    std::memcpy(ext, mesh->host, 8);
    std::memcpy(sums, mesh->host + RES_OFF, sizeof(sums));
    float tot[NT];
    for (int k = 0; k < NT; ++k) {
        out->sums[k] = sums[k];
        tot[k] = (float)sums[k];
    }
    out->cp_non_finite = (int64_t)sums[NT];
    const Chord ch = quarter_chord(ext[0], ext[1], a.fd, a.ctr, a.max_dim);
    close_forces(sp, tot, q, a.fd, a.adir, mach, ch.ac, out);
    return AEROS_OK;
}
