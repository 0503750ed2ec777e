// post.cu — readback and post-processing on the device: world-unit velocity
// and pressure with the readback statistics (the end of stepLBMCPU,
// aeros/src/lbm.cpp:1602-1705), vorticity / Q / strain
// (computeLBMVorticityAndQ, lbm.cpp:2005-2093) and the trilinear samplers
// (lbm.cpp:1782-1969). Compiled with --fmad=false: every float operation
// rounds as the reference's, in the same order.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/aeros_lbm.h"
#include "handle.cuh"
#include "samplers.cuh"

using namespace aeros;

namespace {

constexpr int PB = 256;
constexpr float CS2 = 1.0f / 3.0f;   // lbm.cpp:121

__global__ void k_world_fields(int n, const uint32_t* desc, const float* rho, const float4* u, float scale, float rho0,
                               float* uxw, float* uyw, float* uzw, float* p, unsigned long long* pbad) {
    int bad = 0;
    for (int c = blockIdx.x * PB + threadIdx.x; c < n; c += gridDim.x * PB) {
        if (desc[c] & D_WALL) {   // body and ground cells
            uxw[c] = 0.0f; uyw[c] = 0.0f; uzw[c] = 0.0f;
            p[c] = 0.0f;
            continue;
        }
        const float4 v = u[c];
        float ux = v.x;
        if (!isfinite(ux)) ux = 0.0f;
        uxw[c] = ux * scale;
        uyw[c] = v.y * scale;
        uzw[c] = v.z * scale;
        float r = rho[c];
        if (!isfinite(r)) r = 1.0f;
        const float pLat = CS2 * (r - 1.0f);
        float pPhys = pLat * scale * scale * rho0;
        if (!isfinite(pPhys)) { ++bad; pPhys = 0.0f; }
        p[c] = pPhys;
    }
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(pbad, (unsigned long long)bad);
}

struct PostPartial {
    double sum;
    float pmin, pmax;
    int n, pad;
};

// Strided pressure min / max and the density residual (lbm.cpp:1663-1688):
// per-block partials, the last block combines them in block order.
__global__ void k_world_stats(int total, int stride, const float* p, const float* rho, const float* prev, int valid,
                              PostPartial* parts, unsigned int* counter, PostPartial* out) {
    const int ns = (total + stride - 1) / stride;
    float mn = 1e30f, mx = -1e30f;
    double sum = 0.0;
    int cnt = 0;
    for (int i = blockIdx.x * PB + threadIdx.x; i < ns; i += gridDim.x * PB) {
        const int c = i * stride;
        const float v = p[c];
        if (isfinite(v)) { mn = fminf(mn, v); mx = fmaxf(mx, v); }
        if (valid) {
            const float r = rho[c];
            if (isfinite(r)) {
                const float d = r - prev[c];
                sum += (double)d * (double)d;
                ++cnt;
            }
        }
    }
    __shared__ double s_sum[PB / 32];
    __shared__ float s_mn[PB / 32], s_mx[PB / 32];
    __shared__ int s_n[PB / 32];
    __shared__ bool last;
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { s_sum[wid] = sum; s_mn[wid] = mn; s_mx[wid] = mx; s_n[wid] = cnt; }
    __syncthreads();
    if (threadIdx.x == 0) {
        PostPartial q{0.0, 1e30f, -1e30f, 0, 0};
        for (int w = 0; w < PB / 32; ++w) {
            q.sum += s_sum[w];
            q.pmin = fminf(q.pmin, s_mn[w]);
            q.pmax = fmaxf(q.pmax, s_mx[w]);
            q.n += s_n[w];
        }
        parts[blockIdx.x] = q;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    PostPartial t{0.0, 1e30f, -1e30f, 0, 0};
    const volatile PostPartial* vp = parts;
    for (unsigned b = 0; b < gridDim.x; ++b) {
        t.sum += vp[b].sum;
        t.pmin = fminf(t.pmin, vp[b].pmin);
        t.pmax = fmaxf(t.pmax, vp[b].pmax);
        t.n += vp[b].n;
    }
    *out = t;
    *counter = 0;
}

__global__ void k_keep_rho(int n, const float* rho, float* prev) {
    for (int c = blockIdx.x * PB + threadIdx.x; c < n; c += gridDim.x * PB) {
        const float r = rho[c];
        prev[c] = isfinite(r) ? r : 1.0f;
    }
}

__global__ void k_vort_q(int nx, int ny, int nz, const uint32_t* desc, const float* uxW, const float* uyW,
                         const float* uzW, float invCsx, float invCsy, float invCsz, float* vort, float* qc,
                         float* strain) {
    const long long ni = (long long)(nx - 2) * (ny - 2) * (nz - 2);
    for (long long i = blockIdx.x * (long long)PB + threadIdx.x; i < ni; i += (long long)gridDim.x * PB) {
        const int x = (int)(i % (nx - 2)) + 1;
        const long long r = i / (nx - 2);
        const int y = (int)(r % (ny - 2)) + 1, z = (int)(r / (ny - 2)) + 1;
        const int cell = (z * ny + y) * nx + x;
        if (desc[cell] & D_WALL) { vort[cell] = 0.0f; qc[cell] = 0.0f; continue; }
        const int xm = cell - 1, xp = cell + 1, ym = cell - nx, yp = cell + nx, zm = cell - nx * ny, zp = cell + nx * ny;
        const float dux_dx = (uxW[xp] - uxW[xm]) * 0.5f * invCsx;
        const float dux_dy = (uxW[yp] - uxW[ym]) * 0.5f * invCsy;
        const float dux_dz = (uxW[zp] - uxW[zm]) * 0.5f * invCsz;
        const float duy_dx = (uyW[xp] - uyW[xm]) * 0.5f * invCsx;
        const float duy_dy = (uyW[yp] - uyW[ym]) * 0.5f * invCsy;
        const float duy_dz = (uyW[zp] - uyW[zm]) * 0.5f * invCsz;
        const float duz_dx = (uzW[xp] - uzW[xm]) * 0.5f * invCsx;
        const float duz_dy = (uzW[yp] - uzW[ym]) * 0.5f * invCsy;
        const float duz_dz = (uzW[zp] - uzW[zm]) * 0.5f * invCsz;
        if (!isfinite(dux_dx)) { vort[cell] = 0.0f; qc[cell] = 0.0f; continue; }
        const float wx = duz_dy - duy_dz;
        const float wy = dux_dz - duz_dx;
        const float wz = duy_dx - dux_dy;
        float vm = sqrtf(wx * wx + wy * wy + wz * wz);
        if (!isfinite(vm)) vm = 0.0f;
        if (vm > 1000.0f) vm = 1000.0f;
        vort[cell] = vm;
        const float Sxx = dux_dx, Syy = duy_dy, Szz = duz_dz;
        const float Sxy = 0.5f * (dux_dy + duy_dx);
        const float Sxz = 0.5f * (dux_dz + duz_dx);
        const float Syz = 0.5f * (duy_dz + duz_dy);
        const float Oxy = 0.5f * (dux_dy - duy_dx);
        const float Oxz = 0.5f * (dux_dz - duz_dx);
        const float Oyz = 0.5f * (duy_dz - duz_dy);
        const float S2 = Sxx * Sxx + Syy * Syy + Szz * Szz + 2.0f * (Sxy * Sxy + Sxz * Sxz + Syz * Syz);
        const float O2 = 2.0f * (Oxy * Oxy + Oxz * Oxz + Oyz * Oyz);
        float Q = 0.5f * (O2 - S2);
        if (!isfinite(Q)) Q = 0.0f;
        if (Q > 1e6f) Q = 1e6f;
        if (Q < -1e6f) Q = -1e6f;
        qc[cell] = Q;
        float st = sqrtf(2.0f * S2);
        if (!isfinite(st)) st = 0.0f;
        strain[cell] = st;
    }
}

struct SampleArgs {
    int nx, ny, nz;
    float minx, miny, minz, csx, csy, csz;
    const uint32_t* desc;
    const float4* u;      // velocity (lattice units)
    const float* field;   // scalar field, or NULL for the velocity / solid samplers
    int kind;             // AEROS_FIELD_*
};

__device__ __forceinline__ float clamp01(float t) { return fminf(fmaxf(t, 0.0f), 1.0f); }

__global__ void k_sample(const SampleArgs a, const float* pts, long long n, float* out, uint8_t* valid) {
    for (long long i = blockIdx.x * (long long)PB + threadIdx.x; i < n; i += (long long)gridDim.x * PB) {
        const float wx = pts[3 * i], wy = pts[3 * i + 1], wz = pts[3 * i + 2];
        uint8_t ok = 0;
        if (a.kind == AEROS_FIELD_VELOCITY_LB) {
            // getLBMVelocityLB, lbm.cpp:1782-1840
            float rx = 0.0f, ry = 0.0f, rz = 0.0f;
            if (isfinite(wx)) {
                const float fx = (wx - a.minx) / a.csx, fy = (wy - a.miny) / a.csy, fz = (wz - a.minz) / a.csz;
                const int ix = (int)floorf(fx), iy = (int)floorf(fy), iz = (int)floorf(fz);
                const float tx = clamp01(fx - (float)ix), ty = clamp01(fy - (float)iy), tz = clamp01(fz - (float)iz);
                if (!(ix < 0 || ix >= a.nx - 1 || iy < 0 || iy >= a.ny - 1 || iz < 0 || iz >= a.nz - 1)) {
                    const float w[8] = {(1 - tx) * (1 - ty) * (1 - tz), tx * (1 - ty) * (1 - tz), (1 - tx) * ty * (1 - tz),
                                        tx * ty * (1 - tz), (1 - tx) * (1 - ty) * tz, tx * (1 - ty) * tz,
                                        (1 - tx) * ty * tz, tx * ty * tz};
                    float vx[8], vy[8], vz[8], ws[8];
                    int cnt = 0;
                    float totalW = 0.0f;
                    for (int k = 0; k < 8; ++k) {
                        const int cx = ix + (k & 1), cy = iy + ((k >> 1) & 1), cz = iz + ((k >> 2) & 1);
                        const int cell = (cz * a.ny + cy) * a.nx + cx;
                        if (a.desc[cell] & D_WALL) continue;
                        const float4 v = a.u[cell];
                        if (!isfinite(v.x)) continue;
                        vx[cnt] = v.x; vy[cnt] = v.y; vz[cnt] = v.z; ws[cnt] = w[k];
                        totalW += w[k];
                        ++cnt;
                    }
                    if (cnt > 0) {
                        ok = 1;
                        if (totalW < 1e-6f) {
                            rx = vx[0]; ry = vy[0]; rz = vz[0];
                        } else {
                            for (int k = 0; k < cnt; ++k) {
                                const float s = ws[k] / totalW;
                                rx += vx[k] * s; ry += vy[k] * s; rz += vz[k] * s;
                            }
                            if (!isfinite(rx)) { rx = ry = rz = 0.0f; }
                        }
                    }
                }
            }
            out[3 * i] = rx; out[3 * i + 1] = ry; out[3 * i + 2] = rz;
        } else if (a.kind == AEROS_FIELD_SOLID) {
            // isLBMSolidWorld, lbm.cpp:1954-1969
            float r = 0.0f;
            if (isfinite(wx) && isfinite(wy) && isfinite(wz) && a.csx >= 1e-9f && a.csy >= 1e-9f && a.csz >= 1e-9f) {
                const float fx = (wx - a.minx) / a.csx, fy = (wy - a.miny) / a.csy, fz = (wz - a.minz) / a.csz;
                const int ix = (int)floorf(fx), iy = (int)floorf(fy), iz = (int)floorf(fz);
                if (!(ix < 0 || ix >= a.nx || iy < 0 || iy >= a.ny || iz < 0 || iz >= a.nz)) {
                    ok = 1;
                    r = (a.desc[(iz * a.ny + iy) * a.nx + ix] & D_WALL) ? 1.0f : 0.0f;
                }
            }
            out[i] = r;
        } else {
            // sampleFieldTrilinear(field, pos, skipSolid = true), lbm.cpp:1881-1933
            const smp::FieldView v{a.nx, a.ny, a.nz, {a.minx, a.miny, a.minz}, {a.csx, a.csy, a.csz}, a.desc};
            float r = 0.0f;
            ok = smp::field_trilinear(v, a.field, wx, wy, wz, &r) ? 1 : 0;
            out[i] = r;
        }
        if (valid) valid[i] = ok;
    }
}

int grid_for(long long n) {
    const long long b = (n + PB - 1) / PB;
    return (int)std::max<long long>(1, std::min<long long>(b, 4096));
}

int ensure_post(aeros_lbm* h) {
    if (h->uxw) return AEROS_OK;
    const size_t n = (size_t)h->ncell;
    float** bufs[6] = {&h->uxw, &h->uyw, &h->uzw, &h->pressure, &h->vort, &h->qcrit};
    for (float** b : bufs) {
        if (cudaMalloc((void**)b, n * 4) != cudaSuccess) return set_error(AEROS_ERR_ALLOC, "post-processing fields");
        CUDA_TRY(cudaMemsetAsync(*b, 0, n * 4, h->stream));
        h->dev_bytes += n * 4;
    }
    if (cudaMalloc((void**)&h->post_parts, 4096 * sizeof(PostPartial)) != cudaSuccess ||
        cudaMalloc((void**)&h->post_out, sizeof(PostPartial) + 16) != cudaSuccess ||
        cudaMalloc((void**)&h->post_counter, 16) != cudaSuccess)
        return set_error(AEROS_ERR_ALLOC, "post-processing scratch");
    CUDA_TRY(cudaMemsetAsync(h->post_counter, 0, 16, h->stream));
    return AEROS_OK;
}

int copy_out(aeros_lbm* h, float* dst, const float* src) {
    if (dst) CUDA_TRY(cudaMemcpyAsync(dst, src, (size_t)h->ncell * 4, cudaMemcpyDeviceToHost, h->stream));
    return AEROS_OK;
}

}  // namespace

extern "C" int aeros_lbm_world_fields(aeros_lbm* h, const aeros_world_params* wp, float* ux, float* uy, float* uz,
                                      float* pressure, aeros_world_stats* stats) {
    if (!h || !wp) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (int rc = finish_batch(h)) return rc;
    if (int rc = ensure_post(h)) return rc;
    // velocity scale, lbm.cpp:1603-1608
    const float iu0 = h->p.u_in[0], iu1 = h->p.u_in[1], iu2 = h->p.u_in[2];
    float U0mag2 = std::sqrt(iu0 * iu0 + iu1 * iu1 + iu2 * iu2);
    if (!std::isfinite(U0mag2) || U0mag2 < 1e-6f) U0mag2 = 0.08f;
    float scale = wp->flow_speed / U0mag2;
    if (!std::isfinite(scale) || scale > 1000.0f) scale = 20.0f;
    const int n = h->ncell;
    CUDA_TRY(cudaMemsetAsync(h->post_out, 0, sizeof(PostPartial) + 16, h->stream));
    unsigned long long* pbad = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(h->post_out) + sizeof(PostPartial));
    k_world_fields<<<grid_for(n), PB, 0, h->stream>>>(n, h->desc, h->rho, h->u[h->ubuf], scale, wp->air_density, h->uxw,
                                                       h->uyw, h->uzw, h->pressure, pbad);
    CUDA_TRY(cudaGetLastError());
    // statistics over at most 262,144 strided cells (lbm.cpp:1663-1690)
    int stride = 1;
    while (n / stride > 262144) stride *= 2;
    const long long step = h->ctl_host->steps;
    const bool valid = h->prev_rho != nullptr && h->post_prev_step >= 0 && step >= h->post_prev_step;
    if (!h->prev_rho) {
        if (cudaMalloc((void**)&h->prev_rho, (size_t)n * 4) != cudaSuccess)
            return set_error(AEROS_ERR_ALLOC, "previous density");
        h->dev_bytes += (uint64_t)n * 4;
        std::vector<float> ones((size_t)n, 1.0f);
        CUDA_TRY(cudaMemcpyAsync(h->prev_rho, ones.data(), (size_t)n * 4, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
    }
    const int ns = (n + stride - 1) / stride;
    PostPartial* parts = static_cast<PostPartial*>(h->post_parts);
    PostPartial* res = static_cast<PostPartial*>(h->post_out);
    k_world_stats<<<grid_for(ns), PB, 0, h->stream>>>(n, stride, h->pressure, h->rho, h->prev_rho, valid ? 1 : 0, parts,
                                                      h->post_counter, res);
    CUDA_TRY(cudaGetLastError());
    k_keep_rho<<<grid_for(n), PB, 0, h->stream>>>(n, h->rho, h->prev_rho);
    CUDA_TRY(cudaGetLastError());
    if (int rc = copy_out(h, ux, h->uxw)) return rc;
    if (int rc = copy_out(h, uy, h->uyw)) return rc;
    if (int rc = copy_out(h, uz, h->uzw)) return rc;
    if (int rc = copy_out(h, pressure, h->pressure)) return rc;
    unsigned char host[sizeof(PostPartial) + 16];
    CUDA_TRY(cudaMemcpyAsync(host, h->post_out, sizeof(host), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    PostPartial t;
    memcpy(&t, host, sizeof(t));
    unsigned long long bad = 0;
    memcpy(&bad, host + sizeof(PostPartial), sizeof(bad));
    const float maxu = h->ctl_host->max_u;
    if (stats) {
        stats->pressure_min = (t.pmin <= t.pmax && std::isfinite(t.pmin)) ? t.pmin : 0.0f;
        stats->pressure_max = (t.pmin <= t.pmax && std::isfinite(t.pmax)) ? t.pmax : 0.0f;
        stats->residual_rho = (valid && t.n > 0) ? (float)std::sqrt(t.sum / (double)t.n) : 0.0f;
        stats->residual_u = std::fabs(maxu - h->post_prev_maxu);
        stats->pressure_non_finite = (int64_t)bad;
    }
    h->post_prev_maxu = maxu;
    h->post_prev_step = step;
    h->post_min[0] = wp->min[0]; h->post_min[1] = wp->min[1]; h->post_min[2] = wp->min[2];
    h->post_cell[0] = wp->cell[0]; h->post_cell[1] = wp->cell[1]; h->post_cell[2] = wp->cell[2];
    return AEROS_OK;
}

extern "C" int aeros_lbm_vorticity_q(aeros_lbm* h, float* vorticity, float* q, float* strain) {
    if (!h) return set_error(AEROS_ERR_INVALID, "handle is NULL");
    if (int rc = finish_batch(h)) return rc;
    if (!h->uxw) return set_error(AEROS_ERR_STATE, "no world fields yet: call aeros_lbm_world_fields first");
    // cell sizes, lbm.cpp:2025-2030
    float csx = h->post_cell[0], csy = h->post_cell[1], csz = h->post_cell[2];
    if (csx < 1e-6f) csx = 0.1f;
    if (csy < 1e-6f) csy = 0.1f;
    if (csz < 1e-6f) csz = 0.1f;
    const float ix = 1.0f / csx, iy = 1.0f / csy, iz = 1.0f / csz;
    const long long ni = (long long)(h->nx - 2) * (h->ny - 2) * (h->nz - 2);
    k_vort_q<<<grid_for(ni), PB, 0, h->stream>>>(h->nx, h->ny, h->nz, h->desc, h->uxw, h->uyw, h->uzw, ix, iy, iz, h->vort,
                                                  h->qcrit, h->strain);
    CUDA_TRY(cudaGetLastError());
    if (int rc = copy_out(h, vorticity, h->vort)) return rc;
    if (int rc = copy_out(h, q, h->qcrit)) return rc;
    if (int rc = copy_out(h, strain, h->strain)) return rc;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return AEROS_OK;
}

extern "C" int aeros_lbm_sample(aeros_lbm* h, const aeros_world_params* wp, int field, const float* points, int64_t n,
                                float* out, uint8_t* valid) {
    if (!h || !wp || (n > 0 && (!points || !out))) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (n < 0 || n > (int64_t)1 << 28) return set_error(AEROS_ERR_INVALID, "%lld points", (long long)n);
    if (field < AEROS_FIELD_VELOCITY_LB || field > AEROS_FIELD_SOLID)
        return set_error(AEROS_ERR_INVALID, "unknown field %d", field);
    if (int rc = finish_batch(h)) return rc;
    if (n == 0) return AEROS_OK;
    SampleArgs a;
    a.nx = h->nx; a.ny = h->ny; a.nz = h->nz;
    a.minx = wp->min[0]; a.miny = wp->min[1]; a.minz = wp->min[2];
    a.csx = wp->cell[0]; a.csy = wp->cell[1]; a.csz = wp->cell[2];
    a.desc = h->desc;
    a.u = h->u[h->ubuf];
    a.kind = field;
    a.field = nullptr;
    if (field == AEROS_FIELD_DENSITY) a.field = h->rho;
    else if (field == AEROS_FIELD_STRAIN) a.field = h->strain;
    else if (field == AEROS_FIELD_TKE) a.field = h->tke;
    else if (field == AEROS_FIELD_PRESSURE || field == AEROS_FIELD_VORTICITY || field == AEROS_FIELD_Q) {
        if (!h->uxw) return set_error(AEROS_ERR_STATE, "no world fields yet: call aeros_lbm_world_fields first");
        a.field = field == AEROS_FIELD_PRESSURE ? h->pressure : (field == AEROS_FIELD_VORTICITY ? h->vort : h->qcrit);
    }
    const int per = field == AEROS_FIELD_VELOCITY_LB ? 3 : 1;
    float* dpts = nullptr;
    float* dout = nullptr;
    uint8_t* dval = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&dpts, (size_t)n * 12, h->stream);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dout, (size_t)n * per * 4, h->stream);
    if (e == cudaSuccess && valid) e = cudaMallocAsync((void**)&dval, (size_t)n, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dpts, points, (size_t)n * 12, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        k_sample<<<grid_for(n), PB, 0, h->stream>>>(a, dpts, n, dout, dval);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, (size_t)n * per * 4, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && valid) e = cudaMemcpyAsync(valid, dval, (size_t)n, cudaMemcpyDeviceToHost, h->stream);
    if (dpts) cudaFreeAsync(dpts, h->stream);
    if (dout) cudaFreeAsync(dout, h->stream);
    if (dval) cudaFreeAsync(dval, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return set_error(AEROS_ERR_CUDA, "sample: %s", cudaGetErrorString(e));
    return AEROS_OK;
}
