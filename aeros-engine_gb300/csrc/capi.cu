// capi.cu — the C ABI (include/aeros_lbm.h): solver handles, device memory,
// launches, and the record/consume error convention of the reference CUDA
// layer (aeros/src/kernel.cu:57-82).
//
// Host arithmetic that must match the reference bit for bit (inlet
// equilibrium, thermal parameters, conduction seed) is compiled with
// -ffp-contract=off.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/aeros_lbm.h"
#include "forces.cuh"
#include "handle.cuh"
#include "lbm_aux.cuh"
#include "setup.cuh"

using namespace aeros;

// ---------------------------------------------------------------------------
// error record (thread-local), consumed by aeros_consume_error
// ---------------------------------------------------------------------------
static thread_local int g_err_code = 0;
static thread_local char g_err_msg[1024] = {0};

int set_error(int code, const char* fmt, ...) {
    g_err_code = code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err_msg, sizeof(g_err_msg), fmt, ap);
    va_end(ap);
    return code;
}


extern "C" int aeros_consume_error(char* buf, int buf_size) {
    if (g_err_code == 0) {
        if (buf && buf_size > 0) buf[0] = 0;
        return 0;
    }
    if (buf && buf_size > 0) snprintf(buf, (size_t)buf_size, "%s", g_err_msg);
    const int c = g_err_code;
    g_err_code = 0;
    g_err_msg[0] = 0;
    return c;
}

template <class T>
static int dalloc(aeros_lbm* h, T** p, size_t bytes) {
    cudaError_t e = cudaMalloc((void**)p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        *p = nullptr;
        return set_error(AEROS_ERR_ALLOC, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    h->dev_bytes += bytes;
    return AEROS_OK;
}

static void free_handle(aeros_lbm* h) {
    if (!h) return;
    cudaFree(h->f);
    cudaFree(h->desc);
    cudaFree(h->shell);
    cudaFree(h->shell_kind);
    cudaFree(h->shell_gth);
    cudaFree(h->shell_sct);
    cudaFree(h->zg_src);
    for (float* b : {h->uxw, h->uyw, h->uzw, h->pressure, h->vort, h->qcrit, h->prev_rho, h->u_split}) cudaFree(b);
    cudaFree(h->post_parts);
    cudaFree(h->post_out);
    cudaFree(h->post_counter);
    cudaFree(h->u_alloc[0]);
    cudaFree(h->u_alloc[1]);
    cudaFree(h->rho);
    cudaFree(h->strain);
    cudaFree(h->tke);
    cudaFree(h->out[0]);
    cudaFree(h->out[1]);
    cudaFree(h->g);
    cudaFree(h->T);
    cudaFree(h->T_buoy);
    cudaFree(h->partials);
    cudaFree(h->ctl);
    cudaFree(h->force_partials);
    cudaFree(h->force_out);
    cudaFree(h->force_counter);
    cudaFree(h->area_count);
    if (h->ctl_host) cudaFreeHost(h->ctl_host);
    if (h->force_host) cudaFreeHost(h->force_host);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    delete h;
}

static inline int cidx(const aeros_lbm* h, int x, int y, int z) { return (z * h->ny + y) * h->nx + x; }

// Full-range wall distance (the reference's two-pass chamfer, lbm.cpp:647-675),
// built on the host only when a caller reads it back.
static void host_wall_distance(aeros_lbm* h) {
    const int nx = h->nx, ny = h->ny, nz = h->nz, n = h->ncell;
    const auto& m = h->mask;
    auto& wd = h->wall;
    wd.assign(n, 255);
    for (int c = 0; c < n; ++c)
        if (m[c]) wd[c] = 0;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            const int row = (z * ny + y) * nx;
            for (int x = 0; x < nx; ++x) {
                int v = wd[row + x];
                if (v == 0) continue;
                if (x > 0 && wd[row + x - 1] + 1 < v) v = wd[row + x - 1] + 1;
                if (y > 0 && wd[row - nx + x] + 1 < v) v = wd[row - nx + x] + 1;
                if (z > 0 && wd[row - nx * ny + x] + 1 < v) v = wd[row - nx * ny + x] + 1;
                wd[row + x] = (uint8_t)v;
            }
        }
    for (int z = nz - 1; z >= 0; --z)
        for (int y = ny - 1; y >= 0; --y) {
            const int row = (z * ny + y) * nx;
            for (int x = nx - 1; x >= 0; --x) {
                int v = wd[row + x];
                if (v == 0) continue;
                if (x < nx - 1 && wd[row + x + 1] + 1 < v) v = wd[row + x + 1] + 1;
                if (y < ny - 1 && wd[row + nx + x] + 1 < v) v = wd[row + nx + x] + 1;
                if (z < nz - 1 && wd[row + nx * ny + x] + 1 < v) v = wd[row + nx * ny + x] + 1;
                wd[row + x] = (uint8_t)v;
            }
        }
}

// Shell cells (any coordinate on the domain boundary) in increasing cell
// order, fluid-cell count (sFluidCells, lbm.cpp:677-680).
static void host_geometry(aeros_lbm* h, std::vector<int>& shell) {
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    shell.clear();
    shell.reserve((size_t)2 * (nx * ny + ny * nz + nx * nz));
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            const int row = (z * ny + y) * nx;
            if (z == 0 || z == nz - 1 || y == 0 || y == ny - 1) {
                for (int x = 0; x < nx; ++x) shell.push_back(row + x);
            } else {
                shell.push_back(row);
                shell.push_back(row + nx - 1);
            }
        }
    long long fluid = 0;
    for (uint8_t v : h->mask) fluid += v == 0;
    h->fluid_cells = (int)std::max<long long>(1, fluid);
    h->n_shell = (int)shell.size();
    h->n_interior = (nx - 2) * (ny - 2) * (nz - 2);
}

// Link kind of pre-collision population q at a shell cell: the host twin of
// resolve_src (lbm_step.cuh), evaluated once per shell cell.
static int host_link_kind(const aeros_lbm* h, int x, int y, int z, int q) {
    const int n[3] = {h->nx, h->ny, h->nz};
    int sv[3] = {x - cx19(q), y - cy19(q), z - cz19(q)};
    const int per[3] = {h->p.periodic_x, 0, h->p.periodic_z};
    int outm = 0;
    for (int a = 0; a < 3; ++a) {
        if (per[a]) sv[a] = sv[a] < 0 ? sv[a] + n[a] : (sv[a] >= n[a] ? sv[a] - n[a] : sv[a]);
        if (sv[a] < 0 || sv[a] >= n[a]) outm |= 1 << a;
    }
    if (!outm) return h->mask[cidx(h, sv[0], sv[1], sv[2])] ? L_BOUNCE : L_REGULAR;
    if (h->p.lateral_bc == AEROS_LATERAL_FREESLIP && !((outm >> h->p.flow_axis) & 1)) {
        const int pos[3] = {x, y, z};
        int r[3];
        for (int a = 0; a < 3; ++a) r[a] = ((outm >> a) & 1) ? pos[a] : sv[a];
        return h->mask[cidx(h, r[0], r[1], r[2])] ? L_BOUNCE : L_FREESLIP;
    }
    return L_COPYOWN;
}

// Thermal link kind (0 regular, 1 bounce, 2 Dirichlet), host twin of th_resolve.
static int host_th_kind(const aeros_lbm* h, int x, int y, int z, int i) {
    int sx = x - cx19(i), sy = y - cy19(i), sz = z - cz19(i);
    if (sx < 0) sx = h->nx - 1; else if (sx >= h->nx) sx = 0;
    if (sz < 0) sz = h->nz - 1; else if (sz >= h->nz) sz = 0;
    const bool fixed = h->tp.fixed_wall_temps != 0;
    if (sy < 0 || sy >= h->ny) return fixed ? 2 : 1;
    if (h->mask[cidx(h, sx, sy, sz)]) return (fixed && (sy <= 0 || sy >= h->ny - 1)) ? 2 : 1;
    return 0;
}

static void build_shell_kinds(aeros_lbm* h) {
    h->shell_kind_host.assign(h->shell_host.size(), 0ull);
    for (size_t k = 0; k < h->shell_host.size(); ++k) {
        const int c = h->shell_host[k];
        const int x = c % h->nx, r = c / h->nx, y = r % h->ny, z = r / h->ny;
        unsigned long long v = 0;
        for (int q = 0; q < Q19; ++q) v |= (unsigned long long)host_link_kind(h, x, y, z, q) << (2 * q);
        if (h->th_on)
            for (int i = 0; i < Q7; ++i) v |= (unsigned long long)host_th_kind(h, x, y, z, i) << (40 + 2 * i);
        h->shell_kind_host[k] = v;
    }
}

// Host twin of resolve_kind (lbm_step.cuh): plane and cell of the source of
// population q of a shell cell under link kind `kind`.
static void host_resolve(const aeros_lbm* h, int x, int y, int z, int q, int kind, int& slot, int& idx) {
    const int c = cidx(h, x, y, z);
    if (kind == L_BOUNCE || kind == L_COPYOWN) { slot = q; idx = c; return; }
    int s0 = x - cx19(q), s1 = y - cy19(q), s2 = z - cz19(q);
    if (h->p.periodic_x) s0 = s0 < 0 ? s0 + h->nx : (s0 >= h->nx ? s0 - h->nx : s0);
    if (h->p.periodic_z) s2 = s2 < 0 ? s2 + h->nz : (s2 >= h->nz ? s2 - h->nz : s2);
    if (kind == L_REGULAR) { slot = opp19(q); idx = cidx(h, s0, s1, s2); return; }
    const bool o0 = s0 < 0 || s0 >= h->nx, o1 = s1 < 0 || s1 >= h->ny, o2 = s2 < 0 || s2 >= h->nz;
    const int rq = dir19_of(o0 ? -cx19(q) : cx19(q), o1 ? -cy19(q) : cy19(q), o2 ? -cz19(q) : cz19(q));
    slot = opp19(rq);
    idx = cidx(h, o0 ? x : s0, o1 ? y : s1, o2 ? z : s2);
}

// Odd-step gather and scatter element offsets of every shell cell (as the
// device resolves them), when plane * qstride + cell fits in 32 bits.
static int build_shell_tables(aeros_lbm* h) {
    const size_t ns = h->shell_host.size();
    if (!ns || (unsigned long long)h->qstride * Q19 > 0xffffffffull) return AEROS_OK;
    std::vector<uint32_t> gth(ns * Q19), sct(ns * Q19);
    for (size_t k = 0; k < ns; ++k) {
        const int c = h->shell_host[k];
        const int x = c % h->nx, r = c / h->nx, y = r % h->ny, z = r / h->ny;
        const unsigned long long sk = h->shell_kind_host[k];
        for (int q = 0; q < Q19; ++q) {
            int slot, idx;
            host_resolve(h, x, y, z, q, (int)((sk >> (2 * q)) & 3ull), slot, idx);
            gth[(size_t)q * ns + k] = (uint32_t)((unsigned long long)slot * h->qstride + idx);
            // post-collision f_j goes where the source of population opp(j) lies;
            // bounce-back and copy-own keep it in the cell's own slot opp(j)
            const int oj = opp19(q);
            const int kind = (int)((sk >> (2 * oj)) & 3ull);
            host_resolve(h, x, y, z, oj, kind, slot, idx);
            if (kind == L_BOUNCE || kind == L_COPYOWN) { slot = oj; idx = c; }
            sct[(size_t)q * ns + k] = (uint32_t)((unsigned long long)slot * h->qstride + idx);
        }
    }
    int rc = dalloc(h, &h->shell_gth, gth.size() * 4);
    if (rc == AEROS_OK) rc = dalloc(h, &h->shell_sct, sct.size() * 4);
    if (rc != AEROS_OK) return rc;
    CUDA_TRY(cudaMemcpy(h->shell_gth, gth.data(), gth.size() * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(h->shell_sct, sct.data(), sct.size() * 4, cudaMemcpyHostToDevice));
    return AEROS_OK;
}

static int host_plane_index(const aeros_lbm* h, int x, int y, int z) {
    const int ax = h->p.flow_axis;
    return ax == 0 ? y + h->ny * z : (ax == 1 ? x + h->nx * z : x + h->nx * y);
}

// Zero-gradient outlet: for every outlet-plane cell and unknown population q,
// the plane index of the side-buffer value it takes (the device rule in
// process_shell, evaluated once).
static int build_zerograd_table(aeros_lbm* h) {
    if (h->outlet_mode != 2) return AEROS_OK;
    const int ax = h->p.flow_axis, sg = h->p.flow_sign;
    const int n3[3] = {h->nx, h->ny, h->nz};
    const int per[3] = {h->p.periodic_x, 0, h->p.periodic_z};
    const int opos = sg > 0 ? n3[ax] - 1 : 0;
    const int P = h->out_plane;
    std::vector<int> tab((size_t)Q19 * P, 0);
    for (int z = 0; z < h->nz; ++z)
        for (int y = 0; y < h->ny; ++y)
            for (int x = 0; x < h->nx; ++x) {
                const int pos[3] = {x, y, z};
                if (pos[ax] != opos) continue;
                const int pi = host_plane_index(h, x, y, z);
                for (int q = 0; q < Q19; ++q) {
                    if (ca19(q, ax) * sg >= 0) continue;
                    int t[3] = {x - cx19(q), y - cy19(q), z - cz19(q)};
                    t[ax] = pos[ax];
                    for (int a = 0; a < 3; ++a) {
                        if (a == ax) continue;
                        if (t[a] < 0 || t[a] >= n3[a]) t[a] = per[a] ? (t[a] + n3[a]) % n3[a] : pos[a];
                    }
                    const bool wall = h->mask[cidx(h, t[0], t[1], t[2])] != 0;
                    tab[(size_t)q * P + pi] = wall ? pi : host_plane_index(h, t[0], t[1], t[2]);
                }
            }
    if (int rc = dalloc(h, &h->zg_src, tab.size() * 4)) return rc;
    CUDA_TRY(cudaMemcpy(h->zg_src, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
    return AEROS_OK;
}

static void fill_args(const aeros_lbm* h, FillArgs& fa, const float u[3]) {
    fa.f = h->f;
    fa.desc = h->desc;
    fa.qstride = h->qstride;
    fa.ncell = h->ncell;
    const float ux = u[0], uy = u[1], uz = u[2];
    float usqr = ux * ux + uy * uy + uz * uz;
    float vx = ux, vy = uy, vz = uz;
    if (usqr > 0.09f) {   // init limiter, lbm.cpp:725-730
        const float s = sqrtf(0.09f / usqr);
        vx *= s; vy *= s; vz *= s;
        usqr = vx * vx + vy * vy + vz * vz;
    }
    for (int q = 0; q < Q19; ++q) {
        fa.fluid[q] = eq_checked(q, 1.0f, vx, vy, vz, usqr);
        fa.wall[q] = eq_checked(q, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f);
        fa.dq[q] = h->shift.d[q];
    }
}

static int check_params(const aeros_lbm_params* p) {
    if (!p) return set_error(AEROS_ERR_INVALID, "params is NULL");
    if (p->nx < 4 || p->ny < 4 || p->nz < 4)
        return set_error(AEROS_ERR_INVALID, "grid %dx%dx%d: every dimension must be >= 4", p->nx, p->ny, p->nz);
    const long long n = (long long)p->nx * p->ny * p->nz;
    if (n > (1ll << 30)) return set_error(AEROS_ERR_INVALID, "grid of %lld cells exceeds 2^30", n);
    if (p->storage < AEROS_STORE_FP32 || p->storage > AEROS_STORE_BF16)
        return set_error(AEROS_ERR_INVALID, "unknown storage %d", p->storage);
    if (p->flow_axis < 0 || p->flow_axis > 2 || (p->flow_sign != 1 && p->flow_sign != -1))
        return set_error(AEROS_ERR_INVALID, "flow axis %d / sign %d", p->flow_axis, p->flow_sign);
    if (p->lateral_bc != AEROS_LATERAL_COPY && p->lateral_bc != AEROS_LATERAL_FREESLIP)
        return set_error(AEROS_ERR_INVALID, "unknown lateral_bc %d", p->lateral_bc);
    if (p->outlet_bc != AEROS_OUTLET_REFERENCE && p->outlet_bc != AEROS_OUTLET_ZEROGRAD)
        return set_error(AEROS_ERR_INVALID, "unknown outlet_bc %d", p->outlet_bc);
    if (p->storage_shift != AEROS_SHIFT_FREESTREAM && p->storage_shift != AEROS_SHIFT_WEIGHTS)
        return set_error(AEROS_ERR_INVALID, "unknown storage_shift %d", p->storage_shift);
    if (p->lateral_bc == AEROS_LATERAL_FREESLIP && !p->periodic_x && p->flow_axis != 0 &&
        p->outlet_bc == AEROS_OUTLET_REFERENCE && !p->convective_outlet)
        return set_error(AEROS_ERR_UNSUPPORTED, "free-slip lateral walls need an overriding outlet");
    if (p->lateral_bc == AEROS_LATERAL_FREESLIP && !p->periodic_x && p->outlet_bc == AEROS_OUTLET_REFERENCE &&
        !p->convective_outlet)
        return set_error(AEROS_ERR_UNSUPPORTED, "free-slip lateral walls need a convective or zero-gradient outlet");
    return AEROS_OK;
}

extern "C" int aeros_lbm_create(const aeros_lbm_params* params, const uint8_t* mask, aeros_lbm** out) {
    if (!out) return set_error(AEROS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (int rc = check_params(params)) return rc;
    if (!mask) return set_error(AEROS_ERR_INVALID, "mask is NULL");
    aeros_lbm* h = new (std::nothrow) aeros_lbm();
    if (!h) return set_error(AEROS_ERR_ALLOC, "host allocation failed");
    h->p = *params;
    h->nx = params->nx; h->ny = params->ny; h->nz = params->nz;
    h->ncell = h->nx * h->ny * h->nz;
    h->qstride = ((long long)h->ncell + 63) / 64 * 64;
    h->L = params->storage == AEROS_STORE_FP32 ? &launchers_fp32()
         : params->storage == AEROS_STORE_FP16 ? &launchers_fp16() : &launchers_bf16();
    h->esize = params->storage == AEROS_STORE_FP32 ? 4 : 2;
    h->outlet_mode = params->periodic_x ? 0
                   : (params->outlet_bc == AEROS_OUTLET_ZEROGRAD ? 2 : (params->convective_outlet ? 1 : 0));
    h->mask.assign(mask, mask + h->ncell);
    for (auto& v : h->mask)
        if (v > AEROS_CELL_GROUND) v = AEROS_CELL_SOLID;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (const char* e = getenv("AEROS_SPLIT")) h->split = atoi(e) != 0;
    if (const char* e = getenv("AEROS_FUSED")) h->fused = atoi(e) != 0;
    if (const char* e = getenv("AEROS_WARP")) h->warp = atoi(e) != 0;
    // measured on the sphere workload: 16-bit storage steps fastest with the
    // shell's tiles first in the interior queue, FP32 with one shell block per
    // SM (a domain with the thermal lattice keeps one shell block per SM)
    h->shell_blocks_per_sm = h->esize == 2 ? 0 : 1;
    if (const char* e = getenv("AEROS_SHELL_BLOCKS")) {
        h->shell_blocks_per_sm = std::max(0, std::min(8, atoi(e)));
        h->shell_blocks_set = true;
    }

    std::vector<int> shell;
    host_geometry(h, shell);
    int rc = AEROS_OK;
    const size_t n = (size_t)h->ncell;
#define ALLOC(ptr, bytes)                        \
    if ((rc = dalloc(h, &(ptr), (bytes))) != 0) { \
        free_handle(h);                          \
        return rc;                               \
    }
    // tail padding: the warp tiles' odd-step rows may run up to a tile + 16
    // bytes past the last plane's end, their descriptor copies past ncell
    ALLOC(h->f, ((size_t)h->qstride * Q19 + 64 + 4 * STEP_BLOCK) * h->esize);
    ALLOC(h->desc, (n + 64 + 2 * STEP_BLOCK) * 4);
    ALLOC(h->shell, (size_t)std::max(1, h->n_shell) * 4);
    ALLOC(h->shell_kind, (size_t)std::max(1, h->n_shell) * 8);
    // velocity buffers with VEL_GUARD cells of slack on both sides (the warp
    // tiles' stencil rows of the first and last tiles reach past the domain)
    for (int i = 0; i < 2; ++i) {
        ALLOC(h->u_alloc[i], (n + 2 * (size_t)VEL_GUARD) * 16);
        h->u[i] = h->u_alloc[i] + VEL_GUARD;
    }
    ALLOC(h->rho, n * 4);
    ALLOC(h->strain, n * 4);
    ALLOC(h->tke, n * 4);
    const int ax = params->flow_axis;
    h->out_plane = ax == 0 ? h->ny * h->nz : (ax == 1 ? h->nx * h->nz : h->nx * h->ny);
    if (h->outlet_mode) {
        ALLOC(h->out[0], (size_t)3 * Q19 * h->out_plane * 4);
        ALLOC(h->out[1], (size_t)3 * Q19 * h->out_plane * 4);
    }
    h->max_grid = std::max(1, h->sm_count) * 8;
    ALLOC(h->partials, (size_t)h->max_grid * sizeof(Partial));
    ALLOC(h->ctl, sizeof(Control));
    ALLOC(h->force_partials, (size_t)h->max_grid * 3 * sizeof(double));
    ALLOC(h->force_out, 4 * sizeof(double));
    ALLOC(h->force_counter, sizeof(unsigned int));
    ALLOC(h->area_count, sizeof(unsigned long long));
#undef ALLOC
    if (cudaMallocHost((void**)&h->ctl_host, sizeof(Control)) != cudaSuccess ||
        cudaMallocHost((void**)&h->force_host, 4 * sizeof(double)) != cudaSuccess) {
        free_handle(h);
        return set_error(AEROS_ERR_ALLOC, "pinned readback allocation failed");
    }
    auto fail = [&](cudaError_t e, const char* what) {
        free_handle(h);
        return set_error(AEROS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    };
    cudaError_t e;
    if ((e = cudaEventCreate(&h->ev0)) != cudaSuccess) return fail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&h->ev1)) != cudaSuccess) return fail(e, "cudaEventCreate");
    {
        uint8_t* dm = nullptr;
        // stream-ordered scratch and stream syncs only: creating a domain does
        // not wait for work other streams have in flight (a running batch)
        if ((e = cudaMallocAsync((void**)&dm, 3 * n, nullptr)) != cudaSuccess) return fail(e, "descriptor scratch");
        DescArgs da;
        da.nx = h->nx; da.ny = h->ny; da.nz = h->nz;
        da.flow_axis = params->flow_axis;
        const int na = params->flow_axis == 0 ? h->nx : (params->flow_axis == 1 ? h->ny : h->nz);
        const bool pos = params->flow_sign > 0;
        da.inlet_pos = pos ? 0 : na - 1;
        da.outlet_pos = pos ? na - 1 : 0;
        da.ic = pos ? na - 2 : 1;
        da.ic2 = pos ? na - 3 : 2;
        da.outlet_mode = h->outlet_mode;
        e = cudaMemcpy(dm, h->mask.data(), n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = build_descriptors(da, dm, dm + n, dm + 2 * n, h->desc, nullptr);
        cudaFreeAsync(dm, nullptr);
        if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
        if (e != cudaSuccess) return fail(e, "descriptor build");
    }
    if (h->n_shell && (e = cudaMemcpy(h->shell, shell.data(), shell.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e, "shell upload");
    h->shell_host = shell;
    build_shell_kinds(h);
    if (h->n_shell && (e = cudaMemcpy(h->shell_kind, h->shell_kind_host.data(), h->shell_kind_host.size() * 8,
                                      cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e, "shell kinds upload");
    if (getenv("AEROS_SHELL_TABLES") == nullptr || atoi(getenv("AEROS_SHELL_TABLES")) != 0) {
        int rc2 = build_shell_tables(h);
        if (rc2 == AEROS_OK) rc2 = build_zerograd_table(h);
        if (rc2) {
            free_handle(h);
            return rc2;
        }
    }
    for (auto& b : h->u)
        if ((e = cudaMemset(b, 0, n * 16)) != cudaSuccess) return fail(e, "u memset");
    if ((e = cudaMemset(h->strain, 0, n * 4)) != cudaSuccess) return fail(e, "memset");
    if ((e = cudaMemset(h->force_counter, 0, 4)) != cudaSuccess) return fail(e, "memset");
    if ((e = cudaMemset(h->tke, 0, n * 4)) != cudaSuccess) return fail(e, "memset");
    {
        std::vector<float> ones(n, 1.0f);
        if ((e = cudaMemcpy(h->rho, ones.data(), n * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "rho init");
    }
    Control c0;
    memset(&c0, 0, sizeof(c0));
    c0.avg_rho = 1.0f;
    if ((e = cudaMemcpy(h->ctl, &c0, sizeof(c0), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e, "ctl init");
    *h->ctl_host = c0;

    // inlet equilibrium in storage form (lbm.cpp:1414-1429) and convective
    // coefficient (lbm.cpp:1468-1470)
    const float ui0 = params->u_in[0], ui1 = params->u_in[1], ui2 = params->u_in[2];
    const float usq = ui0 * ui0 + ui1 * ui1 + ui2 * ui2;
    const bool shifted = params->storage != AEROS_STORE_FP32;
    for (int q = 0; q < Q19; ++q) {
        const float v = eq_checked(q, 1.0f, ui0, ui1, ui2, usq);
        h->feq_in[q] = shifted ? v - w19(q) : v;
    }
    if (shifted && params->storage_shift == AEROS_SHIFT_FREESTREAM && !params->periodic_x) {
        // s_q - w_q = w_q (3 c.u + 4.5 (c.u)^2 - 1.5 u^2), u = the inlet velocity
        // (the velocity the far field relaxes to); evaluated in double, rounded
        // once. A domain without an inlet (periodic in x: no inlet override)
        // keeps the rest state s = w: nothing drives it towards its initial
        // velocity, and a flow decaying from it would store ever larger
        // deviations (viscosity decay from u = 0.08: -42 % in FP16 against -0.5 %)
        const float* us = params->u_in;
        const double sx = us[0], sy = us[1], sz = us[2];
        const double u2 = sx * sx + sy * sy + sz * sz;
        for (int q = 0; q < Q19; ++q) {
            const double cu = cx19(q) * sx + cy19(q) * sy + cz19(q) * sz;
            h->shift.d[q] = (float)((double)w19(q) * (3.0 * cu + 4.5 * cu * cu - 1.5 * u2));
        }
    }
    float U0mag = sqrtf(usq);
    if (!std::isfinite(U0mag) || U0mag < 1e-6f) U0mag = 0.08f;
    float conv = U0mag * 0.8f;
    if (conv > 0.5f) conv = 0.5f;
    if (conv < 0.01f) conv = 0.08f;
    h->conv = conv;

    FillArgs fa;
    fill_args(h, fa, params->u_init);
    if ((e = h->L->fill_uniform(fa, nullptr)) != cudaSuccess) return fail(e, "fill");
    if (h->outlet_mode) {
        // side buffer entries of wall cells hold what the reference reads
        // from a wall cell's populations on that step parity: the initial
        // equilibrium on odd steps, zero on even steps
        for (int par = 0; par < 2; ++par) {
            std::vector<float> ob((size_t)3 * Q19 * h->out_plane);
            for (int pl = 0; pl < 3; ++pl)
                for (int q = 0; q < Q19; ++q) {
                    const float plain = par == 1 ? fa.wall[q] : 0.0f;
                    for (int k = 0; k < h->out_plane; ++k)
                        ob[((size_t)pl * Q19 + q) * h->out_plane + k] = shifted ? plain - w19(q) : plain;
                }
            if ((e = cudaMemcpy(h->out[par], ob.data(), ob.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
                return fail(e, "outlet buffer init");
        }
    }
    if ((e = cudaStreamSynchronize(nullptr)) != cudaSuccess) return fail(e, "init");
    for (int o = 0; o < 2; ++o)
        for (int t = 0; t < 2; ++t) h->grid[o][t] = std::min(h->max_grid, std::max(1, h->sm_count) * h->L->occupancy(o, t));
    for (int o = 0; o < 2; ++o)
        for (int t = 0; t < 2; ++t) h->fused_grid[o][t] = std::max(1, h->sm_count) * h->L->fused_occupancy(o, t);
    for (int o = 0; o < 2; ++o) h->warp_grid[o] = std::max(1, h->sm_count) * h->L->warp_occupancy(o);
    h->stats.avg_rho = 1.0f;
    h->stats.fluid_cells = h->fluid_cells;
    *out = h;
    return AEROS_OK;
}

extern "C" int aeros_lbm_destroy(aeros_lbm* h) {
    if (!h) return set_error(AEROS_ERR_INVALID, "handle is NULL");
    if (h->batch) return set_error(AEROS_ERR_STATE, "domain is in a batch: remove it first");
    cudaStreamSynchronize(h->stream);
    free_handle(h);
    return AEROS_OK;
}

extern "C" int aeros_lbm_set_stream(aeros_lbm* h, void* s) {
    if (!h) return set_error(AEROS_ERR_INVALID, "handle is NULL");
    h->stream = (cudaStream_t)s;
    return AEROS_OK;
}

extern "C" int aeros_lbm_synchronize(aeros_lbm* h) {
    if (!h) return set_error(AEROS_ERR_INVALID, "handle is NULL");
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return AEROS_OK;
}

// Shift of the 16-bit D3Q7 storage: the conduction profile between fixed
// wall temperatures (hot wall row 0, cold wall row ny-1, the profile the
// walls impose: hot at y = 0.5, cold at y = ny - 1.5), else Tref.
static ShiftT th_shift(const aeros_lbm* h) {
    ShiftT ts;
    ts.nx = h->nx;
    ts.ny = h->ny;
    const float hot = h->tp.hot_temp, cold = h->tp.cold_temp;
    if (h->tp.fixed_wall_temps && h->ny > 2) {
        ts.tc1 = (cold - hot) / (float)(h->ny - 2);
        ts.tc0 = hot - 0.5f * ts.tc1;
    } else {
        ts.tc0 = 0.5f * (hot + cold);
        ts.tc1 = 0.0f;
    }
    return ts;
}

StepOffsets step_offsets(const aeros_lbm* h) {
    StepOffsets O;
    for (int q = 0; q < Q19; ++q) {
        const long long nb = cx19(q) + cy19(q) * (long long)h->nx + cz19(q) * (long long)h->nx * h->ny;
        O.goff[q] = ((long long)opp19(q) * h->qstride - nb) * h->esize;
        O.soff[q] = ((long long)q * h->qstride + nb) * h->esize;
    }
    return O;
}

void base_args(const aeros_lbm* h, StepArgs& A) {
    memset(&A, 0, sizeof(A));
    A.nx = h->nx; A.ny = h->ny; A.nz = h->nz; A.nxny = h->nx * h->ny; A.ncell = h->ncell;
    A.qstride = h->qstride;
    A.n_interior = h->n_interior;
    A.ntiles_interior = (h->n_interior + STEP_BLOCK - 1) / STEP_BLOCK;
    A.n_shell = h->n_shell;
    A.ntiles = A.ntiles_interior + (h->n_shell + STEP_BLOCK - 1) / STEP_BLOCK;
    {
        const int nsh = A.ntiles - A.ntiles_interior;
        A.shell_stride = nsh > 0 ? std::max(1, A.ntiles / nsh) : 1;
    }
    A.div_ix = FastDiv((uint32_t)(h->nx - 2));
    A.div_iy = FastDiv((uint32_t)(h->ny - 2));
    A.div_x = FastDiv((uint32_t)h->nx);
    A.div_y = FastDiv((uint32_t)h->ny);
    for (int q = 0; q < Q19; ++q) {
        A.fq[q] = static_cast<char*>(h->f) + (size_t)q * (size_t)h->qstride * h->esize;
        A.nbq[q] = cx19(q) + cy19(q) * h->nx + cz19(q) * h->nx * h->ny;
    }
    A.f = h->f; A.desc = h->desc; A.shell = h->shell; A.shell_kind = h->shell_kind;
    A.shell_gth = h->shell_gth; A.shell_sct = h->shell_sct;
    A.zg_src = h->zg_src;
    A.rho = h->rho; A.strain = h->strain; A.tke = h->tke;
    A.out_plane = h->out_plane;
    A.g = h->g; A.T = h->T; A.T_buoy = h->T_buoy;
    A.partials = h->partials; A.ctl = h->ctl;
    const aeros_lbm_params& p = h->p;
    float tau0 = p.tau;   // lbm.cpp:918-920
    if (!std::isfinite(tau0) || tau0 < 0.51f) tau0 = 0.55f;
    if (tau0 > 1.5f) tau0 = 1.5f;
    A.tau0 = tau0;
    float Cs = p.smagorinsky_c;   // lbm.cpp:1130-1133
    if (!std::isfinite(Cs) || Cs < 0.0f) Cs = 0.12f;
    if (Cs > 0.3f) Cs = 0.3f;
    A.Cs = Cs;
    A.velScale2 = p.vel_scale * p.vel_scale;
    A.Fx = p.body_force[0]; A.Fy = p.body_force[1]; A.Fz = p.body_force[2];
    for (int i = 0; i < 3; ++i) A.uin[i] = p.u_in[i];
    for (int q = 0; q < Q19; ++q) A.feq_in[q] = h->feq_in[q];
    {
        const float sc = h->p.storage == AEROS_STORE_FP16 ? STORE_SCALE_F16 : 1.0f;
        for (int q = 0; q < Q19; ++q) {
            A.dq[q] = h->shift.d[q];
            A.dqs[q] = h->shift.d[q] * sc;   // a power of two: exact
        }
    }
    A.conv = h->conv;
    A.flow_axis = p.flow_axis; A.flow_sign = p.flow_sign;
    {
        const int na = p.flow_axis == 0 ? h->nx : (p.flow_axis == 1 ? h->ny : h->nz);
        A.inlet_pos = p.flow_sign > 0 ? 0 : na - 1;   // as the descriptor's D_INLET plane
    }
    A.periodic_x = p.periodic_x; A.periodic_z = p.periodic_z;
    A.use_trt = p.use_trt; A.use_les = p.use_les;
    A.freeslip = p.lateral_bc == AEROS_LATERAL_FREESLIP;
    A.outlet_mode = h->outlet_mode;
    A.total_div10 = h->ncell / 10;
    {
        const int nsh = A.ntiles - A.ntiles_interior;
        A.fused = h->fused;
        // warp tiles (non-thermal): rows start on 16-byte boundaries when nx is
        // a multiple of 16 bytes of storage; tiles are linear runs of WT cells
        // from the first to the last interior cell, inside the domain when
        // nx*ny >= WT; chunk offsets are 32-bit
        const int WT = h->L->warp_tile;
        const bool small = (double)h->qstride * Q19 * h->esize + 64.0 * WT < 2147483647.0;
        A.warp = h->warp && !h->th_on && h->n_interior > 0 && h->nx % h->L->warp_pad == 0 &&
                 h->nx * h->ny >= WT && small;
        if (A.warp) {
            const int first = h->nx * h->ny + h->nx + 1, last = h->ncell - h->nx * h->ny - h->nx - 2;
            A.wt_first = first / WT;
            A.wt_last = last / WT;
            A.warp_grid = h->warp_grid[0];
            A.warp_grid_odd = h->warp_grid[1];
        }
        // the warp tiles need shell blocks; the fused kernel without them takes
        // the shell's tiles first from its queue
        const int per_sm = (A.warp || (h->th_on && !h->shell_blocks_set)) ? std::max(1, h->shell_blocks_per_sm)
                                                                            : h->shell_blocks_per_sm;
        A.shell_blocks = (A.fused || A.warp) ? std::min(nsh, std::max(1, h->sm_count) * per_sm) : 0;
        A.fused_grid = h->fused_grid[0][h->th_on ? 1 : 0];
        A.fused_grid_odd = h->fused_grid[1][h->th_on ? 1 : 0];
        A.split = h->split && nsh > 0 && !A.fused && !A.warp;
        A.shell_grid = A.split ? std::min(nsh, std::max(1, h->sm_count) * 4) : 0;
        A.shell_part_base = 0;   // set by the launcher (after the interior grid's slots)
    }
    {
        // bounded forces keep every intermediate of a clean cell finite
        float fmax = std::max(std::fabs(p.body_force[0]), std::max(std::fabs(p.body_force[1]), std::fabs(p.body_force[2])));
        if (h->th_on) fmax += std::fabs(h->glb) * (std::fabs(h->tp.hot_temp - h->tp.cold_temp) + 2.0f);
        A.fast_ok = std::isfinite(fmax) && fmax <= 1.0f;
        A.shifted_fast = h->esize == 2 && fmax == 0.0f && !h->th_on;
    }
    A.fluid_cells = h->fluid_cells;
    A.conv_threshold = p.convergence_threshold;
    A.th_on = h->th_on;
    if (h->th_on) {
        A.th_fixed = h->tp.fixed_wall_temps;
        A.th_ylo = h->ylo;
        A.th_invtau = 1.0f / h->tau_t;
        A.th_hot = h->tp.hot_temp;
        A.th_cold = h->tp.cold_temp;
        A.th_tref = 0.5f * (h->tp.hot_temp + h->tp.cold_temp);
        const ShiftT ts = th_shift(h);
        A.th_tc0 = ts.tc0;
        A.th_tc1 = ts.tc1;
        A.th_glb = h->glb;
        A.th_H = h->H;
        A.th_buoy_mode = h->th_buoy_mode;
        A.th_rows_n = (double)((long)h->nx * (long)h->nz * (long)(h->yhi - h->ylo + 1));
    }
}

// Brings both lattices into the layout an even step gathers from with no
// pending overrides (after init, reset, or materialize + write-back).
static int normalize_layout(aeros_lbm* h);

StepVar step_var(const aeros_lbm* h, bool write_obs) {
    StepVar V;
    V.up = h->u[h->ubuf];
    V.uc = h->u[h->ubuf ^ 1];
    V.out_w = h->out[h->out_par];
    V.out_r = h->out[h->out_par ^ 1];
    V.apply_overrides = h->overrides_next;
    V.write_obs = write_obs;
    V.write_u = h->p.use_les || write_obs;
    return V;
}

static int launch_materialize(aeros_lbm* h, float* d_f, float* d_g) {
    StepArgs A;
    base_args(h, A);
    A.mat_f = d_f;
    A.mat_g = d_g;
    const StepVar V = step_var(h, false);
    const int grid = h->grid[h->next_odd][h->th_on];
    CUDA_TRY(h->L->step(A, V, step_offsets(h), h->next_odd, h->th_on, true, grid, h->stream));
    return AEROS_OK;
}

static int normalize_layout(aeros_lbm* h) {
    if (!h->next_odd && !h->overrides_next) return AEROS_OK;
    float *df = nullptr, *dg = nullptr;
    const size_t n = (size_t)h->ncell;
    if (cudaMalloc((void**)&df, n * Q19 * 4) != cudaSuccess) return set_error(AEROS_ERR_ALLOC, "normalize buffer");
    if (h->th_on && cudaMalloc((void**)&dg, n * Q7 * 4) != cudaSuccess) {
        cudaFree(df);
        return set_error(AEROS_ERR_ALLOC, "normalize buffer");
    }
    int rc = launch_materialize(h, df, dg);
    if (rc == AEROS_OK) {
        cudaError_t e = h->L->write_pre(h->f, h->desc, h->qstride, h->ncell, df, Q19, th_shift(h), h->shift, h->stream);
        if (e == cudaSuccess && h->th_on)
            e = h->L->write_pre(h->g, h->desc, h->qstride, h->ncell, dg, Q7, th_shift(h), h->shift, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = set_error(AEROS_ERR_CUDA, "normalize: %s", cudaGetErrorString(e));
    }
    cudaFree(df);
    cudaFree(dg);
    if (rc == AEROS_OK) {
        h->next_odd = false;
        h->overrides_next = false;
    }
    return rc;
}

static int enqueue_steps(aeros_lbm* h, int nsteps) {
    if (nsteps < 0) return set_error(AEROS_ERR_INVALID, "nsteps %d < 0", nsteps);
    h->last_launches = 0;
    h->last_kernels = 0;
    h->kexec_before = h->ctl_host->kexec;
    CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
    StepArgs A;
    base_args(h, A);
    for (int i = 0; i < nsteps; ++i) {
        const StepVar V = step_var(h, i == nsteps - 1);
        A.th_buoy_mode = h->th_buoy_mode;
        const int grid = h->grid[h->next_odd][h->th_on];
        CUDA_TRY(h->L->step(A, V, step_offsets(h), h->next_odd, h->th_on, false, grid, h->stream));
        h->last_launches++;
        h->last_kernels += A.split ? 2 : 1;
        h->next_odd = !h->next_odd;
        h->overrides_next = true;
        h->out_par ^= 1;
        h->ubuf ^= 1;
        if (h->th_on) {
            h->th_buoy_mode = 0;
            h->th_stepped = true;
        }
    }
    CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->ctl_host, h->ctl, sizeof(Control), cudaMemcpyDeviceToHost, h->stream));
    h->stats_dirty = true;
    h->last_diverged = false;
    return AEROS_OK;
}

// Reads the control block of the last enqueued batch; on a tripped
// divergence guard re-equilibrates (lbm.cpp:1583-1600).
int finish_batch(aeros_lbm* h) {
    if (!h->stats_dirty) return AEROS_OK;
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->stats_dirty = false;
    Control& c = *h->ctl_host;
    aeros_lbm_stats& s = h->stats;
    if (c.halt) {
        const long long executed = c.kexec - h->kexec_before;
        const long long launched = h->last_launches;
        // undo the host-side layout bookkeeping of launches that returned early
        const long long skipped = launched - executed;
        if (skipped & 1) {
            h->ubuf ^= 1;
            h->out_par ^= 1;
        }
        FillArgs fa;
        fill_args(h, fa, h->p.u_in);
        for (int q = 0; q < Q19; ++q) fa.fluid[q] = eq_checked(q, 1.0f, h->p.u_in[0], h->p.u_in[1], h->p.u_in[2],
                                                                h->p.u_in[0] * h->p.u_in[0] + h->p.u_in[1] * h->p.u_in[1] +
                                                                    h->p.u_in[2] * h->p.u_in[2]);
        const float* uin = h->p.u_in;
        CUDA_TRY(h->L->reset(h->f, h->desc, h->qstride, h->ncell, fa, h->rho, h->u[h->ubuf], uin, h->stream));
        h->next_odd = false;
        h->overrides_next = false;
        const float usqr = uin[0] * uin[0] + uin[1] * uin[1] + uin[2] * uin[2];
        c.avg_rho = 1.0f;
        c.avg_ke = usqr;
        c.halt = 0;
        c.halt_kind = 0;
        // clear the device flag; keep the statistics the guard left
        Control dc = c;
        dc.blocks_done = 0;
        CUDA_TRY(cudaMemcpyAsync(h->ctl, &dc, sizeof(Control), cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        h->last_diverged = true;
    }
    s.step = c.steps;
    s.avg_rho = c.avg_rho;
    s.avg_kinetic = c.avg_ke;
    s.avg_tke = c.avg_tke;
    s.max_velocity_lb = c.max_u;
    s.convergence = c.convergence;
    s.converged = c.converged;
    s.diverged = h->last_diverged ? 1 : 0;
    s.negative_pops = c.neg;
    s.bad_pops = c.bad;
    s.rho_out_of_range = c.rout;
    s.rho_non_finite = c.rnf;
    s.u_limited = c.ulim;
    s.nan_count = c.nan;
    s.sum_rho = c.sum_rho;
    s.sum_kinetic = c.sum_ke;
    s.sum_tke = c.sum_tke;
    s.nusselt = c.nusselt;
    s.mean_t = c.mean_t;
    s.fluid_cells = h->fluid_cells;
    return AEROS_OK;
}

extern "C" int aeros_lbm_step_async(aeros_lbm* h, int nsteps) {
    if (!h) return set_error(AEROS_ERR_INVALID, "handle is NULL");
    if (int rc = finish_batch(h)) return rc;
    return enqueue_steps(h, nsteps);
}

extern "C" int aeros_lbm_step(aeros_lbm* h, int nsteps) {
    if (int rc = aeros_lbm_step_async(h, nsteps)) return rc;
    return finish_batch(h);
}

extern "C" int aeros_lbm_get_stats(aeros_lbm* h, aeros_lbm_stats* out) {
    if (!h || !out) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (int rc = finish_batch(h)) return rc;
    *out = h->stats;
    return AEROS_OK;
}

extern "C" int aeros_lbm_last_step_ms(aeros_lbm* h, float* ms) {
    if (!h || !ms) return set_error(AEROS_ERR_INVALID, "NULL argument");
    CUDA_TRY(cudaEventSynchronize(h->ev1));
    CUDA_TRY(cudaEventElapsedTime(ms, h->ev0, h->ev1));
    return AEROS_OK;
}

extern "C" int aeros_lbm_last_launch_count(aeros_lbm* h, int64_t* n) {
    if (!h || !n) return set_error(AEROS_ERR_INVALID, "NULL argument");
    *n = h->last_kernels;
    return AEROS_OK;
}

extern "C" int aeros_lbm_device_bytes(aeros_lbm* h, uint64_t* b) {
    if (!h || !b) return set_error(AEROS_ERR_INVALID, "NULL argument");
    *b = h->dev_bytes;
    return AEROS_OK;
}

// ---------------------------------------------------------------------------
// state I/O
// ---------------------------------------------------------------------------
namespace {
// the velocity (x, y, z, pad per cell) as three planes, for a direct copy
// into the caller's arrays
__global__ void k_split_u(const float4* __restrict__ u, float* ux, float* uy, float* uz, long long n) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const float4 v = u[c];
        ux[c] = v.x;
        uy[c] = v.y;
        uz[c] = v.z;
    }
}
}  // namespace

extern "C" int aeros_lbm_read_fields(aeros_lbm* h, float* rho, float* ux, float* uy, float* uz, float* strain,
                                     float* tke) {
    if (!h) return set_error(AEROS_ERR_INVALID, "handle is NULL");
    if (int rc = finish_batch(h)) return rc;
    const size_t n = (size_t)h->ncell;
    const size_t b = n * 4;
    if (rho) CUDA_TRY(cudaMemcpyAsync(rho, h->rho, b, cudaMemcpyDeviceToHost, h->stream));
    if (strain) CUDA_TRY(cudaMemcpyAsync(strain, h->strain, b, cudaMemcpyDeviceToHost, h->stream));
    if (tke) CUDA_TRY(cudaMemcpyAsync(tke, h->tke, b, cudaMemcpyDeviceToHost, h->stream));
    if (ux || uy || uz) {
        if (!h->u_split) CUDA_TRY(cudaMalloc((void**)&h->u_split, 3 * b));
        const int blocks = (int)std::min<long long>(((long long)n + 255) / 256, (long long)std::max(1, h->sm_count) * 8);
        k_split_u<<<blocks, 256, 0, h->stream>>>(h->u[h->ubuf], h->u_split, h->u_split + n, h->u_split + 2 * n,
                                                 (long long)n);
        CUDA_TRY(cudaGetLastError());
        float* dst[3] = {ux, uy, uz};
        for (int k = 0; k < 3; ++k)
            if (dst[k]) CUDA_TRY(cudaMemcpyAsync(dst[k], h->u_split + k * n, b, cudaMemcpyDeviceToHost, h->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return AEROS_OK;
}

extern "C" int aeros_host_alloc(size_t bytes, void** out) {
    if (!out) return set_error(AEROS_ERR_INVALID, "NULL argument");
    *out = nullptr;
    if (cudaHostAlloc(out, bytes ? bytes : 16, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return set_error(AEROS_ERR_ALLOC, "page-locked host buffer of %zu bytes", bytes);
    }
    return AEROS_OK;
}

extern "C" int aeros_host_free(void* p) {
    if (p) CUDA_TRY(cudaFreeHost(p));
    return AEROS_OK;
}

extern "C" int aeros_lbm_device_fields(aeros_lbm* h, const float** rho, const float** u4) {
    if (!h) return set_error(AEROS_ERR_INVALID, "handle is NULL");
    if (int rc = finish_batch(h)) return rc;
    if (rho) *rho = h->rho;
    if (u4) *u4 = reinterpret_cast<const float*>(h->u[h->ubuf]);
    return AEROS_OK;
}

extern "C" int aeros_lbm_read_populations(aeros_lbm* h, float* f) {
    if (!h || !f) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (int rc = finish_batch(h)) return rc;
    float* df = nullptr;
    const size_t n = (size_t)h->ncell;
    if (cudaMalloc((void**)&df, n * Q19 * 4) != cudaSuccess) return set_error(AEROS_ERR_ALLOC, "readback buffer");
    float* dg = nullptr;
    if (h->th_on && cudaMalloc((void**)&dg, n * Q7 * 4) != cudaSuccess) {
        cudaFree(df);
        return set_error(AEROS_ERR_ALLOC, "readback buffer");
    }
    int rc = launch_materialize(h, df, dg);
    if (rc == AEROS_OK) {
        cudaError_t e = cudaMemcpyAsync(f, df, n * Q19 * 4, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = set_error(AEROS_ERR_CUDA, "readback: %s", cudaGetErrorString(e));
    }
    cudaFree(df);
    cudaFree(dg);
    if (rc) return rc;
    // wall cells: initial equilibrium (never touched by the solver)
    for (size_t c = 0; c < n; ++c)
        if (h->mask[c])
            for (int q = 0; q < Q19; ++q) f[(size_t)q * n + c] = w19(q);
    return AEROS_OK;
}

extern "C" int aeros_lbm_write_populations(aeros_lbm* h, const float* f) {
    if (!h || !f) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (int rc = finish_batch(h)) return rc;
    if (int rc = normalize_layout(h)) return rc;
    float* df = nullptr;
    const size_t n = (size_t)h->ncell;
    if (cudaMalloc((void**)&df, n * Q19 * 4) != cudaSuccess) return set_error(AEROS_ERR_ALLOC, "upload buffer");
    cudaError_t e = cudaMemcpyAsync(df, f, n * Q19 * 4, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = h->L->write_pre(h->f, h->desc, h->qstride, h->ncell, df, Q19, th_shift(h), h->shift, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(df);
    if (e != cudaSuccess) return set_error(AEROS_ERR_CUDA, "write populations: %s", cudaGetErrorString(e));
    return AEROS_OK;
}

extern "C" int aeros_lbm_set_equilibrium(aeros_lbm* h, const float* rho, const float* ux, const float* uy,
                                         const float* uz) {
    if (!h || !ux || !uy || !uz) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (int rc = finish_batch(h)) return rc;
    if (int rc = normalize_layout(h)) return rc;
    const size_t n = (size_t)h->ncell;
    float* d = nullptr;
    if (cudaMalloc((void**)&d, n * 4 * 4) != cudaSuccess) return set_error(AEROS_ERR_ALLOC, "upload buffer");
    cudaError_t e = cudaSuccess;
    if (rho) e = cudaMemcpyAsync(d, rho, n * 4, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d + n, ux, n * 4, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d + 2 * n, uy, n * 4, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d + 3 * n, uz, n * 4, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = h->L->set_equilibrium(h->f, h->desc, h->qstride, h->ncell, rho ? d : nullptr, d + n, d + 2 * n, d + 3 * n,
                                  h->shift, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    if (e != cudaSuccess) return set_error(AEROS_ERR_CUDA, "set equilibrium: %s", cudaGetErrorString(e));
    return AEROS_OK;
}

extern "C" int aeros_lbm_read_mask(aeros_lbm* h, uint8_t* mask, uint8_t* wall_dist) {
    if (!h) return set_error(AEROS_ERR_INVALID, "handle is NULL");
    if (mask) memcpy(mask, h->mask.data(), h->mask.size());
    if (wall_dist) {
        if (h->wall.size() != h->mask.size()) host_wall_distance(h);
        memcpy(wall_dist, h->wall.data(), h->wall.size());
    }
    return AEROS_OK;
}

// ---------------------------------------------------------------------------
// thermal (host side mirrors thermal_lbm.cpp:84-197)
// ---------------------------------------------------------------------------
static bool th_wall_temp(const aeros_lbm* h, int y, float* Tw) {
    if (!h->tp.fixed_wall_temps) return false;
    if (y <= 0) { *Tw = h->tp.hot_temp; return true; }
    if (y >= h->ny - 1) { *Tw = h->tp.cold_temp; return true; }
    return false;
}

static int upload_T(aeros_lbm* h, const std::vector<float>& T) {
    CUDA_TRY(cudaMemcpyAsync(h->T, T.data(), T.size() * 4, cudaMemcpyHostToDevice, h->stream));
    StepArgs A;
    base_args(h, A);
    CUDA_TRY(h->L->thermal_fill(A, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return AEROS_OK;
}

extern "C" int aeros_lbm_thermal_init(aeros_lbm* h, const aeros_thermal_params* tp) {
    if (!h || !tp) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (int rc = finish_batch(h)) return rc;
    if (!tp->enabled) {
        h->th_on = false;
        return AEROS_OK;
    }
    if (int rc = normalize_layout(h)) return rc;
    h->tp = *tp;
    float nu = tp->nu_lb;
    if (!std::isfinite(nu) || nu <= 0.0f) nu = 0.05f;
    h->ylo = -1;
    h->yhi = -1;
    for (int y = 0; y < h->ny; ++y) {
        bool fluid = false;
        for (int z = 0; z < h->nz && !fluid; ++z)
            for (int x = 0; x < h->nx && !fluid; ++x)
                if (!h->mask[cidx(h, x, y, z)]) fluid = true;
        if (fluid) {
            if (h->ylo < 0) h->ylo = y;
            h->yhi = y;
        }
    }
    if (h->ylo < 0 || h->yhi <= h->ylo) return set_error(AEROS_ERR_INVALID, "thermal: fewer than two fluid rows");
    h->H = (float)(h->yhi - h->ylo + 1);
    const float pr = std::max(0.05f, tp->prandtl);
    h->alpha = nu / pr;
    h->tau_t = 0.5f + h->alpha / 0.25f;
    if (!std::isfinite(h->tau_t) || h->tau_t < 0.505f) h->tau_t = 0.505f;
    if (h->tau_t > 1.5f) {
        h->tau_t = 1.5f;
        h->alpha = 0.25f * (h->tau_t - 0.5f);
    }
    const float dT = tp->hot_temp - tp->cold_temp;
    h->glb = tp->rayleigh * nu * h->alpha / (std::max(1e-6f, std::fabs(dT)) * h->H * h->H * h->H);
    const size_t n = (size_t)h->ncell;
    if (!h->g) {
        int rc;
        if ((rc = dalloc(h, &h->g, (size_t)h->qstride * Q7 * h->esize))) return rc;
        if ((rc = dalloc(h, &h->T, n * 4))) return rc;
        if ((rc = dalloc(h, &h->T_buoy, n * 4))) return rc;
    }
    // thermalResetField, thermal_lbm.cpp:154-185
    std::vector<float> T(n);
    const float Th = tp->hot_temp, Tc = tp->cold_temp;
    const float amp = tp->perturbation * (Th - Tc);
    for (int z = 0; z < h->nz; ++z)
        for (int y = 0; y < h->ny; ++y)
            for (int x = 0; x < h->nx; ++x) {
                const int c = cidx(h, x, y, z);
                float t;
                if (h->mask[c]) {
                    float Tw;
                    t = th_wall_temp(h, y, &Tw) ? Tw : 0.5f * (Th + Tc);
                } else {
                    const float s = (float)(y - h->ylo) / std::max(1.0f, h->H - 1.0f);
                    t = Th + (Tc - Th) * s;
                    const float px = 6.2831853f * (float)x / (float)h->nx;
                    const float py = 3.1415926f * s;
                    t += amp * std::cos(px) * std::sin(py);
                }
                T[c] = t;
            }
    h->th_on = true;
    build_shell_kinds(h);
    if (h->n_shell)
        CUDA_TRY(cudaMemcpy(h->shell_kind, h->shell_kind_host.data(), h->shell_kind_host.size() * 8,
                            cudaMemcpyHostToDevice));
    h->th_buoy_mode = 1;   // buoyancy field starts at zero (thermal_lbm.cpp:132)
    h->th_stepped = false;
    Control c = *h->ctl_host;
    c.nusselt = 0.0f;
    c.th_valid = 0;
    {
        double sum = 0.0;
        for (int z = 0; z < h->nz; ++z)
            for (int y = h->ylo; y <= h->yhi; ++y)
                for (int x = 0; x < h->nx; ++x)
                    if (!h->mask[cidx(h, x, y, z)]) sum += T[cidx(h, x, y, z)];
        const long nn = (long)h->nx * h->nz * (h->yhi - h->ylo + 1);
        c.mean_t = nn > 0 ? (float)(sum / (double)nn) : 0.5f;
    }
    *h->ctl_host = c;
    CUDA_TRY(cudaMemcpy(h->ctl, &c, sizeof(c), cudaMemcpyHostToDevice));
    h->stats.mean_t = c.mean_t;
    h->stats.nusselt = 0.0f;
    return upload_T(h, T);
}

extern "C" int aeros_lbm_thermal_upload(aeros_lbm* h, const float* T) {
    if (!h || !T) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (!h->th_on) return set_error(AEROS_ERR_STATE, "thermal lattice not initialised");
    if (int rc = finish_batch(h)) return rc;
    if (int rc = normalize_layout(h)) return rc;
    const size_t n = (size_t)h->ncell;
    if (h->th_stepped) {
        // the buoyancy field keeps the last step's values until the next
        // thermal step (thermalUpload does not touch it)
        CUDA_TRY(cudaMemcpyAsync(h->T_buoy, h->T, n * 4, cudaMemcpyDeviceToDevice, h->stream));
        h->th_buoy_mode = 2;
    }
    std::vector<float> t(T, T + n);
    double sum = 0.0;
    for (int z = 0; z < h->nz; ++z)
        for (int y = h->ylo; y <= h->yhi; ++y)
            for (int x = 0; x < h->nx; ++x)
                if (!h->mask[cidx(h, x, y, z)]) sum += t[cidx(h, x, y, z)];
    const long nn = (long)h->nx * h->nz * (h->yhi - h->ylo + 1);
    h->stats.mean_t = nn > 0 ? (float)(sum / (double)nn) : 0.5f;
    h->ctl_host->mean_t = h->stats.mean_t;
    CUDA_TRY(cudaMemcpy(&h->ctl->mean_t, &h->stats.mean_t, sizeof(float), cudaMemcpyHostToDevice));
    return upload_T(h, t);
}

extern "C" int aeros_lbm_thermal_read(aeros_lbm* h, float* T, float* buoyancy) {
    if (!h) return set_error(AEROS_ERR_INVALID, "handle is NULL");
    if (!h->th_on) return set_error(AEROS_ERR_STATE, "thermal lattice not initialised");
    if (int rc = finish_batch(h)) return rc;
    const size_t n = (size_t)h->ncell;
    std::vector<float> t(n);
    CUDA_TRY(cudaMemcpy(t.data(), h->T, n * 4, cudaMemcpyDeviceToHost));
    if (T) memcpy(T, t.data(), n * 4);
    if (buoyancy) {
        std::vector<float> tb;
        if (h->th_buoy_mode == 2) {
            tb.resize(n);
            CUDA_TRY(cudaMemcpy(tb.data(), h->T_buoy, n * 4, cudaMemcpyDeviceToHost));
        }
        const float tref = 0.5f * (h->tp.hot_temp + h->tp.cold_temp);
        for (size_t c = 0; c < n; ++c) {
            if (h->mask[c] || h->th_buoy_mode == 1) buoyancy[c] = 0.0f;
            else buoyancy[c] = h->glb * ((h->th_buoy_mode == 2 ? tb[c] : t[c]) - tref);
        }
    }
    return AEROS_OK;
}

// ---------------------------------------------------------------------------
// forces
// ---------------------------------------------------------------------------
extern "C" int aeros_lbm_cv_force_box(aeros_lbm* h, const int32_t box[6], double out[3]) {
    if (!h || !box || !out) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (box[0] < 0 || box[1] >= h->nx || box[0] > box[1] || box[2] < 0 || box[3] >= h->ny || box[2] > box[3] ||
        box[4] < 0 || box[5] >= h->nz || box[4] > box[5])
        return set_error(AEROS_ERR_INVALID, "box [%d,%d]x[%d,%d]x[%d,%d] outside the grid", box[0], box[1], box[2],
                         box[3], box[4], box[5]);
    ForceArgs a;
    a.nx = h->nx; a.ny = h->ny; a.nz = h->nz;
    a.desc = h->desc;
    a.rho = h->rho;
    a.u = h->u[h->ubuf];
    for (int k = 0; k < 6; ++k) a.box[k] = box[k];
    a.partials = h->force_partials;
    a.out = h->force_out;
    a.counter = h->force_counter;
    // Queued behind steps still in flight (stream order), so that one wait
    // covers the steps, their statistics and the force; the destination is
    // pinned (a plain DMA).
    const bool pending = h->stats_dirty;
    auto enqueue = [&]() -> cudaError_t {
        a.u = h->u[h->ubuf];
        cudaError_t e = launch_cv_force(a, cv_force_blocks(a.box, h->max_grid), h->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h->force_host, h->force_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
        return e;
    };
    CUDA_TRY(enqueue());
    if (int rc = finish_batch(h)) return rc;   // waits for the stream when steps were pending
    if (pending && h->last_diverged) CUDA_TRY(enqueue());   // the guard reset the state: take the force again
    if (!pending || h->last_diverged) CUDA_TRY(cudaStreamSynchronize(h->stream));
    const double* sums = h->force_host;
    // force on the body = minus the momentum flux through the box (lbm.cpp:2231)
    out[0] = -sums[0]; out[1] = -sums[1]; out[2] = -sums[2];
    return AEROS_OK;
}

extern "C" int aeros_lbm_cv_force(aeros_lbm* h, float half_x, float half_y, float half_z, double out[3]) {
    if (!h || !out) return set_error(AEROS_ERR_INVALID, "NULL argument");
    // box centred on the domain centre, lbm.cpp:2188-2197
    auto clamp_side = [](int v, int n) { return v < 1 ? 1 : (v > n - 2 ? n - 2 : v); };
    const int cx = (int)(h->nx * 0.5f), cy = (int)(h->ny * 0.5f), cz = (int)(h->nz * 0.5f);
    const int hx = std::max(2, (int)(h->nx * half_x));
    const int hy = std::max(2, (int)(h->ny * half_y));
    const int hz = std::max(2, (int)(h->nz * half_z));
    const int32_t box[6] = {clamp_side(cx - hx, h->nx), clamp_side(cx + hx, h->nx), clamp_side(cy - hy, h->ny),
                            clamp_side(cy + hy, h->ny), clamp_side(cz - hz, h->nz), clamp_side(cz + hz, h->nz)};
    return aeros_lbm_cv_force_box(h, box, out);
}

namespace {
// lbmEquilibriumMoments, aeros/src/lbm.cpp:249-267: one thread per state.
__global__ void k_eq_moments(const float* st, long long n, float* out, uint8_t* ok) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float rho = st[4 * i], ux = st[4 * i + 1], uy = st[4 * i + 2], uz = st[4 * i + 3];
        float m = 0.0f, px = 0.0f, py = 0.0f, pz = 0.0f;
        bool good = isfinite(rho) && isfinite(ux) && isfinite(uy) && isfinite(uz);
        if (good) {
            const float usqr = ux * ux + uy * uy + uz * uz;
            for (int q = 0; q < 19 && good; ++q) {
                const float feq = aeros::eq_checked(q, rho, ux, uy, uz, usqr);
                good = isfinite(feq);
                m += feq;
                px += feq * (float)aeros::cx19(q);
                py += feq * (float)aeros::cy19(q);
                pz += feq * (float)aeros::cz19(q);
            }
        }
        out[4 * i] = good ? m : 0.0f;
        out[4 * i + 1] = good ? px : 0.0f;
        out[4 * i + 2] = good ? py : 0.0f;
        out[4 * i + 3] = good ? pz : 0.0f;
        ok[i] = good ? 1 : 0;
    }
}
}  // namespace

extern "C" int aeros_equilibrium_moments(const float* states, int64_t n, float* out, uint8_t* ok) {
    if (n < 0 || n > ((int64_t)1 << 24)) return set_error(AEROS_ERR_INVALID, "%lld states", (long long)n);
    if (n > 0 && (!states || !out || !ok)) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (n == 0) return AEROS_OK;
    const size_t fb = (size_t)n * 4 * sizeof(float);
    char* d = nullptr;
    cudaStream_t s = nullptr;
    CUDA_TRY(cudaMallocAsync((void**)&d, 2 * fb + (size_t)n, s));
    float* dst = (float*)d;
    float* dout = (float*)(d + fb);
    uint8_t* dok = (uint8_t*)(d + 2 * fb);
    cudaError_t e = cudaMemcpyAsync(dst, states, fb, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
        k_eq_moments<<<blocks, 256, 0, s>>>(dst, n, dout, dok);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, fb, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ok, dok, (size_t)n, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(AEROS_ERR_CUDA, "equilibrium moments: %s", cudaGetErrorString(e));
    return AEROS_OK;
}

extern "C" int aeros_lbm_projected_area(aeros_lbm* h, int axis, double* area) {
    if (!h || !area) return set_error(AEROS_ERR_INVALID, "NULL argument");
    if (axis < 0 || axis > 2) return set_error(AEROS_ERR_INVALID, "axis %d", axis);
    if (int rc = finish_batch(h)) return rc;
    CUDA_TRY(launch_projected_area(h->nx, h->ny, h->nz, h->desc, axis, h->area_count, h->stream));
    unsigned long long cnt = 0;
    CUDA_TRY(cudaMemcpyAsync(&cnt, h->area_count, sizeof(cnt), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    *area = (double)cnt;
    return AEROS_OK;
}

// ---------------------------------------------------------------------------
// voxelizer
// ---------------------------------------------------------------------------
namespace aeros {
int voxelize_impl(const float* tris, int64_t ntri, const aeros_voxel_grid* g, uint8_t* d_mask, cudaStream_t s,
                  char* err, size_t errn);
int voxelize_noalloc_impl(const float* tris, int64_t ntri, const aeros_voxel_grid* g, uint8_t* d_mask,
                          cudaStream_t s, char* err, size_t errn);
}

static int check_grid(const float* tris, int64_t ntri, const aeros_voxel_grid* g) {
    if (!g) return set_error(AEROS_ERR_INVALID, "grid is NULL");
    if (ntri < 0 || (ntri > 0 && !tris)) return set_error(AEROS_ERR_INVALID, "triangles");
    if (ntri > (1ll << 31) / 9) return set_error(AEROS_ERR_INVALID, "%lld triangles exceed the limit", (long long)ntri);
    if (g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || (long long)g->nx * g->ny * g->nz > (1ll << 31))
        return set_error(AEROS_ERR_INVALID, "grid %dx%dx%d", g->nx, g->ny, g->nz);
    return AEROS_OK;
}

extern "C" int aeros_voxelize_device(const float* tris, int64_t ntri, const aeros_voxel_grid* g, uint8_t* d_mask) {
    if (int rc = check_grid(tris, ntri, g)) return rc;
    if (!d_mask) return set_error(AEROS_ERR_INVALID, "mask is NULL");
    char err[512] = {0};
    const int rc = voxelize_impl(tris, ntri, g, d_mask, nullptr, err, sizeof(err));
    if (rc) return set_error(rc, "%s", err);
    return AEROS_OK;
}

// Fixed-scratch variant of aeros_voxelize_device for callers that cannot
// allocate device memory (see voxelize_noalloc_impl in voxel.cu).
extern "C" int aeros_voxelize_device_noalloc(const float* tris, int64_t ntri, const aeros_voxel_grid* g,
                                             uint8_t* d_mask, void* stream) {
    if (int rc = check_grid(tris, ntri, g)) return rc;
    if (!d_mask) return set_error(AEROS_ERR_INVALID, "mask is NULL");
    char err[512] = {0};
    const int rc = voxelize_noalloc_impl(tris, ntri, g, d_mask, (cudaStream_t)stream, err, sizeof(err));
    if (rc) return set_error(rc, "%s", err);
    return AEROS_OK;
}

extern "C" int aeros_voxelize(const float* tris, int64_t ntri, const aeros_voxel_grid* g, uint8_t* mask_out) {
    if (int rc = check_grid(tris, ntri, g)) return rc;
    if (!mask_out) return set_error(AEROS_ERR_INVALID, "mask is NULL");
    const size_t total = (size_t)g->nx * g->ny * g->nz;
    uint8_t* d = nullptr;
    if (cudaMallocAsync((void**)&d, total, nullptr) != cudaSuccess) return set_error(AEROS_ERR_ALLOC, "mask buffer");
    char err[512] = {0};
    int rc = voxelize_impl(tris, ntri, g, d, nullptr, err, sizeof(err));
    if (rc == AEROS_OK) {
        cudaError_t e = cudaMemcpyAsync(mask_out, d, total, cudaMemcpyDeviceToHost, nullptr);
        if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
        if (e != cudaSuccess) snprintf(err, sizeof(err), "mask copy: %s", cudaGetErrorString(e)), rc = AEROS_ERR_CUDA;
    }
    cudaFreeAsync(d, nullptr);
    if (rc) return set_error(rc, "%s", err);
    return AEROS_OK;
}

// voxelPlan, aeros/src/voxel_grid.cpp:172-215 (224 bytes per cell, res 8..512)
extern "C" int aeros_voxel_plan(const float size[3], int res, uint64_t budget, aeros_voxel_plan_t* p) {
    if (!size || !p) return set_error(AEROS_ERR_INVALID, "NULL argument");
    memset(p, 0, sizeof(*p));
    p->requested_res = res;
    const int r = res < 8 ? 8 : (res > 512 ? 512 : res);
    float sx = size[0], sy = size[1], sz = size[2];
    if (!(sx > 1e-6f) || !std::isfinite(sx)) sx = 1.0f;
    if (!(sy > 1e-6f) || !std::isfinite(sy)) sy = 1.0f;
    if (!(sz > 1e-6f) || !std::isfinite(sz)) sz = 1.0f;
    const float m = std::max(sx, std::max(sy, sz));
    auto dims = [&](int rr, int& nx, int& ny, int& nz) {
        nx = rr;
        ny = (int)std::floor(rr * sy / m);
        if (ny < 4) ny = 4;
        nz = (int)std::floor(rr * sz / m);
        if (nz < 4) nz = 4;
    };
    int nx, ny, nz;
    dims(r, nx, ny, nz);
    p->nx = nx; p->ny = ny; p->nz = nz;
    p->cells = (int64_t)nx * ny * nz;
    p->bytes = (uint64_t)p->cells * 224ull;
    p->fits = (budget == 0) || (p->bytes <= budget);
    if (!p->fits && budget > 0) {
        const double scale = std::cbrt((double)budget / (double)p->bytes) * 0.95;
        int cand = (int)(r * scale);
        for (int guard = 0; guard < 64 && cand >= 8; ++guard, --cand) {
            int a, b, c;
            dims(cand, a, b, c);
            if ((uint64_t)a * b * c * 224ull <= budget) { p->suggested_res = cand; break; }
        }
        if (p->suggested_res < 8) p->suggested_res = 0;
    }
    return AEROS_OK;
}
