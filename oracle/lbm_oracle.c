/*
 * lbm_oracle.c — CPU restatement of the reference D3Q19/D3Q7 solver step.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): loaded by tests/, smoke() and the
 * CPU-baseline leg of bench.py; never by the product path.
 *
 * Every function follows the reference file:line cited beside it and keeps
 * its floating-point expression trees (same operand order, no contraction:
 * built with -ffp-contract=off), so the float build is bitwise equal to the
 * reference compiled without FMA. Built with AO_REAL=double it is the FP64
 * run of the same algorithm.
 */
#include "aeros_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef AO_REAL
#define AO_REAL float
#endif
typedef AO_REAL real;

#if defined(AO_IS_DOUBLE) && AO_IS_DOUBLE
#define K(x) (x)
#define RSQRT(x) sqrt(x)
#define RABS(x) fabs(x)
#define RFLOOR(x) floor(x)
#else
#define K(x) (x##f)
#define RSQRT(x) sqrtf(x)
#define RABS(x) fabsf(x)
#define RFLOOR(x) floorf(x)
#endif

#define Q19 19
#define Q7 7

/* D3Q19 tables: aeros/src/lbm.cpp:92-109 (same ordering). */
static const int C19[Q19][3] = {
    {0, 0, 0},
    {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
    {1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0},
    {1, 0, 1}, {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
    {0, 1, 1}, {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
static const int OPP19[Q19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
static real W19[Q19];
/* Van Driest factor 1 - exp(-d/2), d = 0..6: aeros/src/lbm.cpp:112-120. */
static const real VAN_DRIEST[7] = {K(0.0), K(0.3934693403), K(0.6321205588), K(0.7768698399),
                                   K(0.8646647168), K(0.9179150014), K(0.9502129316)};
/* D3Q7 tables: aeros/src/thermal_lbm.cpp:31-40. */
static const int C7[Q7][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
static const int OPP7[Q7] = {0, 2, 1, 4, 3, 6, 5};
static real W7[Q7];

static void init_tables(void) {
    static int done = 0;
    if (done) return;
    W19[0] = K(1.0) / K(3.0);
    for (int q = 1; q <= 6; ++q) W19[q] = K(1.0) / K(18.0);
    for (int q = 7; q < Q19; ++q) W19[q] = K(1.0) / K(36.0);
    W7[0] = K(0.25);
    for (int q = 1; q < Q7; ++q) W7[q] = K(0.125);
    done = 1;
}

struct ao_lbm {
    aeros_lbm_params p;
    int nx, ny, nz, total;
    uint8_t* mask;      /* AEROS_CELL_* */
    uint8_t* wall;      /* lbmWallDist, saturating at 255 */
    int fluid_cells;    /* sFluidCells */
    real *f, *fn;       /* AoS [cell*19+q] */
    real *rho, *ux, *uy, *uz, *strain, *tke;
    /* stats of the last step */
    int64_t step;
    real avg_rho, avg_ke, avg_tke, max_u, convergence, prev_kinetic;
    int converged, diverged;
    double sum_rho, sum_ke, sum_tke;
    int64_t neg, bad, rho_out, rho_nonfin, ulim, nan_count;
    /* thermal */
    int th_on;
    aeros_thermal_params tp;
    real *g, *gn, *T, *buoy;
    int ylo, yhi;
    real H, tau_t, alpha, glb, nusselt, mean_t;
    /* readback / post-processing */
    real *uxw, *uyw, *uzw, *pres, *vort, *qc, *prev_rho;
    int64_t prev_step;
    real prev_maxu;
};

static inline int ao_idx(const ao_lbm* s, int x, int y, int z) { return (z * s->ny + y) * s->nx + x; }
static inline int is_wall(const ao_lbm* s, int c) { return s->mask[c] != AEROS_CELL_FLUID; }

/* equilibriumKernel, aeros/src/lbm.cpp:141-144. */
static inline real eq_kernel(int q, real rho, real ux, real uy, real uz, real usqr) {
    const real cu = (real)C19[q][0] * ux + (real)C19[q][1] * uy + (real)C19[q][2] * uz;
    return W19[q] * rho * (K(1.0) + cu * K(3.0) + cu * cu * K(4.5) - usqr * K(1.5));
}

/* computeEquilibriumFast, aeros/src/lbm.cpp:146-184. */
static real eq_checked(int q, real rho, real ux, real uy, real uz, real usqr) {
    if (!isfinite(rho)) rho = K(1.0);
    if (usqr > K(0.09)) {
        real scale = RSQRT(K(0.09) / usqr);
        ux *= scale; uy *= scale; uz *= scale;
        usqr = ux * ux + uy * uy + uz * uz;
    }
    real cu = (real)C19[q][0] * ux + (real)C19[q][1] * uy + (real)C19[q][2] * uz;
    if (!isfinite(cu)) cu = K(0.0);
    real feq = W19[q] * rho * (K(1.0) + cu * K(3.0) + cu * cu * K(4.5) - usqr * K(1.5));
    if (!isfinite(feq)) feq = W19[q] * rho;
    return feq;
}

int ao_real_bytes(void) { return (int)sizeof(real); }

int ao_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* lbmEquilibriumMoments, aeros/src/lbm.cpp:307-327. */
int ao_equilibrium_moments(float rho_f, float ux_f, float uy_f, float uz_f,
                           float* sum, float* mx, float* my, float* mz) {
    init_tables();
    if (!sum || !mx || !my || !mz) return 0;
    if (!isfinite(rho_f) || !isfinite(ux_f) || !isfinite(uy_f) || !isfinite(uz_f)) return 0;
    real rho = rho_f, ux = ux_f, uy = uy_f, uz = uz_f;
    real usqr = ux * ux + uy * uy + uz * uz;
    real m = 0, px = 0, py = 0, pz = 0;
    for (int q = 0; q < Q19; ++q) {
        real feq = eq_checked(q, rho, ux, uy, uz, usqr);
        if (!isfinite(feq)) return 0;
        m += feq;
        px += feq * C19[q][0];
        py += feq * C19[q][1];
        pz += feq * C19[q][2];
    }
    *sum = (float)m; *mx = (float)px; *my = (float)py; *mz = (float)pz;
    return 1;
}

/* Equilibrium of one cell from (rho, u) with the init limiter:
 * aeros/src/lbm.cpp:720-737 (and the reset loop :1583-1593). */
static void set_cell_eq(ao_lbm* s, int c, real rho, real ux, real uy, real uz) {
    real usqr = ux * ux + uy * uy + uz * uz;
    if (usqr > K(0.09)) {
        real scale = RSQRT(K(0.09) / usqr);
        ux *= scale; uy *= scale; uz *= scale;
        usqr = ux * ux + uy * uy + uz * uz;
    }
    for (int q = 0; q < Q19; ++q) s->f[(size_t)c * Q19 + q] = eq_checked(q, rho, ux, uy, uz, usqr);
}

/* Wall-distance chamfer, aeros/src/lbm.cpp:647-675. */
static void wall_distance(ao_lbm* s) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    uint8_t* d = s->wall;
    for (int c = 0; c < s->total; ++c) d[c] = is_wall(s, c) ? 0 : 255;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            const int row = (z * ny + y) * nx;
            for (int x = 0; x < nx; ++x) {
                int v = d[row + x];
                if (v == 0) continue;
                if (x > 0 && d[row + x - 1] + 1 < v) v = d[row + x - 1] + 1;
                if (y > 0 && d[row - nx + x] + 1 < v) v = d[row - nx + x] + 1;
                if (z > 0 && d[row - nx * ny + x] + 1 < v) v = d[row - nx * ny + x] + 1;
                d[row + x] = (uint8_t)v;
            }
        }
    for (int z = nz - 1; z >= 0; --z)
        for (int y = ny - 1; y >= 0; --y) {
            const int row = (z * ny + y) * nx;
            for (int x = nx - 1; x >= 0; --x) {
                int v = d[row + x];
                if (v == 0) continue;
                if (x < nx - 1 && d[row + x + 1] + 1 < v) v = d[row + x + 1] + 1;
                if (y < ny - 1 && d[row + nx + x] + 1 < v) v = d[row + nx + x] + 1;
                if (z < nz - 1 && d[row + nx * ny + x] + 1 < v) v = d[row + nx * ny + x] + 1;
                d[row + x] = (uint8_t)v;
            }
        }
}

ao_lbm* ao_lbm_create(const aeros_lbm_params* p, const uint8_t* mask) {
    init_tables();
    if (!p || !mask || p->nx < 4 || p->ny < 4 || p->nz < 4) return NULL;
    ao_lbm* s = (ao_lbm*)calloc(1, sizeof(ao_lbm));
    if (!s) return NULL;
    s->p = *p;
    s->nx = p->nx; s->ny = p->ny; s->nz = p->nz;
    s->total = s->nx * s->ny * s->nz;
    const size_t n = (size_t)s->total;
    s->mask = (uint8_t*)malloc(n);
    s->wall = (uint8_t*)malloc(n);
    s->f = (real*)calloc(n * Q19, sizeof(real));
    s->fn = (real*)calloc(n * Q19, sizeof(real));
    s->rho = (real*)malloc(n * sizeof(real));
    s->ux = (real*)calloc(n, sizeof(real));
    s->uy = (real*)calloc(n, sizeof(real));
    s->uz = (real*)calloc(n, sizeof(real));
    s->strain = (real*)calloc(n, sizeof(real));
    s->tke = (real*)calloc(n, sizeof(real));
    if (!s->mask || !s->wall || !s->f || !s->fn || !s->rho || !s->ux || !s->uy || !s->uz ||
        !s->strain || !s->tke) {
        ao_lbm_destroy(s);
        return NULL;
    }
    memcpy(s->mask, mask, n);
    for (size_t c = 0; c < n; ++c) s->rho[c] = K(1.0);
    wall_distance(s);
    s->fluid_cells = 0;
    for (int c = 0; c < s->total; ++c)
        if (!is_wall(s, c)) ++s->fluid_cells;
    if (s->fluid_cells < 1) s->fluid_cells = 1;
    for (int c = 0; c < s->total; ++c) {
        if (is_wall(s, c)) set_cell_eq(s, c, K(1.0), K(0.0), K(0.0), K(0.0));
        else set_cell_eq(s, c, K(1.0), (real)p->u_init[0], (real)p->u_init[1], (real)p->u_init[2]);
    }
    s->avg_rho = K(1.0);
    return s;
}

void ao_lbm_destroy(ao_lbm* s) {
    if (!s) return;
    free(s->mask); free(s->wall); free(s->f); free(s->fn);
    free(s->uxw); free(s->uyw); free(s->uzw); free(s->pres); free(s->vort); free(s->qc); free(s->prev_rho);
    free(s->rho); free(s->ux); free(s->uy); free(s->uz); free(s->strain); free(s->tke);
    free(s->g); free(s->gn); free(s->T); free(s->buoy);
    free(s);
}

/* ------------------------------------------------------------------------ */
/* Thermal lattice: aeros/src/thermal_lbm.cpp                                */
/* ------------------------------------------------------------------------ */

/* geq, thermal_lbm.cpp:53-56. */
static inline real th_geq(int i, real T, real ux, real uy, real uz) {
    const real cu = (real)C7[i][0] * ux + (real)C7[i][1] * uy + (real)C7[i][2] * uz;
    return W7[i] * T * (K(1.0) + K(4.0) * cu);
}

/* wallTemp, thermal_lbm.cpp:60-65. */
static inline int th_wall_temp(const ao_lbm* s, int y, real* Tw) {
    if (!s->tp.fixed_wall_temps) return 0;
    if (y <= 0) { *Tw = (real)s->tp.hot_temp; return 1; }
    if (y >= s->ny - 1) { *Tw = (real)s->tp.cold_temp; return 1; }
    return 0;
}

/* computeDiagnostics, thermal_lbm.cpp:67-80. */
static void th_diagnostics(ao_lbm* s) {
    double sum = 0.0;
    for (int z = 0; z < s->nz; ++z)
        for (int y = s->ylo; y <= s->yhi; ++y)
            for (int x = 0; x < s->nx; ++x) {
                const int c = ao_idx(s, x, y, z);
                if (is_wall(s, c)) continue;
                sum += s->T[c];
            }
    const long n = (long)s->nx * (long)s->nz * (long)(s->yhi - s->ylo + 1);
    s->mean_t = n > 0 ? (real)(sum / (double)n) : K(0.5);
}

static void th_populations_from_T(ao_lbm* s) {
    for (int c = 0; c < s->total; ++c)
        for (int i = 0; i < Q7; ++i) s->g[(size_t)c * Q7 + i] = th_geq(i, s->T[c], 0, 0, 0);
}

/* thermalResetField, thermal_lbm.cpp:154-185. */
static void th_reset_field(ao_lbm* s) {
    const real Th = (real)s->tp.hot_temp, Tc = (real)s->tp.cold_temp;
    const real dT = Th - Tc;
    const real amp = (real)s->tp.perturbation * dT;
    for (int z = 0; z < s->nz; ++z)
        for (int y = 0; y < s->ny; ++y)
            for (int x = 0; x < s->nx; ++x) {
                const int c = ao_idx(s, x, y, z);
                real T;
                if (is_wall(s, c)) {
                    real Tw;
                    T = th_wall_temp(s, y, &Tw) ? Tw : K(0.5) * (Th + Tc);
                } else {
                    real hm1 = s->H - K(1.0);
                    const real sy = (real)(y - s->ylo) / (hm1 > K(1.0) ? hm1 : K(1.0));
                    T = Th + (Tc - Th) * sy;
                    const real px = K(6.2831853) * (real)x / (real)s->nx;
                    const real py = K(3.1415926) * sy;
#if defined(AO_IS_DOUBLE) && AO_IS_DOUBLE
                    T += amp * cos(px) * sin(py);
#else
                    T += amp * cosf(px) * sinf(py);
#endif
                }
                s->T[c] = T;
            }
    th_populations_from_T(s);
    th_diagnostics(s);
}

int ao_thermal_init(ao_lbm* s, const aeros_thermal_params* tp) {
    if (!s || !tp) return -1;
    if (!tp->enabled) { s->th_on = 0; return 0; }
    if (s->nx < 4 || s->ny < 4 || s->nz < 1) return -1;
    s->tp = *tp;
    real nu = (real)tp->nu_lb;
    if (!isfinite(nu) || nu <= K(0.0)) nu = K(0.05);
    /* fluid rows by mask, thermal_lbm.cpp:96-105 */
    s->ylo = -1; s->yhi = -1;
    for (int y = 0; y < s->ny; ++y) {
        int fluid = 0;
        for (int z = 0; z < s->nz && !fluid; ++z)
            for (int x = 0; x < s->nx && !fluid; ++x)
                if (!is_wall(s, ao_idx(s, x, y, z))) fluid = 1;
        if (fluid) { if (s->ylo < 0) s->ylo = y; s->yhi = y; }
    }
    if (s->ylo < 0 || s->yhi <= s->ylo) return -1;
    s->H = (real)(s->yhi - s->ylo + 1);
    real pr = (real)tp->prandtl;
    if (pr < K(0.05)) pr = K(0.05);
    s->alpha = nu / pr;
    s->tau_t = K(0.5) + s->alpha / K(0.25);
    if (!isfinite(s->tau_t) || s->tau_t < K(0.505)) s->tau_t = K(0.505);
    if (s->tau_t > K(1.5)) {
        s->tau_t = K(1.5);
        s->alpha = K(0.25) * (s->tau_t - K(0.5));
    }
    const real dT = (real)tp->hot_temp - (real)tp->cold_temp;
    real adT = RABS(dT);
    if (adT < K(1e-6)) adT = K(1e-6);
    s->glb = (real)tp->rayleigh * nu * s->alpha / (adT * s->H * s->H * s->H);
    const size_t n = (size_t)s->total;
    free(s->g); free(s->gn); free(s->T); free(s->buoy);
    s->g = (real*)calloc(n * Q7, sizeof(real));
    s->gn = (real*)calloc(n * Q7, sizeof(real));
    s->T = (real*)malloc(n * sizeof(real));
    s->buoy = (real*)calloc(n, sizeof(real));
    if (!s->g || !s->gn || !s->T || !s->buoy) return -1;
    s->nusselt = K(0.0);
    th_reset_field(s);
    s->th_on = 1;
    return 0;
}

/* thermalUpload, thermal_lbm.cpp:187-197. */
int ao_thermal_upload(ao_lbm* s, const float* T) {
    if (!s || !s->th_on || !T) return -1;
    for (int c = 0; c < s->total; ++c) s->T[c] = (real)T[c];
    th_populations_from_T(s);
    th_diagnostics(s);
    return 0;
}

/* thermalStep, thermal_lbm.cpp:199-355 (fixed-wall fast-path split kept: the
 * interior range excludes the rows next to fixed-temperature walls). */
static void th_step(ao_lbm* s) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const real invTau = K(1.0) / s->tau_t;
    const int fixed = s->tp.fixed_wall_temps;
    const int yA = fixed ? 2 : 1, yB = fixed ? ny - 2 : ny - 1;
    int off[Q7];
    for (int i = 0; i < Q7; ++i) off[i] = -(C7[i][2] * ny * nx) - C7[i][1] * nx - C7[i][0];
    real* g = s->g;
    real* gn = s->gn;
#pragma omp parallel for
    for (int z = 1; z < nz - 1; ++z)
        for (int y = yA; y < yB; ++y)
            for (int x = 1; x < nx - 1; ++x) {
                const int c = ao_idx(s, x, y, z);
                if (is_wall(s, c)) {
                    for (int i = 0; i < Q7; ++i) gn[(size_t)c * Q7 + i] = g[(size_t)c * Q7 + i];
                    continue;
                }
                for (int i = 0; i < Q7; ++i) {
                    const int src = c + off[i];
                    gn[(size_t)c * Q7 + i] = is_wall(s, src) ? g[(size_t)c * Q7 + OPP7[i]] : g[(size_t)src * Q7 + i];
                }
            }
#pragma omp parallel for
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            const int yEdge = (y < yA || y >= yB);
            const int zEdge = (z == 0 || z == nz - 1);
            for (int x = 0; x < nx; ++x) {
                if (!yEdge && !zEdge && x > 0 && x < nx - 1) continue;
                const int c = ao_idx(s, x, y, z);
                if (is_wall(s, c)) {
                    for (int i = 0; i < Q7; ++i) gn[(size_t)c * Q7 + i] = g[(size_t)c * Q7 + i];
                    continue;
                }
                for (int i = 0; i < Q7; ++i) {
                    int sx = x - C7[i][0], sy = y - C7[i][1], sz = z - C7[i][2];
                    const int outX = (sx < 0 || sx >= nx), outY = (sy < 0 || sy >= ny), outZ = (sz < 0 || sz >= nz);
                    if (outX) sx = (sx < 0) ? nx - 1 : 0;
                    if (outZ) sz = (sz < 0) ? nz - 1 : 0;
                    real Tw = K(0.0);
                    int dirichlet = 0, bounce = 0;
                    if (outY) {
                        bounce = 1;
                        dirichlet = th_wall_temp(s, sy < 0 ? 0 : ny - 1, &Tw);
                    } else if (is_wall(s, ao_idx(s, sx, sy, sz))) {
                        bounce = 1;
                        dirichlet = th_wall_temp(s, sy, &Tw);
                    }
                    if (bounce) {
                        const real gOpp = g[(size_t)c * Q7 + OPP7[i]];
                        gn[(size_t)c * Q7 + i] = dirichlet ? (-gOpp + K(2.0) * W7[i] * Tw) : gOpp;
                    } else {
                        gn[(size_t)c * Q7 + i] = g[(size_t)ao_idx(s, sx, sy, sz) * Q7 + i];
                    }
                }
            }
        }
    const real Th = (real)s->tp.hot_temp, Tc = (real)s->tp.cold_temp;
    const real Tref = K(0.5) * (Th + Tc);
    const real gLb = s->glb;
#pragma omp parallel for
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int c = ao_idx(s, x, y, z);
                if (is_wall(s, c)) { s->buoy[c] = K(0.0); continue; }
                const real vx = s->ux[c], vy = s->uy[c], vz = s->uz[c];
                real gi[Q7];
                real T = K(0.0);
                for (int i = 0; i < Q7; ++i) { gi[i] = gn[(size_t)c * Q7 + i]; T += gi[i]; }
                if (!isfinite(T)) T = Tref;
                {
                    real lo = Tc - K(1.0), hi = Th + K(1.0);
                    real m = (lo < T) ? T : lo;      /* std::max(lo, T) */
                    T = (m < hi) ? m : hi;           /* std::min(hi, m) */
                }
                for (int i = 0; i < Q7; ++i) {
                    const real eq = th_geq(i, T, vx, vy, vz);
                    gn[(size_t)c * Q7 + i] = gi[i] - (gi[i] - eq) * invTau;
                }
                s->T[c] = T;
                s->buoy[c] = gLb * (T - Tref);
            }
    /* Nusselt at the bottom wall, thermal_lbm.cpp:338-351 */
    double qSum = 0.0;
    long qN = 0;
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nx; ++x) {
            const int c = ao_idx(s, x, s->ylo, z);
            if (is_wall(s, c)) continue;
            qSum += (double)(Th - s->T[c]) / 0.5; /* float subtraction, as the reference */
            ++qN;
        }
    if (qN > 0) {
        real dT = RABS(Th - Tc);
        if (dT < K(1e-6)) dT = K(1e-6);
        s->nusselt = (real)(qSum / (double)qN) * s->H / dT;
    }
    th_diagnostics(s);
    real* t = s->g; s->g = s->gn; s->gn = t;
}

/* ------------------------------------------------------------------------ */
/* D3Q19 step: aeros/src/lbm.cpp:907-1600                                    */
/* ------------------------------------------------------------------------ */

/* Flow-plane flags, aeros/src/lbm.cpp:1091-1101. */
static inline void flow_planes(const ao_lbm* s, int x, int y, int z, int* in, int* out) {
    const int ax = s->p.flow_axis, sg = s->p.flow_sign;
    const int v = ax == 0 ? x : (ax == 1 ? y : z);
    const int n = ax == 0 ? s->nx : (ax == 1 ? s->ny : s->nz);
    *in = (sg > 0) ? (v == 0) : (v == n - 1);
    *out = (sg > 0) ? (v == n - 1) : (v == 0);
}

/* Source resolution of the stream for one (dest, q), the shell rules of
 * aeros/src/lbm.cpp:1376-1406 plus the two new wall modes.
 * Writes the pulled value. */
static real stream_pull(const ao_lbm* s, const real* f, int x, int y, int z, int q) {
    const int n[3] = {s->nx, s->ny, s->nz};
    const int dc = ao_idx(s, x, y, z);
    int src[3] = {x - C19[q][0], y - C19[q][1], z - C19[q][2]};
    const int per[3] = {s->p.periodic_x, 0, s->p.periodic_z};
    int outm = 0;
    for (int a = 0; a < 3; ++a) {
        if (per[a]) {
            if (src[a] < 0) src[a] += n[a];
            else if (src[a] >= n[a]) src[a] -= n[a];
        }
        if (src[a] < 0 || src[a] >= n[a]) outm |= 1 << a;
    }
    if (!outm) {
        const int sc = ao_idx(s, src[0], src[1], src[2]);
        return is_wall(s, sc) ? f[(size_t)dc * Q19 + OPP19[q]] : f[(size_t)sc * Q19 + q];
    }
    if (s->p.lateral_bc == AEROS_LATERAL_FREESLIP && !(outm & (1 << s->p.flow_axis))) {
        /* specular reflection off the out-of-domain faces */
        int rs[3], rc[3];
        const int pos[3] = {x, y, z};
        for (int a = 0; a < 3; ++a) {
            const int o = (outm >> a) & 1;
            rs[a] = o ? pos[a] : src[a];
            rc[a] = o ? -C19[q][a] : C19[q][a];
        }
        int rq = 0;
        for (int k = 0; k < Q19; ++k)
            if (C19[k][0] == rc[0] && C19[k][1] == rc[1] && C19[k][2] == rc[2]) { rq = k; break; }
        const int sc = ao_idx(s, rs[0], rs[1], rs[2]);
        if (is_wall(s, sc)) return f[(size_t)dc * Q19 + OPP19[q]];
        return f[(size_t)sc * Q19 + rq];
    }
    return f[(size_t)dc * Q19 + q]; /* copy own post-collision population */
}

void ao_lbm_step(ao_lbm* s, int steps) {
    init_tables();
    const int nx = s->nx, ny = s->ny, nz = s->nz, total = s->total;
    const aeros_lbm_params* P = &s->p;
    real tau0 = (real)P->tau;
    if (!isfinite(tau0) || tau0 < K(0.51)) tau0 = K(0.55);
    if (tau0 > K(1.5)) tau0 = K(1.5);
    const real inUx = (real)P->u_in[0], inUy = (real)P->u_in[1], inUz = (real)P->u_in[2];
    real U0mag = RSQRT(inUx * inUx + inUy * inUy + inUz * inUz);
    if (!isfinite(U0mag) || U0mag < K(1e-6)) U0mag = K(0.08);
    const real velScale = (real)P->vel_scale;
    const real velScale2 = velScale * velScale;
    const int strideY = nx, strideZ = nx * ny;
    real Cs = (real)P->smagorinsky_c;
    if (!isfinite(Cs) || Cs < K(0.0)) Cs = K(0.12);
    if (Cs > K(0.3)) Cs = K(0.3);
    const real Fx0 = (real)P->body_force[0], Fy0 = (real)P->body_force[1], Fz0 = (real)P->body_force[2];
    int hasDiverged = 0;
    s->diverged = 0;

    for (int st = 0; st < steps; ++st) {
        real* f = s->f;
        real* fn = s->fn;
        real maxVel = K(0.0);
        double avgRhoAcc = 0.0, kineticAcc = 0.0, tkeAcc = 0.0;
        int nanCount = 0;
        long long negPops = 0, badPops = 0, rhoOut = 0, rhoNonFin = 0, uLim = 0;

        /* LES pre-pass on previous-step u, lbm.cpp:979-1036 */
        if (P->use_les) {
#pragma omp parallel for
            for (int z = 0; z < nz; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x) {
                        const int c = (z * ny + y) * nx + x;
                        if (is_wall(s, c)) { s->strain[c] = K(0.0); continue; }
                        int lin, lout;
                        flow_planes(s, x, y, z, &lin, &lout);
                        if (lin || lout || !(x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1)) {
                            s->strain[c] = K(0.0);
                            continue;
                        }
                        const int xm = c - 1, xp = c + 1, ym = c - strideY, yp = c + strideY, zm = c - strideZ, zp = c + strideZ;
                        if (s->mask[xm] == AEROS_CELL_SOLID || s->mask[xp] == AEROS_CELL_SOLID ||
                            s->mask[ym] == AEROS_CELL_SOLID || s->mask[yp] == AEROS_CELL_SOLID ||
                            s->mask[zm] == AEROS_CELL_SOLID || s->mask[zp] == AEROS_CELL_SOLID) {
                            s->strain[c] = K(0.0);
                            continue;
                        }
                        const real* ux = s->ux; const real* uy = s->uy; const real* uz = s->uz;
                        real dux_dx = (ux[xp] - ux[xm]) * K(0.5);
                        real duy_dy = (uy[yp] - uy[ym]) * K(0.5);
                        real duz_dz = (uz[zp] - uz[zm]) * K(0.5);
                        real dux_dy = (ux[yp] - ux[ym]) * K(0.5);
                        real dux_dz = (ux[zp] - ux[zm]) * K(0.5);
                        real duy_dx = (uy[xp] - uy[xm]) * K(0.5);
                        real duy_dz = (uy[zp] - uy[zm]) * K(0.5);
                        real duz_dx = (uz[xp] - uz[xm]) * K(0.5);
                        real duz_dy = (uz[yp] - uz[ym]) * K(0.5);
                        real Sxx = dux_dx, Syy = duy_dy, Szz = duz_dz;
                        real Sxy = K(0.5) * (dux_dy + duy_dx);
                        real Sxz = K(0.5) * (dux_dz + duz_dx);
                        real Syz = K(0.5) * (duy_dz + duz_dy);
                        real S2 = Sxx * Sxx + Syy * Syy + Szz * Szz + K(2.0) * (Sxy * Sxy + Sxz * Sxz + Syz * Syz);
                        s->strain[c] = RSQRT(K(2.0) * S2);
                    }
        }

        /* Collision, lbm.cpp:1038-1311 */
#pragma omp parallel for reduction(+ : avgRhoAcc, kineticAcc, tkeAcc, nanCount, negPops, badPops, rhoOut, rhoNonFin, uLim) reduction(max : maxVel)
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) {
                    const int c = (z * ny + y) * nx + x;
                    if (is_wall(s, c)) {
                        s->rho[c] = K(1.0);
                        s->ux[c] = 0; s->uy[c] = 0; s->uz[c] = 0;
                        s->tke[c] = 0; s->strain[c] = 0;
                        continue;
                    }
                    real rho = K(0.0), ux = K(0.0), uy = K(0.0), uz = K(0.0);
                    for (int q = 0; q < Q19; ++q) {
                        real fi = f[(size_t)c * Q19 + q];
                        if (!isfinite(fi)) { fi = W19[q]; nanCount++; badPops++; }
                        if (fi < K(-1.0) || fi > K(10.0)) { fi = W19[q]; badPops++; }
                        rho += fi;
                        ux += fi * (real)C19[q][0];
                        uy += fi * (real)C19[q][1];
                        uz += fi * (real)C19[q][2];
                    }
                    if (!isfinite(rho)) { rhoNonFin++; nanCount++; rho = K(1.0); }
                    else if (rho < K(0.5) || rho > K(1.5)) { rhoOut++; nanCount++; rho = K(1.0); }
                    real invRho = K(1.0) / rho;
                    ux *= invRho; uy *= invRho; uz *= invRho;
                    if (!isfinite(ux)) { ux = 0; uy = 0; uz = 0; nanCount++; }
                    real usqrTmp = ux * ux + uy * uy + uz * uz;
                    if (usqrTmp > K(0.09)) {
                        real scale = RSQRT(K(0.09) / usqrTmp);
                        ux *= scale; uy *= scale; uz *= scale;
                    }
                    int isInlet, isOutlet;
                    flow_planes(s, x, y, z, &isInlet, &isOutlet);
                    if (isInlet && !P->periodic_x) { rho = K(1.0); ux = inUx; uy = inUy; uz = inUz; }

                    real tauEff = tau0;
                    real strainMag = K(0.0);
                    if (P->use_les && !isInlet && !isOutlet) {
                        strainMag = s->strain[c];
                        if (isfinite(strainMag) && strainMag < K(10.0) && strainMag > K(1e-6)) {
                            real cs = Cs;
                            const int wd = (int)s->wall[c];
                            if (wd <= 5) cs *= VAN_DRIEST[wd];
                            const real nu_t = cs * cs * strainMag;
                            tauEff = tau0 + nu_t / (K(1.0) / K(3.0));
                            if (tauEff > K(1.5)) tauEff = K(1.5);
                            if (tauEff < K(0.51)) tauEff = K(0.51);
                        }
                    }
                    real usqr = ux * ux + uy * uy + uz * uz;
                    if (usqr > K(0.09)) {
                        uLim++;
                        real scale = RSQRT(K(0.09) / usqr);
                        ux *= scale; uy *= scale; uz *= scale;
                        usqr = ux * ux + uy * uy + uz * uz;
                    }
                    const real invTau = K(1.0) / tauEff;
                    real Fx = Fx0, Fy = Fy0, Fz = Fz0;
                    if (s->th_on) Fy += s->buoy[c];
                    const int hasForce = (Fx != K(0.0) || Fy != K(0.0) || Fz != K(0.0));
                    real ueX = ux, ueY = uy, ueZ = uz, ueSqr = usqr;
                    if (hasForce) {
                        const real half = K(0.5) / rho;
                        ueX += Fx * half; ueY += Fy * half; ueZ += Fz * half;
                        ueSqr = ueX * ueX + ueY * ueY + ueZ * ueZ;
                    }
                    real sMinus = invTau;
                    if (P->use_trt) {
                        const real m = invTau - K(0.5);
                        const real denom = (RABS(m) > K(1e-6)) ? (K(0.1875) / m + K(0.5)) : K(1.0);
                        sMinus = K(1.0) / (denom > K(0.05) ? denom : K(0.05));
                    }
                    for (int qi = 0; qi < Q19; ++qi) {
                        const int qo = OPP19[qi];
                        if (qo < qi) continue;
                        const real feq = eq_kernel(qi, rho, ueX, ueY, ueZ, ueSqr);
                        real fi = f[(size_t)c * Q19 + qi];
                        if (!isfinite(fi)) fi = feq;
                        real srcI = K(0.0);
                        if (hasForce) {
                            const real cx = (real)C19[qi][0], cy = (real)C19[qi][1], cz = (real)C19[qi][2];
                            const real cu = cx * ueX + cy * ueY + cz * ueZ;
                            srcI = K(3.0) * W19[qi] * ((cx - ueX + K(3.0) * cu * cx) * Fx + (cy - ueY + K(3.0) * cu * cy) * Fy +
                                                      (cz - ueZ + K(3.0) * cu * cz) * Fz);
                        }
                        if (qo == qi) {
                            real fNew = fi - (fi - feq) * invTau + (K(1.0) - K(0.5) * invTau) * srcI;
                            if (!isfinite(fNew)) fNew = feq;
                            if (fNew < K(0.0)) negPops++;
                            f[(size_t)c * Q19 + qi] = fNew;
                            continue;
                        }
                        const real feqO = eq_kernel(qo, rho, ueX, ueY, ueZ, ueSqr);
                        real fo = f[(size_t)c * Q19 + qo];
                        if (!isfinite(fo)) fo = feqO;
                        real srcO = K(0.0);
                        if (hasForce) {
                            const real cx = (real)C19[qo][0], cy = (real)C19[qo][1], cz = (real)C19[qo][2];
                            const real cu = cx * ueX + cy * ueY + cz * ueZ;
                            srcO = K(3.0) * W19[qo] * ((cx - ueX + K(3.0) * cu * cx) * Fx + (cy - ueY + K(3.0) * cu * cy) * Fy +
                                                      (cz - ueZ + K(3.0) * cu * cz) * Fz);
                        }
                        const real srcP = K(0.5) * (srcI + srcO);
                        const real srcM = K(0.5) * (srcI - srcO);
                        const real fp = K(0.5) * (fi + fo), fm = K(0.5) * (fi - fo);
                        const real ep = K(0.5) * (feq + feqO), em = K(0.5) * (feq - feqO);
                        const real fpN = fp - invTau * (fp - ep);
                        const real fmN = fm - sMinus * (fm - em);
                        real newI = fpN + fmN + (K(1.0) - K(0.5) * invTau) * srcP + (K(1.0) - K(0.5) * sMinus) * srcM;
                        real newO = fpN - fmN + (K(1.0) - K(0.5) * invTau) * srcP - (K(1.0) - K(0.5) * sMinus) * srcM;
                        if (!isfinite(newI)) newI = feq;
                        if (!isfinite(newO)) newO = feqO;
                        if (newI < K(0.0)) negPops++;
                        if (newO < K(0.0)) negPops++;
                        f[(size_t)c * Q19 + qi] = newI;
                        f[(size_t)c * Q19 + qo] = newO;
                    }
                    s->rho[c] = rho;
                    if (hasForce) {
                        const real halfInvRho = K(0.5) / rho;
                        s->ux[c] = ux + Fx * halfInvRho;
                        s->uy[c] = uy + Fy * halfInvRho;
                        s->uz[c] = uz + Fz * halfInvRho;
                    } else {
                        s->ux[c] = ux; s->uy[c] = uy; s->uz[c] = uz;
                    }
                    s->strain[c] = strainMag;
                    real tkeLb = (Cs * strainMag) * (Cs * strainMag);
                    real tke = tkeLb * velScale2;
                    if (!isfinite(tke) || tke < K(0.0)) tke = K(0.0);
                    if (tke > K(1.0e6)) tke = K(1.0e6);
                    s->tke[c] = tke;
                    const real velMag = RSQRT(usqr);
                    if (velMag > maxVel) maxVel = velMag;
                    avgRhoAcc += rho;
                    kineticAcc += usqr;
                    tkeAcc += tke;
                }

        s->nan_count = nanCount;
        if (nanCount > total / 10) { hasDiverged = 1; break; }

        /* Stream: interior (lbm.cpp:1331-1360) and shell (:1362-1409) share one
         * source-resolution rule; the interior never meets the shell branches. */
#pragma omp parallel for
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) {
                    const int c = (z * ny + y) * nx + x;
                    if (is_wall(s, c)) continue;
                    for (int q = 0; q < Q19; ++q) fn[(size_t)c * Q19 + q] = stream_pull(s, f, x, y, z, q);
                }

        /* Inlet equilibrium, lbm.cpp:1411-1463 */
        if (!P->periodic_x) {
            const real usq = inUx * inUx + inUy * inUy + inUz * inUz;
            for (int z = 0; z < nz; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x) {
                        int in, out;
                        flow_planes(s, x, y, z, &in, &out);
                        const int c = (z * ny + y) * nx + x;
                        if (!in || is_wall(s, c)) continue;
                        for (int q = 0; q < Q19; ++q) fn[(size_t)c * Q19 + q] = eq_checked(q, K(1.0), inUx, inUy, inUz, usq);
                    }
        }
        /* Outlet: convective (lbm.cpp:1465-1544) or zero-gradient (new). */
        if (!P->periodic_x && (P->convective_outlet || P->outlet_bc == AEROS_OUTLET_ZEROGRAD)) {
            const int ax = P->flow_axis;
            const int na = ax == 0 ? nx : (ax == 1 ? ny : nz);
            const int oc = P->flow_sign > 0 ? na - 1 : 0;
            const int ic = P->flow_sign > 0 ? na - 2 : 1;
            const int ic2 = P->flow_sign > 0 ? na - 3 : 2;
            const int step_a = ax == 0 ? 1 : (ax == 1 ? nx : nx * ny);
            real conv = U0mag * K(0.8);
            if (conv > K(0.5)) conv = K(0.5);
            if (conv < K(0.01)) conv = K(0.08);
            for (int z = 0; z < nz; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x) {
                        const int pos[3] = {x, y, z};
                        if (pos[ax] != oc) continue;
                        const int cOut = (z * ny + y) * nx + x;
                        if (is_wall(s, cOut)) continue;
                        const int cIn = cOut + (ic - oc) * step_a;
                        const int cIn2 = cOut + (ic2 - oc) * step_a;
                        if (P->outlet_bc == AEROS_OUTLET_ZEROGRAD) {
                            /* unknowns (source beyond the outlet) copy the value
                             * the upstream plane pulls: post of the outlet plane
                             * shifted tangentially. */
                            for (int q = 0; q < Q19; ++q) {
                                if (C19[q][ax] * P->flow_sign >= 0) continue;
                                int t[3] = {x - C19[q][0], y - C19[q][1], z - C19[q][2]};
                                t[ax] = oc;
                                const int per[3] = {P->periodic_x, 0, P->periodic_z};
                                const int n3[3] = {nx, ny, nz};
                                for (int a = 0; a < 3; ++a) {
                                    if (a == ax) continue;
                                    if (t[a] < 0 || t[a] >= n3[a]) {
                                        if (per[a]) t[a] = (t[a] + n3[a]) % n3[a];
                                        else t[a] = pos[a];
                                    }
                                }
                                const int tc = ao_idx(s, t[0], t[1], t[2]);
                                fn[(size_t)cOut * Q19 + q] = is_wall(s, tc) ? f[(size_t)cOut * Q19 + q] : f[(size_t)tc * Q19 + q];
                            }
                        } else {
                            for (int q = 0; q < Q19; ++q) {
                                const real fOut = f[(size_t)cOut * Q19 + q];
                                const real fIn = f[(size_t)cIn * Q19 + q];
                                const real fIn2 = (cIn2 >= 0 && cIn2 < total) ? f[(size_t)cIn2 * Q19 + q] : fIn;
                                const real df = fIn - fOut;
                                const real df2 = fIn - fIn2;
                                fn[(size_t)cOut * Q19 + q] = fOut + conv * df + K(0.15) * conv * df2;
                            }
                        }
                    }
        }
        { real* t = s->f; s->f = s->fn; s->fn = t; }
        if (s->th_on) th_step(s);

        s->step++;
        s->sum_rho = avgRhoAcc; s->sum_ke = kineticAcc; s->sum_tke = tkeAcc;
        s->avg_rho = (real)(avgRhoAcc / s->fluid_cells);
        s->avg_ke = (real)(kineticAcc / s->fluid_cells);
        s->max_u = maxVel;
        s->avg_tke = (real)(tkeAcc / s->fluid_cells);
        s->neg = negPops; s->bad = badPops; s->rho_out = rhoOut; s->rho_nonfin = rhoNonFin; s->ulim = uLim;
        s->convergence = RABS(s->avg_ke - s->prev_kinetic);
        s->prev_kinetic = s->avg_ke;
        s->converged = (s->convergence < (real)P->convergence_threshold);
        if (!isfinite(s->avg_rho) || s->avg_rho > K(1.2) || s->avg_rho < K(0.8)) { hasDiverged = 1; break; }
    }
    if (hasDiverged) {
        /* re-equilibration, lbm.cpp:1583-1600 */
        const real usqr = inUx * inUx + inUy * inUy + inUz * inUz;
        for (int c = 0; c < total; ++c) {
            if (is_wall(s, c)) continue;
            for (int q = 0; q < Q19; ++q) s->f[(size_t)c * Q19 + q] = eq_checked(q, K(1.0), inUx, inUy, inUz, usqr);
            s->rho[c] = K(1.0);
            s->ux[c] = inUx; s->uy[c] = inUy; s->uz[c] = inUz;
        }
        s->avg_rho = K(1.0);
        s->avg_ke = usqr;
        s->diverged = 1;
    }
}

void ao_lbm_get_stats(const ao_lbm* s, aeros_lbm_stats* o) {
    memset(o, 0, sizeof(*o));
    o->step = s->step;
    o->avg_rho = (float)s->avg_rho;
    o->avg_kinetic = (float)s->avg_ke;
    o->avg_tke = (float)s->avg_tke;
    o->max_velocity_lb = (float)s->max_u;
    o->convergence = (float)s->convergence;
    o->converged = s->converged;
    o->diverged = s->diverged;
    o->negative_pops = s->neg;
    o->bad_pops = s->bad;
    o->rho_out_of_range = s->rho_out;
    o->rho_non_finite = s->rho_nonfin;
    o->u_limited = s->ulim;
    o->nan_count = s->nan_count;
    o->sum_rho = s->sum_rho;
    o->sum_kinetic = s->sum_ke;
    o->sum_tke = s->sum_tke;
    o->nusselt = (float)s->nusselt;
    o->mean_t = (float)s->mean_t;
    o->fluid_cells = s->fluid_cells;
}

void ao_lbm_get_fields(const ao_lbm* s, float* rho, float* ux, float* uy, float* uz, float* strain, float* tke) {
    for (int c = 0; c < s->total; ++c) {
        if (rho) rho[c] = (float)s->rho[c];
        if (ux) ux[c] = (float)s->ux[c];
        if (uy) uy[c] = (float)s->uy[c];
        if (uz) uz[c] = (float)s->uz[c];
        if (strain) strain[c] = (float)s->strain[c];
        if (tke) tke[c] = (float)s->tke[c];
    }
}

void ao_lbm_get_fields_f64(const ao_lbm* s, double* rho, double* ux, double* uy, double* uz) {
    for (int c = 0; c < s->total; ++c) {
        if (rho) rho[c] = (double)s->rho[c];
        if (ux) ux[c] = (double)s->ux[c];
        if (uy) uy[c] = (double)s->uy[c];
        if (uz) uz[c] = (double)s->uz[c];
    }
}

void ao_lbm_get_populations(const ao_lbm* s, float* out) {
    const size_t n = (size_t)s->total;
    for (size_t c = 0; c < n; ++c)
        for (int q = 0; q < Q19; ++q) out[(size_t)q * n + c] = (float)s->f[c * Q19 + q];
}

void ao_lbm_set_populations(ao_lbm* s, const float* in) {
    const size_t n = (size_t)s->total;
    for (size_t c = 0; c < n; ++c)
        for (int q = 0; q < Q19; ++q) s->f[c * Q19 + q] = (real)in[(size_t)q * n + c];
}

void ao_lbm_set_equilibrium(ao_lbm* s, const float* rho, const float* ux, const float* uy, const float* uz) {
    for (int c = 0; c < s->total; ++c) {
        if (is_wall(s, c)) continue;
        set_cell_eq(s, c, rho ? (real)rho[c] : K(1.0), (real)ux[c], (real)uy[c], (real)uz[c]);
    }
}

void ao_lbm_get_wall_dist(const ao_lbm* s, uint8_t* wd) { memcpy(wd, s->wall, (size_t)s->total); }

void ao_thermal_get(const ao_lbm* s, float* T, float* buoy) {
    if (!s->th_on) return;
    for (int c = 0; c < s->total; ++c) {
        if (T) T[c] = (float)s->T[c];
        if (buoy) buoy[c] = (float)s->buoy[c];
    }
}

/* ------------------------------------------------------------------------ */
/* Control-volume momentum balance, aeros/src/lbm.cpp:2183-2232              */
/* ------------------------------------------------------------------------ */
static void cv_add(const ao_lbm* s, int c, real nx_, real ny_, real nz_, double* fx, double* fy, double* fz) {
    if (c < 0 || c >= s->total) return;
    if (s->mask[c] == AEROS_CELL_SOLID) return;
    const real rho = s->rho[c];
    const real ux = s->ux[c], uy = s->uy[c], uz = s->uz[c];
    const real p = (K(1.0) / K(3.0)) * (rho - K(1.0));
    const real un = ux * nx_ + uy * ny_ + uz * nz_;
    *fx += p * nx_ + rho * ux * un;
    *fy += p * ny_ + rho * uy * un;
    *fz += p * nz_ + rho * uz * un;
}

void ao_lbm_cv_force_box(const ao_lbm* s, const int32_t b[6], double out[3]) {
    const int nx = s->nx, ny = s->ny;
    const int x0 = b[0], x1 = b[1], y0 = b[2], y1 = b[3], z0 = b[4], z1 = b[5];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int z = z0; z <= z1; ++z)
        for (int y = y0; y <= y1; ++y) {
            cv_add(s, (z * ny + y) * nx + x0, K(-1.0), K(0.0), K(0.0), &fx, &fy, &fz);
            cv_add(s, (z * ny + y) * nx + x1, K(1.0), K(0.0), K(0.0), &fx, &fy, &fz);
        }
    for (int z = z0; z <= z1; ++z)
        for (int x = x0; x <= x1; ++x) {
            cv_add(s, (z * ny + y0) * nx + x, K(0.0), K(-1.0), K(0.0), &fx, &fy, &fz);
            cv_add(s, (z * ny + y1) * nx + x, K(0.0), K(1.0), K(0.0), &fx, &fy, &fz);
        }
    for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x) {
            cv_add(s, (z0 * ny + y) * nx + x, K(0.0), K(0.0), K(-1.0), &fx, &fy, &fz);
            cv_add(s, (z1 * ny + y) * nx + x, K(0.0), K(0.0), K(1.0), &fx, &fy, &fz);
        }
    out[0] = -fx; out[1] = -fy; out[2] = -fz;
}

static int clamp_side(int v, int n) { return v < 1 ? 1 : (v > n - 2 ? n - 2 : v); }

void ao_lbm_cv_force(const ao_lbm* s, float hx_, float hy_, float hz_, double out[3]) {
    const int cx = (int)(s->nx * 0.5f), cy = (int)(s->ny * 0.5f), cz = (int)(s->nz * 0.5f);
    int hx = (int)(s->nx * hx_), hy = (int)(s->ny * hy_), hz = (int)(s->nz * hz_);
    if (hx < 2) hx = 2;
    if (hy < 2) hy = 2;
    if (hz < 2) hz = 2;
    int32_t b[6] = {clamp_side(cx - hx, s->nx), clamp_side(cx + hx, s->nx), clamp_side(cy - hy, s->ny),
                    clamp_side(cy + hy, s->ny), clamp_side(cz - hz, s->nz), clamp_side(cz + hz, s->nz)};
    double r[3];
    ao_lbm_cv_force_box(s, b, r);
#if defined(AO_IS_DOUBLE) && AO_IS_DOUBLE
    out[0] = r[0]; out[1] = r[1]; out[2] = r[2];
#else
    /* the reference returns the negated double sums cast to float */
    out[0] = (double)(float)r[0]; out[1] = (double)(float)r[1]; out[2] = (double)(float)r[2];
#endif
}

/* lbmProjectedAreaCells, aeros/src/lbm.cpp:2236-2256. */
double ao_lbm_projected_area(const ao_lbm* s, int axis) {
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    const int amax = axis == 0 ? ny : nx;
    const int bmax = axis == 2 ? ny : nz;
    char* hit = (char*)calloc((size_t)amax * bmax, 1);
    double area = 0.0;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const int c = (z * ny + y) * nx + x;
                if (s->mask[c] != AEROS_CELL_SOLID) continue;
                int a, b;
                if (axis == 0) { a = y; b = z; }
                else if (axis == 1) { a = x; b = z; }
                else { a = x; b = y; }
                const size_t k = (size_t)b * amax + a;
                if (!hit[k]) { hit[k] = 1; area += 1.0; }
            }
    free(hit);
    return (double)(float)area;
}


/* ---- readback and post-processing --------------------------------------------
 * The readback prep at the end of stepLBMCPU (aeros/src/lbm.cpp:1602-1705):
 * world velocity and pressure, strided pressure min / max, the density
 * residual against the previous readback and the change of max |u|. */
int ao_lbm_world_fields(ao_lbm* s, const aeros_world_params* wp, float* oux, float* ouy, float* ouz, float* op,
                        aeros_world_stats* st) {
    const int total = s->total;
    if (!s->uxw) {
        s->uxw = (real*)calloc((size_t)total, sizeof(real));
        s->uyw = (real*)calloc((size_t)total, sizeof(real));
        s->uzw = (real*)calloc((size_t)total, sizeof(real));
        s->pres = (real*)calloc((size_t)total, sizeof(real));
        s->vort = (real*)calloc((size_t)total, sizeof(real));
        s->qc = (real*)calloc((size_t)total, sizeof(real));
        s->prev_step = -1;
        s->prev_maxu = K(0.0);
        if (!s->uxw || !s->uyw || !s->uzw || !s->pres || !s->vort || !s->qc) return -1;
    }
    const real in0 = (real)s->p.u_in[0], in1 = (real)s->p.u_in[1], in2 = (real)s->p.u_in[2];
    real U0mag2 = RSQRT(in0 * in0 + in1 * in1 + in2 * in2);
    if (!isfinite(U0mag2) || U0mag2 < K(1e-6)) U0mag2 = K(0.08);
    real scale = (real)wp->flow_speed / U0mag2;
    if (!isfinite(scale) || scale > K(1000.0)) scale = K(20.0);
    const real rho0 = (real)wp->air_density;
    const real cs2 = K(1.0) / K(3.0);
    long long pbad = 0;
    for (int c = 0; c < total; ++c) {
        if (is_wall(s, c)) {
            s->uxw[c] = K(0.0); s->uyw[c] = K(0.0); s->uzw[c] = K(0.0);
            s->pres[c] = K(0.0);
            continue;
        }
        real ux = s->ux[c], uy = s->uy[c], uz = s->uz[c];
        if (!isfinite(ux)) ux = K(0.0);
        s->uxw[c] = ux * scale;
        s->uyw[c] = uy * scale;
        s->uzw[c] = uz * scale;
        real rho = s->rho[c];
        if (!isfinite(rho)) rho = K(1.0);
        const real pLat = cs2 * (rho - K(1.0));
        real pPhys = pLat * scale * scale * rho0;
        if (!isfinite(pPhys)) { pbad++; pPhys = K(0.0); }
        s->pres[c] = pPhys;
    }
    int stride = 1;
    while (total / stride > 262144) stride *= 2;
    real pMin = K(1e30), pMax = K(-1e30);
    const int valid = s->prev_rho != NULL && s->prev_step >= 0 && s->step >= s->prev_step;
    if (!s->prev_rho) {
        s->prev_rho = (real*)malloc((size_t)total * sizeof(real));
        if (!s->prev_rho) return -1;
        for (int c = 0; c < total; ++c) s->prev_rho[c] = K(1.0);
    }
    double sumSq = 0.0;
    int nSampled = 0;
    for (int c = 0; c < total; c += stride) {
        const real p = s->pres[c];
        if (isfinite(p)) { if (p < pMin) pMin = p; if (p > pMax) pMax = p; }
        if (valid) {
            const real r = s->rho[c];
            if (isfinite(r)) {
                const real d = r - s->prev_rho[c];
                sumSq += (double)d * (double)d;
                ++nSampled;
            }
        }
    }
    if (st) {
        st->pressure_min = (pMin <= pMax && isfinite(pMin)) ? (float)pMin : 0.0f;
        st->pressure_max = (pMin <= pMax && isfinite(pMax)) ? (float)pMax : 0.0f;
        st->residual_rho = (valid && nSampled > 0) ? (float)sqrt(sumSq / (double)nSampled) : 0.0f;
        st->residual_u = (float)RABS(s->max_u - s->prev_maxu);
        st->pressure_non_finite = pbad;
    }
    s->prev_maxu = s->max_u;
    for (int c = 0; c < total; ++c) {
        const real r = s->rho[c];
        s->prev_rho[c] = isfinite(r) ? r : K(1.0);
    }
    s->prev_step = s->step;
    for (int c = 0; c < total; ++c) {
        if (oux) oux[c] = (float)s->uxw[c];
        if (ouy) ouy[c] = (float)s->uyw[c];
        if (ouz) ouz[c] = (float)s->uzw[c];
        if (op) op[c] = (float)s->pres[c];
    }
    return 0;
}

/* computeLBMVorticityAndQ, aeros/src/lbm.cpp:2005-2093 (from the world
 * velocity of the last ao_lbm_world_fields call). */
int ao_lbm_vorticity_q(ao_lbm* s, const aeros_world_params* wp, float* ovort, float* oq, float* ostrain) {
    if (!s->uxw) return -1;
    const int Nx = s->nx, Ny = s->ny, Nz = s->nz, total = s->total;
    real csx = (real)wp->cell[0], csy = (real)wp->cell[1], csz = (real)wp->cell[2];
    if (csx < K(1e-6)) csx = K(0.1);
    if (csy < K(1e-6)) csy = K(0.1);
    if (csz < K(1e-6)) csz = K(0.1);
    const real ix = K(1.0) / csx, iy = K(1.0) / csy, iz = K(1.0) / csz;
    const real* uxW = s->uxw;
    const real* uyW = s->uyw;
    const real* uzW = s->uzw;
    for (int z = 1; z < Nz - 1; ++z)
        for (int y = 1; y < Ny - 1; ++y)
            for (int x = 1; x < Nx - 1; ++x) {
                const int cell = (z * Ny + y) * Nx + x;
                if (is_wall(s, cell)) { s->vort[cell] = K(0.0); s->qc[cell] = K(0.0); continue; }
                const int xm = cell - 1, xp = cell + 1, ym = cell - Nx, yp = cell + Nx;
                const int zm = cell - Nx * Ny, zp = cell + Nx * Ny;
                const real dux_dx = (uxW[xp] - uxW[xm]) * K(0.5) * ix;
                const real dux_dy = (uxW[yp] - uxW[ym]) * K(0.5) * iy;
                const real dux_dz = (uxW[zp] - uxW[zm]) * K(0.5) * iz;
                const real duy_dx = (uyW[xp] - uyW[xm]) * K(0.5) * ix;
                const real duy_dy = (uyW[yp] - uyW[ym]) * K(0.5) * iy;
                const real duy_dz = (uyW[zp] - uyW[zm]) * K(0.5) * iz;
                const real duz_dx = (uzW[xp] - uzW[xm]) * K(0.5) * ix;
                const real duz_dy = (uzW[yp] - uzW[ym]) * K(0.5) * iy;
                const real duz_dz = (uzW[zp] - uzW[zm]) * K(0.5) * iz;
                if (!isfinite(dux_dx)) { s->vort[cell] = K(0.0); s->qc[cell] = K(0.0); continue; }
                const real wx = duz_dy - duy_dz, wy = dux_dz - duz_dx, wz = duy_dx - dux_dy;
                real vm = RSQRT(wx * wx + wy * wy + wz * wz);
                if (!isfinite(vm)) vm = K(0.0);
                if (vm > K(1000.0)) vm = K(1000.0);
                s->vort[cell] = vm;
                const real Sxx = dux_dx, Syy = duy_dy, Szz = duz_dz;
                const real Sxy = K(0.5) * (dux_dy + duy_dx);
                const real Sxz = K(0.5) * (dux_dz + duz_dx);
                const real Syz = K(0.5) * (duy_dz + duz_dy);
                const real Oxy = K(0.5) * (dux_dy - duy_dx);
                const real Oxz = K(0.5) * (dux_dz - duz_dx);
                const real Oyz = K(0.5) * (duy_dz - duz_dy);
                const real S2 = Sxx * Sxx + Syy * Syy + Szz * Szz + K(2.0) * (Sxy * Sxy + Sxz * Sxz + Syz * Syz);
                const real O2 = K(2.0) * (Oxy * Oxy + Oxz * Oxz + Oyz * Oyz);
                real Q = K(0.5) * (O2 - S2);
                if (!isfinite(Q)) Q = K(0.0);
                if (Q > K(1e6)) Q = K(1e6);
                if (Q < K(-1e6)) Q = K(-1e6);
                s->qc[cell] = Q;
                real strain = RSQRT(K(2.0) * S2);
                if (!isfinite(strain)) strain = K(0.0);
                s->strain[cell] = strain;
            }
    for (int c = 0; c < total; ++c) {
        if (ovort) ovort[c] = (float)s->vort[c];
        if (oq) oq[c] = (float)s->qc[c];
        if (ostrain) ostrain[c] = (float)s->strain[c];
    }
    return 0;
}

static real clamp01r(real t) { return t < K(0.0) ? K(0.0) : (t > K(1.0) ? K(1.0) : t); }

/* getLBMVelocityLB (lbm.cpp:1782-1840), sampleFieldTrilinear with solid
 * corners skipped (lbm.cpp:1881-1933), isLBMSolidWorld (lbm.cpp:1954-1969). */
int ao_lbm_sample(const ao_lbm* s, const aeros_world_params* wp, int field, const float* pts, int64_t n, float* out,
                  uint8_t* valid) {
    const real* fld = NULL;
    if (field == AEROS_FIELD_DENSITY) fld = s->rho;
    else if (field == AEROS_FIELD_PRESSURE) fld = s->pres;
    else if (field == AEROS_FIELD_VORTICITY) fld = s->vort;
    else if (field == AEROS_FIELD_Q) fld = s->qc;
    else if (field == AEROS_FIELD_STRAIN) fld = s->strain;
    else if (field == AEROS_FIELD_TKE) fld = s->tke;
    if (field != AEROS_FIELD_VELOCITY_LB && field != AEROS_FIELD_SOLID && !fld) return -1;
    const int Nx = s->nx, Ny = s->ny, Nz = s->nz;
    const real mnx = (real)wp->min[0], mny = (real)wp->min[1], mnz = (real)wp->min[2];
    const real csx = (real)wp->cell[0], csy = (real)wp->cell[1], csz = (real)wp->cell[2];
    for (int64_t i = 0; i < n; ++i) {
        const real wx = (real)pts[3 * i], wy = (real)pts[3 * i + 1], wz = (real)pts[3 * i + 2];
        uint8_t ok = 0;
        if (field == AEROS_FIELD_VELOCITY_LB) {
            real rx = K(0.0), ry = K(0.0), rz = K(0.0);
            if (isfinite(wx)) {
                const real fx = (wx - mnx) / csx, fy = (wy - mny) / csy, fz = (wz - mnz) / csz;
                const int ix = (int)RFLOOR(fx), iy = (int)RFLOOR(fy), iz = (int)RFLOOR(fz);
                const real tx = clamp01r(fx - (real)ix), ty = clamp01r(fy - (real)iy), tz = clamp01r(fz - (real)iz);
                if (!(ix < 0 || ix >= Nx - 1 || iy < 0 || iy >= Ny - 1 || iz < 0 || iz >= Nz - 1)) {
                    const real w[8] = {(1 - tx) * (1 - ty) * (1 - tz), tx * (1 - ty) * (1 - tz), (1 - tx) * ty * (1 - tz),
                                       tx * ty * (1 - tz), (1 - tx) * (1 - ty) * tz, tx * (1 - ty) * tz,
                                       (1 - tx) * ty * tz, tx * ty * tz};
                    real vx[8], vy[8], vz[8], ws[8], totalW = K(0.0);
                    int cnt = 0;
                    for (int k = 0; k < 8; ++k) {
                        const int cell = ((iz + ((k >> 2) & 1)) * Ny + (iy + ((k >> 1) & 1))) * Nx + (ix + (k & 1));
                        if (is_wall(s, cell)) continue;
                        if (!isfinite(s->ux[cell])) continue;
                        vx[cnt] = s->ux[cell]; vy[cnt] = s->uy[cell]; vz[cnt] = s->uz[cell]; ws[cnt] = w[k];
                        totalW += w[k];
                        ++cnt;
                    }
                    if (cnt > 0) {
                        ok = 1;
                        if (totalW < K(1e-6)) {
                            rx = vx[0]; ry = vy[0]; rz = vz[0];
                        } else {
                            for (int k = 0; k < cnt; ++k) {
                                const real sc = ws[k] / totalW;
                                rx += vx[k] * sc; ry += vy[k] * sc; rz += vz[k] * sc;
                            }
                            if (!isfinite(rx)) { rx = K(0.0); ry = K(0.0); rz = K(0.0); }
                        }
                    }
                }
            }
            out[3 * i] = (float)rx; out[3 * i + 1] = (float)ry; out[3 * i + 2] = (float)rz;
        } else if (field == AEROS_FIELD_SOLID) {
            real r = K(0.0);
            if (isfinite(wx) && isfinite(wy) && isfinite(wz) && csx >= K(1e-9) && csy >= K(1e-9) && csz >= K(1e-9)) {
                const real fx = (wx - mnx) / csx, fy = (wy - mny) / csy, fz = (wz - mnz) / csz;
                const int ix = (int)RFLOOR(fx), iy = (int)RFLOOR(fy), iz = (int)RFLOOR(fz);
                if (!(ix < 0 || ix >= Nx || iy < 0 || iy >= Ny || iz < 0 || iz >= Nz)) {
                    ok = 1;
                    r = is_wall(s, (iz * Ny + iy) * Nx + ix) ? K(1.0) : K(0.0);
                }
            }
            out[i] = (float)r;
        } else {
            real r = K(0.0);
            if (isfinite(wx) && isfinite(wy) && isfinite(wz) && !(csx < K(1e-9) || csy < K(1e-9) || csz < K(1e-9)) &&
                !(Nx < 2 || Ny < 2 || Nz < 2)) {
                const real fx = (wx - mnx) / csx, fy = (wy - mny) / csy, fz = (wz - mnz) / csz;
                const int ix = (int)RFLOOR(fx), iy = (int)RFLOOR(fy), iz = (int)RFLOOR(fz);
                if (!(ix < 0 || iy < 0 || iz < 0) && !(ix > Nx - 2 || iy > Ny - 2 || iz > Nz - 2)) {
                    const real tx = clamp01r(fx - (real)ix), ty = clamp01r(fy - (real)iy), tz = clamp01r(fz - (real)iz);
                    const real wxs[2] = {K(1.0) - tx, tx}, wys[2] = {K(1.0) - ty, ty}, wzs[2] = {K(1.0) - tz, tz};
                    real acc = K(0.0), wsum = K(0.0);
                    for (int dz = 0; dz <= 1; ++dz)
                        for (int dy = 0; dy <= 1; ++dy)
                            for (int dx = 0; dx <= 1; ++dx) {
                                const int cell = ((iz + dz) * Ny + (iy + dy)) * Nx + (ix + dx);
                                if (is_wall(s, cell)) continue;
                                const real v = fld[cell];
                                if (!isfinite(v)) continue;
                                const real w = wxs[dx] * wys[dy] * wzs[dz];
                                acc += v * w;
                                wsum += w;
                            }
                    if (!(wsum < K(1e-6))) {
                        acc /= wsum;
                        if (isfinite(acc)) { r = acc; ok = 1; }
                    }
                }
            }
            out[i] = (float)r;
        }
        if (valid) valid[i] = ok;
    }
    return 0;
}
