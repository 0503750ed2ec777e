/*
 * surface_oracle.c — CPU restatement of the surface-pressure lift and drag
 * (TEST INFRASTRUCTURE ONLY: the checker of aeros_lbm_surface_forces, never
 * the product).
 *
 * Follows computeLiftDrag (aeros/src/forces.cpp:401-688) on its LBM branch,
 * with computeLBMRefArea (aeros/src/lbm.cpp:2111-2160) and wallSamplePoint
 * (forces.cpp:75-90). All arithmetic is FP32 in the reference's operation
 * order (glm: dot = (x*x' + y*y') + z*z', length = sqrt(dot), cross as glm,
 * normalize = v * (1 / sqrt(dot)), clamp = min(max(x, lo), hi) with glm's
 * comparison forms). The per-triangle sums either accumulate in FP32 in
 * triangle order (f32_sums = 1: the reference run on one thread, pinned bit
 * for bit against its own build) or in FP64 (f32_sums = 0: the form the device
 * computes, whose reduction order does not change the result beyond FP64
 * rounding).
 */
#include <math.h>
#include <string.h>

#include "aeros_oracle.h"

typedef struct { float x, y, z; } v3;

static v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 scale(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static v3 divs(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
static float dot3(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static float len3(v3 a) { return sqrtf(dot3(a, a)); }
static v3 cross3(v3 a, v3 b) {
    return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static float gmax(float a, float b) { return (a < b) ? b : a; }
static float gmin(float a, float b) { return (b < a) ? b : a; }
static float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
static v3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }

/* wallSamplePoint, forces.cpp:75-90 */
static v3 wall_sample_point(v3 p, v3 n, float lbm_cell, const float* sdf, const aeros_voxel_grid* g) {
    const float nl = len3(n);
    if (!(nl > 1e-6f) || !isfinite(nl)) return p;
    const v3 nn = divs(n, nl);
    float cs = lbm_cell;
    if (!isfinite(cs) || cs <= 1e-9f) cs = 0.01f;
    const float off = 0.6f * cs;
    const v3 q = add(p, scale(nn, off));
    if (sdf) {
        const float pt[3] = {q.x, q.y, q.z};
        float d = 0.0f;
        ao_sdf_sample(sdf, g->nx, g->ny, g->nz, g->min, g->cell, pt, 1, &d, NULL);
        if (d <= 0.0f) return p;
    }
    return q;
}

/* computeLBMRefArea's direction, lbm.cpp:2114-2121 */
static v3 angle_dir(float az_deg, float el_deg) {
    const float az = az_deg * 0.01745329251994329576923690768489f;
    const float el = el_deg * 0.01745329251994329576923690768489f;
    const float ce = cosf(el), se = sinf(el), ca = cosf(az), sa = sinf(az);
    v3 d = mk(ce * ca, se, ce * sa);
    const float l = len3(d);
    if (l > 1e-6f) d = divs(d, l);
    else d = mk(1.0f, 0.0f, 0.0f);
    return d;
}

/* computeLBMRefArea's bounding-box fallback, lbm.cpp:2146-2156 */
static float bbox_area(const aeros_surface_params* sp, v3 fd) {
    float sy = sp->bb_max[1] - sp->bb_min[1], sz = sp->bb_max[2] - sp->bb_min[2], sx = sp->bb_max[0] - sp->bb_min[0];
    if (!isfinite(sy) || sy < 0.01f) sy = sp->max_dim;
    if (!isfinite(sz) || sz < 0.01f) sz = sp->max_dim;
    if (!isfinite(sx) || sx < 0.01f) sx = sp->max_dim;
    float a = (fabsf(fd.x) * sy * sz + fabsf(fd.y) * sx * sz + fabsf(fd.z) * sx * sy);
    if (!isfinite(a) || a < 1e-6f) a = sp->max_dim * sp->max_dim * 0.5f;
    return a;
}

enum { S_FX, S_FY, S_FZ, S_CX, S_CY, S_CZ, S_MX, S_MY, S_MZ, S_AREA, S_PRESS, S_FRONT, S_BASEA, S_BASEF, S_PROJ };

/* the pressure at a world point: 1 with *out set, or 0 (no data) */
typedef int (*pressure_fn)(const void* ctx, const aeros_world_params* wp, const float pt[3], float* out);

static int pressure_of_state(const void* ctx, const aeros_world_params* wp, const float pt[3], float* out) {
    uint8_t ok = 0;
    ao_lbm_sample((const ao_lbm*)ctx, wp, AEROS_FIELD_PRESSURE, pt, 1, out, &ok);
    return ok;
}

typedef struct {
    const float* p;
    const uint8_t* wall;
    int nx, ny, nz;
} field_ctx;

/* sampleFieldTrilinear(lbmPressure, pos, skipSolid = true), lbm.cpp:1881-1933,
   over a pressure array and its wall (solid or ground) cells */
static int pressure_of_field(const void* ctx, const aeros_world_params* wp, const float pt[3], float* out) {
    const field_ctx* f = (const field_ctx*)ctx;
    *out = 0.0f;
    const float wx = pt[0], wy = pt[1], wz = pt[2];
    if (!(isfinite(wx) && isfinite(wy) && isfinite(wz))) return 0;
    if (wp->cell[0] < 1e-9f || wp->cell[1] < 1e-9f || wp->cell[2] < 1e-9f) return 0;
    if (f->nx < 2 || f->ny < 2 || f->nz < 2) return 0;
    const float fx = (wx - wp->min[0]) / wp->cell[0], fy = (wy - wp->min[1]) / wp->cell[1];
    const float fz = (wz - wp->min[2]) / wp->cell[2];
    const float flx = floorf(fx), fly = floorf(fy), flz = floorf(fz);
    if (!(flx >= 0.0f && fly >= 0.0f && flz >= 0.0f)) return 0;
    if (flx > (float)(f->nx - 2) || fly > (float)(f->ny - 2) || flz > (float)(f->nz - 2)) return 0;
    const int ix = (int)flx, iy = (int)fly, iz = (int)flz;
    const float tx = fminf(fmaxf(fx - (float)ix, 0.0f), 1.0f), ty = fminf(fmaxf(fy - (float)iy, 0.0f), 1.0f);
    const float tz = fminf(fmaxf(fz - (float)iz, 0.0f), 1.0f);
    const float wxs[2] = {1.0f - tx, tx}, wys[2] = {1.0f - ty, ty}, wzs[2] = {1.0f - tz, tz};
    float acc = 0.0f, wsum = 0.0f;
    for (int dz = 0; dz <= 1; ++dz)
        for (int dy = 0; dy <= 1; ++dy)
            for (int dx = 0; dx <= 1; ++dx) {
                const int64_t c = ((int64_t)(iz + dz) * f->ny + (iy + dy)) * f->nx + (ix + dx);
                if (f->wall[c]) continue;
                const float v = f->p[c];
                if (!isfinite(v)) continue;
                const float w = wxs[dx] * wys[dy] * wzs[dz];
                acc += v * w;
                wsum += w;
            }
    if (wsum < 1e-6f) return 0;
    acc /= wsum;
    if (!isfinite(acc)) return 0;
    *out = acc;
    return 1;
}

static int surface_forces(pressure_fn pfn, const void* ctx, const aeros_world_params* wp,
                          const aeros_surface_params* sp, const float* sdf, const aeros_voxel_grid* sdf_grid,
                          const float* vert, const float* nrm, int64_t ntri, int f32_sums, aeros_surface_forces* out,
                          float* cp_out) {
    memset(out, 0, sizeof(*out));
    if (cp_out)
        for (int64_t t = 0; t < ntri; ++t) cp_out[t] = 0.0f;
    out->status = AEROS_SURFACE_NOT_RUN;
    out->ref_area = sp->ref_area;   /* aeroRefArea stays as it was on the early returns */
    if (ntri <= 0 || !vert || !nrm) return 0;   /* forces.cpp:403-406 */

    /* scalar set-up, forces.cpp:408-430 */
    const v3 vel = ld3(sp->velocity);
    float vinf = sqrtf(vel.x * vel.x + vel.y * vel.y + vel.z * vel.z);
    if (!isfinite(vinf) || vinf < 1e-4f) vinf = 1e-4f;
    v3 fd = vel;
    const float fdl = len3(fd);
    if (fdl < 1e-6f || !isfinite(fdl)) {
        out->status = AEROS_SURFACE_NO_FLOW;
        return 0;
    }
    fd = divs(fd, fdl);
    const float T = sp->air_temperature;
    const float T0s = 273.15f, S = 110.4f, mu0 = 1.716e-5f;
    float mu = mu0 * powf(T / T0s, 1.5f) * (T0s + S) / (T + S);
    if (!isfinite(mu) || mu < 1e-6f) mu = 1.81e-5f;
    float rho = sp->use_real_density ? sp->air_density : 1.225f;
    rho = gclamp(rho, 0.0001f, 10.0f);
    float q = 0.5f * rho * vinf * vinf;
    if (q < 1e-9f) q = 1e-6f;
    const v3 adir = angle_dir(sp->flow_azimuth_deg, sp->flow_elevation_deg);

    /* leading edge and quarter-chord point, forces.cpp:444-461 */
    float min_al = 1e9f, max_al = -1e9f;
    for (int64_t t = 0; t < ntri; ++t) {
        const float al = dot3(ld3(vert + 9 * t), fd);
        if (al < min_al) min_al = al;
        if (al > max_al) max_al = al;
    }
    if (!isfinite(min_al)) { min_al = 0.0f; max_al = sp->max_dim; }
    float chord = max_al - min_al;
    if (chord < 1e-6f) chord = sp->max_dim;
    const v3 ctr = ld3(sp->center);
    const v3 cperp = sub(ctr, scale(fd, dot3(ctr, fd)));
    const v3 ac = add(scale(fd, min_al + chord * 0.25f), cperp);
    const float mach = vinf / (sp->speed_of_sound + 1e-6f);
    const int comp = sp->mach_effects && mach > 0.3f && mach < 0.85f;
    const float beta = comp ? gmax(0.2f, sqrtf(1.0f - mach * mach)) : 1.0f;

    float fs[15];
    double ds[15];
    for (int k = 0; k < 15; ++k) { fs[k] = 0.0f; ds[k] = 0.0; }
    long long bad = 0;
    for (int64_t t = 0; t < ntri; ++t) {
        const v3 v0 = ld3(vert + 9 * t), v1 = ld3(vert + 9 * t + 3), v2 = ld3(vert + 9 * t + 6);
        float c[15];
        int has = 0;
        /* computeLBMRefArea's projected area, lbm.cpp:2128-2139 */
        {
            const v3 cr = cross3(sub(v1, v0), sub(v2, v0));
            const float area = 0.5f * len3(cr);
            c[S_PROJ] = 0.0f;
            if (isfinite(area) && !(area < 1e-12f)) {
                const v3 n = scale(cr, 1.0f / sqrtf(dot3(cr, cr)));
                c[S_PROJ] = area * fabsf(dot3(n, adir));
            }
        }
        /* computeTri, forces.cpp:486-582 */
        v3 n = ld3(nrm + 9 * t);
        float cp = 0.0f;
        if (isfinite(v0.x) && isfinite(n.x)) {
            const float nl = len3(n);
            if (!(nl < 1e-6f || !isfinite(nl))) {
                n = divs(n, nl);
                const v3 tc = scale(add(add(v0, v1), v2), 1.0f / 3.0f);
                const v3 cr = cross3(sub(v1, v0), sub(v2, v0));
                const float area = 0.5f * len3(cr);
                if (!(!isfinite(area) || area < 1e-9f || area > 1e6f)) {
                    has = 1;
                    const v3 ps = wall_sample_point(tc, n, wp->cell[0], sdf, sdf_grid);
                    const float pt[3] = {ps.x, ps.y, ps.z};
                    float p = 0.0f;
                    if (!pfn(ctx, wp, pt, &p)) p = 0.0f;
                    cp = p / q;
                    if (comp) {
                        const float den = beta + (mach * mach / (1.0f + beta)) * cp * 0.5f;
                        if (fabsf(den) > 1e-6f) cp = cp / den;
                        else cp /= beta;
                    }
                    if (!isfinite(cp)) { ++bad; cp = 0.0f; }
                    const v3 pf = scale(scale(n, -cp * q), area);
                    const float fdn = dot3(fd, n);
                    c[S_FRONT] = area * fabsf(fdn);
                    c[S_BASEA] = 0.0f;
                    c[S_BASEF] = 0.0f;
                    if (fdn > 0.7f) { c[S_BASEA] = area; c[S_BASEF] = cp * q * area; }
                    float xa = dot3(tc, fd) - min_al;
                    if (xa < 0.001f) xa = 0.001f;
                    if (xa > chord * 1.5f) xa = chord * 1.5f;
                    float re = rho * vinf * xa / mu;
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
                    const float skin = cf * q * area * ff;
                    const v3 force = add(pf, scale(mk(-fd.x, -fd.y, -fd.z), skin));
                    float pw = fabsf(cp) * area;
                    if (cp < 0) pw *= 0.8f;
                    const v3 cw = scale(tc, pw);
                    const v3 m = cross3(sub(tc, ac), force);
                    c[S_FX] = force.x; c[S_FY] = force.y; c[S_FZ] = force.z;
                    c[S_CX] = cw.x; c[S_CY] = cw.y; c[S_CZ] = cw.z;
                    c[S_MX] = m.x; c[S_MY] = m.y; c[S_MZ] = m.z;
                    c[S_AREA] = area;
                    c[S_PRESS] = pw;
                }
            }
        }
        if (cp_out) cp_out[t] = cp;
        for (int k = 0; k < 15; ++k) {
            if (k != S_PROJ && !has) continue;
            if (f32_sums) fs[k] += c[k];
            else ds[k] += (double)c[k];
        }
    }
    float tot[15];
    for (int k = 0; k < 15; ++k) {
        out->sums[k] = f32_sums ? (double)fs[k] : ds[k];
        tot[k] = f32_sums ? fs[k] : (float)ds[k];
    }

    /* reference area: aeroRefArea = computeLBMRefArea() when automatic
       (lbm.cpp:2140-2145, forces.cpp:426-429) */
    float ref_global = sp->ref_area;
    if (sp->auto_ref_area) {
        const float fr = tot[S_PROJ] * 0.5f;
        ref_global = (isfinite(fr) && fr > 1e-6f && fr < 1e6f) ? fr : bbox_area(sp, adir);
    }
    float ref = ref_global;
    if (!isfinite(ref) || ref < 1e-6f) ref = 1.0f;
    ref = gclamp(ref, 1e-6f, 1e6f);

    /* closing formulas, forces.cpp:615-687 */
    v3 F = mk(tot[S_FX], tot[S_FY], tot[S_FZ]);
    if (!isfinite(F.x)) F = mk(0.0f, 0.0f, 0.0f);
    if (sp->auto_ref_area && tot[S_FRONT] > 1e-6f) {
        const float fr = tot[S_FRONT] * 0.5f;
        if (fr > 1e-6f) ref_global = fr;
    }
    float base = 0.0f;
    if (tot[S_BASEA] > 1e-6f) {
        const float avg = tot[S_BASEF] / (q * tot[S_BASEA] + 1e-9f);
        if (avg > -0.05f) {
            float cpb = -0.14f;
            if (sp->reynolds > 1e6f) cpb = -0.12f;
            base = -cpb * q * tot[S_BASEA] * 0.6f;
        }
    }
    float drag = dot3(F, fd) + base;
    if (!isfinite(drag)) drag = base;
    v3 up = mk(0.0f, 1.0f, 0.0f);
    v3 ldir = sub(up, scale(fd, dot3(up, fd)));
    float ldl = len3(ldir);
    if (ldl < 1e-6f || !isfinite(ldl)) {
        up = mk(0.0f, 0.0f, 1.0f);
        ldir = sub(up, scale(fd, dot3(up, fd)));
        ldl = len3(ldir);
    }
    float lift;
    v3 lvec;
    if (ldl < 1e-6f || !isfinite(ldl)) {
        lift = 0.0f;
        lvec = mk(0.0f, 0.0f, 0.0f);
    } else {
        ldir = divs(ldir, ldl);
        lift = dot3(F, ldir);
        if (!isfinite(lift)) lift = 0.0f;
        if (sp->ground_effect) {
            const float gy = sp->vox_min_y + sp->ground_height;
            const float h = sp->center[1] - gy;
            if (h > 0.01f && h < sp->max_dim * 1.0f) {
                const float ge = 1.0f + 0.35f * expf(-h / (sp->max_dim * 0.3f));
                if (lift < 0) lift *= ge;
            }
        }
        lvec = scale(ldir, lift);
        if (!isfinite(lvec.x)) lvec = mk(0.0f, 0.0f, 0.0f);
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
    const float ind = cdi * q * ref;
    if (fabsf(cl) > 0.05f) drag += ind;
    if (sp->mach_effects && mach > 0.7f) {
        float cw = 0.0f;
        if (mach < 0.9f) cw = 20.0f * powf(mach - 0.7f, 4.0f);
        else cw = 0.1f + 0.2f * (mach - 0.9f);
        cw = gclamp(cw, 0.0f, 0.5f);
        drag += cw * q * ref;
    }
    v3 dvec = scale(fd, drag);
    if (!isfinite(dvec.x)) dvec = mk(0.0f, 0.0f, 0.0f);
    const float l2d = fabsf(drag) > 1e-9f ? lift / drag : 0.0f;
    v3 mom = mk(tot[S_MX], tot[S_MY], tot[S_MZ]);
    float mm = len3(mom);
    if (!isfinite(mm)) { mm = 0.0f; mom = mk(0.0f, 0.0f, 0.0f); }
    const v3 cps = mk(tot[S_CX], tot[S_CY], tot[S_CZ]);
    v3 cop;
    if (tot[S_PRESS] > 1e-9f && isfinite(cps.x)) cop = divs(cps, tot[S_PRESS]);
    else if (tot[S_AREA] > 1e-9f) cop = divs(cps, tot[S_AREA]);
    else cop = ac;
    if (!isfinite(cop.x)) cop = ac;

    out->status = AEROS_SURFACE_DONE;
    out->drag = drag;
    out->lift = lift;
    out->lift_to_drag = l2d;
    out->moment_magnitude = mm;
    out->drag_vector[0] = dvec.x; out->drag_vector[1] = dvec.y; out->drag_vector[2] = dvec.z;
    out->lift_vector[0] = lvec.x; out->lift_vector[1] = lvec.y; out->lift_vector[2] = lvec.z;
    out->moment[0] = mom.x; out->moment[1] = mom.y; out->moment[2] = mom.z;
    out->center_of_pressure[0] = cop.x; out->center_of_pressure[1] = cop.y; out->center_of_pressure[2] = cop.z;
    out->ref_area = ref_global;
    out->ref_area_used = ref;
    out->cp_non_finite = bad;
    return 0;
}

int ao_surface_forces(const ao_lbm* s, const aeros_world_params* wp, const aeros_surface_params* sp, const float* sdf,
                      const aeros_voxel_grid* sdf_grid, const float* vert, const float* nrm, int64_t ntri, int f32_sums,
                      aeros_surface_forces* out, float* cp_out) {
    return surface_forces(pressure_of_state, s, wp, sp, sdf, sdf_grid, vert, nrm, ntri, f32_sums, out, cp_out);
}

int ao_surface_forces_field(const float* pressure, const uint8_t* wall, int nx, int ny, int nz,
                            const aeros_world_params* wp, const aeros_surface_params* sp, const float* sdf,
                            const aeros_voxel_grid* sdf_grid, const float* vert, const float* nrm, int64_t ntri,
                            int f32_sums, aeros_surface_forces* out, float* cp_out) {
    const field_ctx f = {pressure, wall, nx, ny, nz};
    return surface_forces(pressure_of_field, &f, wp, sp, sdf, sdf_grid, vert, nrm, ntri, f32_sums, out, cp_out);
}
