/*
 * aeros_oracle.h — CPU restatement of the reference LBM step (TEST INFRASTRUCTURE).
 *
 * This is the checker, never the product: only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load it. It restates, in plain C, the
 * algorithm of the reference solver step (aeros/src/lbm.cpp:907-1709), the
 * thermal lattice (aeros/src/thermal_lbm.cpp:84-355), the control-volume force
 * (aeros/src/lbm.cpp:2183-2256) and the voxelizer's inside test
 * (aeros/src/mesh_bvh.h:62-185), keeping the reference's floating-point
 * operation order so that the FP32 build reproduces the reference bit for bit
 * on the same inputs (pinned against the reference's own build, see
 * tests/golden/). Compiled twice: AO_REAL=float (liboracle_f32.so) and
 * AO_REAL=double (liboracle_f64.so, the FP64 run the precision form is
 * measured against). Both builds export the same symbols.
 *
 * Layout follows the reference: populations AoS f[cell*19 + q].
 */
#ifndef AEROS_ORACLE_H
#define AEROS_ORACLE_H
#include <stdint.h>
#include "../include/aeros_lbm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ao_lbm ao_lbm;

/* initLBM on an explicit grid (aeros/src/lbm.cpp:405-886, padding 0). */
ao_lbm* ao_lbm_create(const aeros_lbm_params* p, const uint8_t* mask);
void    ao_lbm_destroy(ao_lbm* s);
/* thermalInit (aeros/src/thermal_lbm.cpp:84-140). Returns 0 on success. */
int     ao_thermal_init(ao_lbm* s, const aeros_thermal_params* tp);
int     ao_thermal_upload(ao_lbm* s, const float* T);
/* stepLBMCPU(steps) without the readback prep. */
void    ao_lbm_step(ao_lbm* s, int steps);
void    ao_lbm_get_stats(const ao_lbm* s, aeros_lbm_stats* out);
/* Fields as float (converted from the build's real type). */
void    ao_lbm_get_fields(const ao_lbm* s, float* rho, float* ux, float* uy,
                          float* uz, float* strain, float* tke);
/* Fields in the build's native precision (double for the f64 build). */
void    ao_lbm_get_fields_f64(const ao_lbm* s, double* rho, double* ux,
                              double* uy, double* uz);
/* Pre-collision populations, layout [19][cells] (SoA on output). */
void    ao_lbm_get_populations(const ao_lbm* s, float* f);
void    ao_lbm_set_populations(ao_lbm* s, const float* f);
void    ao_lbm_set_equilibrium(ao_lbm* s, const float* rho, const float* ux,
                               const float* uy, const float* uz);
void    ao_lbm_get_wall_dist(const ao_lbm* s, uint8_t* wd);
void    ao_thermal_get(const ao_lbm* s, float* T, float* buoy);
/* lbmControlVolumeForce / explicit box / lbmProjectedAreaCells. */
void    ao_lbm_cv_force(const ao_lbm* s, float hx, float hy, float hz, double out[3]);
void    ao_lbm_cv_force_box(const ao_lbm* s, const int32_t box[6], double out[3]);
double  ao_lbm_projected_area(const ao_lbm* s, int axis);
/* lbmEquilibriumMoments (aeros/src/lbm.cpp:307-327). Returns 1 on success. */
/* readback and post-processing (lbm.cpp:1602-1705, 2005-2093, 1782-1969) */
int     ao_lbm_world_fields(ao_lbm* s, const aeros_world_params* wp, float* ux, float* uy,
                            float* uz, float* pressure, aeros_world_stats* st);
int     ao_lbm_vorticity_q(ao_lbm* s, const aeros_world_params* wp, float* vort, float* q,
                           float* strain);
int     ao_lbm_sample(const ao_lbm* s, const aeros_world_params* wp, int field, const float* pts,
                      int64_t n, float* out, uint8_t* valid);
int     ao_equilibrium_moments(float rho, float ux, float uy, float uz,
                               float* sum, float* mx, float* my, float* mz);
int     ao_real_bytes(void);

/* Voxelizer inside test by brute force over all triangles (no BVH): three
 * jittered axis rays, parity, majority (aeros/src/mesh_bvh.h:168-185). */
int     ao_voxelize_brute(const float* tris, int64_t ntri,
                          const aeros_voxel_grid* g, uint8_t* mask);
int     ao_count_hits_brute(const float* tris, int64_t ntri, const float o[3],
                            int axis);
void    ao_voxel_plan(const float size[3], int res, uint64_t budget,
                      aeros_voxel_plan_t* out);
/* OpenMP thread count used by the oracle loops. */
int     ao_set_threads(int n);

/* sdf_oracle.c: buildVoxelGrid's distance field as the reference computes it,
 * and the least-fixed-point form the device computes (see its header). */
int     ao_sdf_reference(const uint8_t* mask, int nx, int ny, int nz, const float cs[3], float* d);
int     ao_sdf_exact(const uint8_t* mask, int nx, int ny, int nz, const float cs[3], float* d);
int     ao_sdf_sample(const float* sdf, int nx, int ny, int nz, const float mn[3], const float cs[3],
                      const float* pts, int64_t n, float* dist, float* normal);

/* surface_oracle.c: computeLiftDrag (forces.cpp:401-688) on the state's world
 * pressure (ao_lbm_world_fields first); f32_sums: FP32 sums in triangle order
 * (the reference on one thread), else FP64 sums (the device's form). */
int     ao_surface_forces(const ao_lbm* s, const aeros_world_params* wp, const aeros_surface_params* sp,
                          const float* sdf, const aeros_voxel_grid* sdf_grid, const float* vert, const float* nrm,
                          int64_t ntri, int f32_sums, aeros_surface_forces* out, float* cp_out);
/* The same over a world pressure array and its wall cells (1 = solid or
 * ground: the sampler skips them), nx*ny*nz each. */
int     ao_surface_forces_field(const float* pressure, const uint8_t* wall, int nx, int ny, int nz,
                                const aeros_world_params* wp, const aeros_surface_params* sp, const float* sdf,
                                const aeros_voxel_grid* sdf_grid, const float* vert, const float* nrm, int64_t ntri,
                                int f32_sums, aeros_surface_forces* out, float* cp_out);

#ifdef __cplusplus
}
#endif
#endif
