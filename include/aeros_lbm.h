/*
 * aeros_lbm.h — C ABI of the GB300 lattice-Boltzmann solver step.
 *
 * Plain C, plain pointers and sizes. Every entry point returns an int status
 * (AEROS_OK == 0, negative on failure) and records a message that
 * aeros_consume_error() hands back and clears — the same record/consume
 * convention as the reference CUDA layer (aeros/src/cuda_api.h:53-56,
 * aeros/src/kernel.cu:57-82). No exceptions cross this boundary.
 *
 * Lattice: D3Q19 (fluid) and D3Q7 (temperature), velocity sets, weights and
 * opposite tables identical to aeros/src/lbm.cpp:92-109 and
 * aeros/src/thermal_lbm.cpp:31-40. Cell index = (z*ny + y)*nx + x.
 *
 * Reference functions each entry point replaces are cited beside it.
 */
#ifndef AEROS_LBM_H
#define AEROS_LBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define AEROS_OK               0
#define AEROS_ERR_INVALID     -1   /* bad argument (null pointer, size, mode) */
#define AEROS_ERR_CUDA        -2   /* CUDA runtime error (message has the call) */
#define AEROS_ERR_ALLOC       -3   /* device or host allocation failed */
#define AEROS_ERR_UNSUPPORTED -4   /* mode combination not implemented */
#define AEROS_ERR_STATE       -5   /* call not valid in the handle's state */
#define AEROS_ERR_TIMEOUT     -6   /* a bounded device wait gave up */

/* ---- enums --------------------------------------------------------------- */
enum { AEROS_CELL_FLUID = 0, AEROS_CELL_SOLID = 1, AEROS_CELL_GROUND = 2 };

/* Population storage. FP32 is the drop-in form (bitwise the reference's
 * arithmetic); FP16/BF16 store shifted deviations f_i - s_i and compute in
 * FP32. */
enum { AEROS_STORE_FP32 = 0, AEROS_STORE_FP16 = 1, AEROS_STORE_BF16 = 2 };

/* What FP16/BF16 storage subtracts from each population (storage_shift).
 * FREESTREAM: the equilibrium f_eq(rho = 1, u_in) when the domain has an
 * inlet (periodic_x == 0); away from a body the stored deviations are then
 * only the non-equilibrium part, which 16 bits resolve. A domain without an
 * inlet keeps the rest state (as WEIGHTS): its flow is not held at any
 * velocity.
 * WEIGHTS: the lattice weights w_i (f_eq at rest). */
enum { AEROS_SHIFT_FREESTREAM = 0, AEROS_SHIFT_WEIGHTS = 1 };

/* Lateral (non-flow-axis, non-periodic) faces. COPY is the reference's rule
 * (an out-of-domain source copies the cell's own post-collision population,
 * aeros/src/lbm.cpp:1392-1394). FREESLIP is a specular-reflection wall that
 * the reference does not have. */
enum { AEROS_LATERAL_COPY = 0, AEROS_LATERAL_FREESLIP = 1 };

/* Outlet face. REFERENCE = convective outlet when convective_outlet != 0
 * (aeros/src/lbm.cpp:1465-1544), otherwise copy-own. ZEROGRAD copies the
 * post-streaming unknowns of the plane upstream (not in the reference). */
enum { AEROS_OUTLET_REFERENCE = 0, AEROS_OUTLET_ZEROGRAD = 1 };

/* ---- parameters ------------------------------------------------------------
 * Lattice-unit parameters after the host has resolved world units; mirrors
 * LBMParams (aeros/src/lbm.h:11-75) plus the inlet velocity that
 * computeInletVelocityLB derives from flowAzimuth/flowElevation/U0
 * (aeros/src/lbm.cpp:186-199). */
typedef struct aeros_lbm_params {
    int32_t nx, ny, nz;          /* grid, each >= 4                                */
    float   tau;                 /* BGK tau / TRT s+ = 1/tau (clamped as the reference) */
    float   smagorinsky_c;       /* Cs (reference clamps to [0, 0.3])              */
    int32_t use_les;             /* useTurbulence: two-pass |S| + Van Driest       */
    int32_t use_trt;             /* useTRT                                          */
    int32_t periodic_x;          /* periodicX (disables inlet/outlet)               */
    int32_t periodic_z;          /* periodicZ                                       */
    int32_t convective_outlet;   /* useConvectiveOutlet                             */
    int32_t flow_axis;           /* 0,1,2 : axis of the inlet/outlet planes         */
    int32_t flow_sign;           /* +1 : inlet at coordinate 0, -1 : at N-1          */
    float   u_in[3];             /* inlet lattice velocity (equilibrium at rho = 1)  */
    float   u_init[3];           /* initial uniform velocity of fluid cells          */
    float   body_force[3];       /* Guo body force, lattice units                    */
    float   vel_scale;           /* flowSpeed / |u_in| (TKE in m^2/s^2)              */
    float   convergence_threshold; /* lbmParams.convergenceThreshold                  */
    int32_t storage;             /* AEROS_STORE_*                                    */
    int32_t lateral_bc;          /* AEROS_LATERAL_*                                  */
    int32_t outlet_bc;           /* AEROS_OUTLET_*                                   */
    int32_t storage_shift;       /* AEROS_SHIFT_* (FP16/BF16 storage only)          */
    int32_t reserved[7];         /* zero                                             */
} aeros_lbm_params;

/* Mirrors ThermalParams (aeros/src/thermal_lbm.h:33-41); nu_lb is the solver
 * viscosity handed to thermalInit (aeros/src/lbm.cpp:876-885). */
typedef struct aeros_thermal_params {
    int32_t enabled;
    float   rayleigh;
    float   prandtl;
    int32_t fixed_wall_temps;    /* hot wall y = 0, cold wall y = ny-1 */
    float   hot_temp;
    float   cold_temp;
    float   perturbation;        /* cos*sin seed amplitude (fraction of dT) */
    float   nu_lb;
    int32_t reserved[4];
} aeros_thermal_params;

/* Per-step diagnostics of the last executed step, as the reference exposes
 * them through globals (aeros/src/lbm.h:78-125, aeros/src/lbm.cpp:1554-1580). */
typedef struct aeros_lbm_stats {
    int64_t step;                /* lbmCurrentStep                               */
    float   avg_rho;             /* lbmAvgRho (fluid mean, FP64 sum)             */
    float   avg_kinetic;         /* lbmAvgKineticEnergy                          */
    float   avg_tke;             /* lbmTKE                                       */
    float   max_velocity_lb;     /* lbmMaxVelocityLB                             */
    float   convergence;         /* lbmConvergence = |dKE|                       */
    int32_t converged;           /* lbmConverged                                 */
    int32_t diverged;            /* last call tripped the divergence guard and   */
                                 /* re-equilibrated (lbm.cpp:1313-1319,1574-1600) */
    int32_t pad0;
    int64_t negative_pops;       /* lbmNegativePops                              */
    int64_t bad_pops;            /* lbmBadPops                                   */
    int64_t rho_out_of_range;    /* lbmRhoOutOfRange                             */
    int64_t rho_non_finite;      /* lbmRhoNonFinite                              */
    int64_t u_limited;           /* lbmULimited                                  */
    int64_t nan_count;           /* nanCount of the last step                    */
    double  sum_rho;             /* raw FP64 sums of the last step               */
    double  sum_kinetic;
    double  sum_tke;
    float   nusselt;             /* thermalNusselt (FP64 row sum)                */
    float   mean_t;              /* thermalMeanT                                 */
    int32_t fluid_cells;
    int32_t pad1;
} aeros_lbm_stats;

typedef struct aeros_lbm aeros_lbm;   /* opaque solver handle (one domain) */

/* ---- errors --------------------------------------------------------------- */
/* Replaces cudaConsumeError (aeros/src/cuda_api.h:56): returns the last error
 * code (0 = none), copies its message into buf, clears it. Thread-local. */
int aeros_consume_error(char* buf, int buf_size);

/* ---- lifecycle ------------------------------------------------------------- */
/* Replaces initLBM (aeros/src/lbm.cpp:405-886) once the host has resolved the
 * domain: mask (nx*ny*nz bytes, AEROS_CELL_*), wall-distance chamfer
 * (lbm.cpp:647-675), fluid count (:677-680), equilibrium at u_init
 * (:686-739). Allocates all device memory. */
int aeros_lbm_create(const aeros_lbm_params* params, const uint8_t* mask,
                     aeros_lbm** out);
/* Replaces shutdownLBM (aeros/src/lbm.cpp:894-904) + cudaReleaseAll. */
int aeros_lbm_destroy(aeros_lbm* h);

/* Stream the handle launches on (a cudaStream_t; NULL = legacy default). */
int aeros_lbm_set_stream(aeros_lbm* h, void* cuda_stream);
int aeros_lbm_synchronize(aeros_lbm* h);

/* Replaces thermalInit (aeros/src/thermal_lbm.cpp:84-140): alpha, tau_T, g,
 * H from the mask, conduction profile + cos*sin seed. */
int aeros_lbm_thermal_init(aeros_lbm* h, const aeros_thermal_params* tp);

/* ---- stepping --------------------------------------------------------------- */
/* Replaces stepLBMCPU(steps) (aeros/src/lbm.cpp:907-1709) minus the readback
 * prep: LES pre-pass, collision, stream + BCs, thermal step, per-step stats,
 * divergence guard + re-equilibration. Enqueued on the handle's stream; the
 * call waits for the final stats (one device->host read per call). */
int aeros_lbm_step(aeros_lbm* h, int nsteps);
/* Same, without the final wait; stats are read by aeros_lbm_get_stats. */
int aeros_lbm_step_async(aeros_lbm* h, int nsteps);
int aeros_lbm_get_stats(aeros_lbm* h, aeros_lbm_stats* out);

/* ---- state I/O (host buffers, nx*ny*nz elements each unless stated) ------- */
/* Field readback (lbmRho, lbmUx/Uy/Uz, lbmStrainMag, lbmTKEField; lbm.h:132-152).
 * Any pointer may be NULL. */
int aeros_lbm_read_fields(aeros_lbm* h, float* rho, float* ux, float* uy,
                          float* uz, float* strain, float* tke);
/* Page-locked host memory for readback targets (no reference counterpart:
 * the reference's fields are std::vector mirrors). A copy into pageable
 * memory goes through the driver's staging buffer at a fraction of the link
 * speed; into these buffers aeros_lbm_read_fields copies each field with one
 * direct DMA. aeros_host_free releases a buffer from aeros_host_alloc. */
int aeros_host_alloc(size_t bytes, void** out);
int aeros_host_free(void* p);
/* Device pointers of the density and of the velocity, interleaved as
 * (ux, uy, uz, 0) per cell (valid until the next step call). Either may be
 * NULL. */
int aeros_lbm_device_fields(aeros_lbm* h, const float** rho, const float** u4);
/* Pre-collision populations, layout [19][nx*ny*nz] (the reference's f after
 * stepLBMCPU, lbm.cpp:89,1546). Converted to FP32 for shifted storage. */
int aeros_lbm_read_populations(aeros_lbm* h, float* f);
/* Overwrite pre-collision populations (checkpoint restore / fault injection). */
int aeros_lbm_write_populations(aeros_lbm* h, const float* f);
/* Equilibrium re-initialisation from per-cell rho and u (fluid cells; rho may
 * be NULL = 1). |u| limited to 0.3 as initLBM does (lbm.cpp:725-730). */
int aeros_lbm_set_equilibrium(aeros_lbm* h, const float* rho, const float* ux,
                              const float* uy, const float* uz);
int aeros_lbm_read_mask(aeros_lbm* h, uint8_t* mask, uint8_t* wall_dist);

/* ---- thermal ---------------------------------------------------------------- */
/* Replaces thermalUpload (aeros/src/thermal_lbm.cpp:187-197). */
int aeros_lbm_thermal_upload(aeros_lbm* h, const float* T);
/* thermalT and thermalBuoyancyY (thermal_lbm.h:46-49). Either may be NULL. */
int aeros_lbm_thermal_read(aeros_lbm* h, float* T, float* buoyancy);

/* ---- forces ------------------------------------------------------------------ */
/* Replaces lbmControlVolumeForce (aeros/src/lbm.cpp:2183-2232): box centred on
 * the domain centre, half sizes as fractions of N, FP64 accumulation. */
int aeros_lbm_cv_force(aeros_lbm* h, float half_x, float half_y, float half_z,
                       double out[3]);
/* Same momentum balance on an explicit box [x0,x1]x[y0,y1]x[z0,z1] (cells,
 * inclusive; not in the reference, which only centres the box). */
int aeros_lbm_cv_force_box(aeros_lbm* h, const int32_t box[6], double out[3]);
/* Replaces lbmProjectedAreaCells (aeros/src/lbm.cpp:2236-2256). */
int aeros_lbm_projected_area(aeros_lbm* h, int axis, double* area);

/* lbmEquilibriumMoments (aeros/src/lbm.cpp:249-267), evaluated on the device
 * with the equilibrium the solver's kernels use (computeEquilibriumFast,
 * lbm.cpp:146-184, velocity limiter included): for n states
 * states[4i..4i+3] = (rho, ux, uy, uz), out[4i..4i+3] = the sum of the 19
 * equilibrium populations and their three momentum sums, each accumulated in
 * FP32 over q = 0..18 as the reference does. ok[i] = 0 where an input or a
 * population is not finite (the reference's false); out is then 0. No
 * handle: a validation helper on the current device. */
int aeros_equilibrium_moments(const float* states, int64_t n, float* out, uint8_t* ok);

/* ---- voxelizer ------------------------------------------------------------------ */
typedef struct aeros_voxel_grid {
    int32_t nx, ny, nz;
    float   min[3];              /* lower corner                      */
    float   cell[3];             /* cell size; centre = min + (i+0.5)*cell */
} aeros_voxel_grid;

/* Solid mask of a closed triangle mesh at the grid's cell centres: the
 * three-ray parity vote with FP64 Moller-Trumbore of the reference's inside
 * test (aeros/src/mesh_bvh.h:62-96,168-185), the mask loop of buildVoxelGrid
 * (aeros/src/voxel_grid.cpp:337-351); the same mask bit for bit. Rays are
 * traced once per grid row through a Morton-code BVH; each cell evaluates the
 * row's candidate triangles from its own origin. tris: ntri*9 floats.
 * mask_out: nx*ny*nz bytes, 1 = inside. Degenerate / non-finite triangles are
 * dropped as voxel_grid.cpp:313-325 does. */
int aeros_voxelize(const float* tris, int64_t ntri, const aeros_voxel_grid* grid,
                   uint8_t* mask_out);
/* Same with a device-resident output mask (nx*ny*nz bytes). */
int aeros_voxelize_device(const float* tris, int64_t ntri,
                          const aeros_voxel_grid* grid, uint8_t* d_mask_out);
/* No reference counterpart. aeros_voxelize_device without device allocation,
 * for callers that cannot allocate while they voxelize (a serving loop whose
 * HBM budget is spent on resident domains; callers whose other streams must
 * not be stalled by the device-wide synchronization of cudaFree). BVH,
 * triangles and overflow flag live in one fixed 24 MiB device array per
 * device, present from the library's load on (the level-7 icosphere's
 * 327,680 triangles fit, about 36 bytes per triangle plus 32 per BVH node); a
 * larger mesh returns AEROS_ERR_INVALID before any device work. All work runs
 * on `stream` (a cudaStream_t; NULL = the legacy default stream, which
 * synchronizes with the device's blocking streams), and the call returns
 * after it has completed there. Calls share the array: they must not overlap
 * in time. The array's address is looked up on every call, before any work is
 * queued. Same mask as aeros_voxelize_device. */
int aeros_voxelize_device_noalloc(const float* tris, int64_t ntri,
                                  const aeros_voxel_grid* grid, uint8_t* d_mask, void* stream);

/* ---- signed distance field -------------------------------------------------------- */
/* The voxel grid's signed distance field (the distance-field part of
 * buildVoxelGrid, aeros/src/voxel_grid.cpp:384-553) on the device. Seeds:
 * cells with a 6-neighbour of the other solidity (mask == 1 is solid; other
 * values are not) start at -0.5 (solid) or +0.5 of the smallest cell size,
 * the rest at +1e6. Propagation over the 26 neighbours with the weights
 * sqrtf(wx^2 + wy^2 + wz^2) runs to its least fixed point: the float
 * shortest-path length from a seed, with that seed's sign (negative on
 * equal lengths). The reference's four sweeps and 1e-3 FIFO stop short of
 * that limit (same signs; on the test meshes 99.99 % of the cells within
 * 1e-4, all within 2e-3).
 * Then the reference's two rounds of x, y, z smoothing beyond 3 cells.
 * Device mask and output, nx*ny*nz each; stream: a cudaStream_t or NULL.
 * Returns when the field is complete. AEROS_ERR_TIMEOUT if the propagation
 * has not converged after 4 (nx + ny + nz) + 64 passes. */
int aeros_sdf_device(const uint8_t* d_mask, const aeros_voxel_grid* grid, float* d_sdf, void* stream);
/* Same with a host mask and a host output field. */
int aeros_sdf(const uint8_t* mask, const aeros_voxel_grid* grid, float* sdf);
/* sampleSDFCPU / sdfNormalCPU (voxel_grid.cpp:32-123) of a device field at n
 * world points (host xyz): trilinear between cell centres, 1000 outside the
 * grid; the unit normal from central differences (half the smallest cell),
 * falling back to the cell gradient. dist (n) and normal (3n) are host
 * arrays; either may be NULL. d_sdf NULL: 1000 and (0, 1, 0), as the
 * reference without a field. */
int aeros_sdf_sample(const float* d_sdf, const aeros_voxel_grid* grid, const float* points, int64_t n,
                     float* dist, float* normal);
/* A field built on the device and kept there (the reference keeps
 * g_distanceField for its samplers): create from a host mask, read back,
 * sample (aeros_sdf_sample on the field's own device array and grid),
 * destroy. */
typedef struct aeros_sdf_field aeros_sdf_field;
int aeros_sdf_field_create(const uint8_t* mask, const aeros_voxel_grid* grid, aeros_sdf_field** out);
int aeros_sdf_field_destroy(aeros_sdf_field* field);
const float* aeros_sdf_field_device(const aeros_sdf_field* field);   /* NULL for NULL */
int aeros_sdf_field_read(const aeros_sdf_field* field, float* sdf);
int aeros_sdf_field_sample(const aeros_sdf_field* field, const float* points, int64_t n, float* dist,
                           float* normal);
/* Propagation passes and tile runs (8x8x8 tiles) of the calling thread's
 * last distance-field build. No reference counterpart: diagnostics. */
int aeros_sdf_last_stats(int64_t* passes, int64_t* tile_runs);

/* ---- STL ingest ------------------------------------------------------------------- */
/* Format detection by content (stlformat::detect, aeros/src/stl_format.h:86-140):
 * ASCII when the file starts with "solid" and holds facet / vertex keywords;
 * else binary when the 80-byte header's triangle count fits the data (a tail
 * after the triangles is allowed); else ASCII for keyword text without
 * "solid"; else unknown (truncated binary, text without keywords, other). */
enum { AEROS_STL_UNKNOWN = 0, AEROS_STL_BINARY = 1, AEROS_STL_ASCII = 2 };
enum {
    AEROS_STL_REASON_EMPTY = 0,
    AEROS_STL_REASON_ASCII = 1,              /* "solid" + facet/vertex               */
    AEROS_STL_REASON_BINARY = 2,             /* size matches the count exactly       */
    AEROS_STL_REASON_BINARY_TAIL = 3,        /* trailing bytes after the triangles   */
    AEROS_STL_REASON_TEXT_NO_SOLID = 4,      /* keyword text without "solid"         */
    AEROS_STL_REASON_TEXT_NO_KEYWORDS = 5,   /* text without facet/vertex (unknown)  */
    AEROS_STL_REASON_TRUNCATED = 6,          /* the count promises more than there is */
    AEROS_STL_REASON_UNRECOGNIZED = 7
};
typedef struct aeros_stl_info {
    int32_t  format;               /* AEROS_STL_*                                     */
    int32_t  reason;               /* AEROS_STL_REASON_*                              */
    uint32_t declared_triangles;   /* header count (binary files)                     */
    uint32_t reserved0;
    uint64_t payload_bytes;        /* 50 per declared triangle (binary)               */
    uint64_t trailing_bytes;       /* after the last triangle (binary)                */
    int64_t  triangles;            /* triangles parsed (after aeros_stl_parse)        */
    int64_t  dropped;              /* binary: triangles with a non-finite coordinate;
                                      ASCII: non-finite vertices, rounded down to 3s  */
} aeros_stl_info;
int aeros_stl_detect(const uint8_t* data, uint64_t size, aeros_stl_info* info);
/* loadSTL's parse (aeros/src/stl_loader.cpp:30-223) of an in-memory file.
 * Binary: each normal made finite and unit ((0, 0, 1) when not), triangles
 * with a non-finite coordinate dropped. ASCII: vertex lines in threes (the
 * number extraction of the C++ standard library streams), each triangle's
 * normal from its edges ((0, 1, 0) when degenerate). vertices gets 9 floats
 * per triangle, normals 9 per triangle (the normal once per vertex); either
 * may be NULL; at most `capacity` triangles are written while
 * info->triangles counts them all (call with capacity 0 to size the
 * buffers). budget: refuse a binary file whose vertices + normals need more
 * bytes (0: no limit; the reference uses half of the available RAM). Files
 * under 10 bytes or over 2 GiB, unknown formats and files without a usable
 * triangle return AEROS_ERR_INVALID. */
int aeros_stl_parse(const uint8_t* data, uint64_t size, uint64_t budget, float* vertices, float* normals,
                    int64_t capacity, aeros_stl_info* info);
/* Same for a file path. */
int aeros_stl_read_file(const char* path, uint64_t budget, float* vertices, float* normals, int64_t capacity,
                        aeros_stl_info* info);

/* Grid plan (aeros/src/voxel_grid.cpp:172-215): dimensions for a bounding box
 * and resolution against a byte budget (0 = unlimited). */
typedef struct aeros_voxel_plan_t {
    int32_t nx, ny, nz;
    int32_t fits;
    int64_t cells;
    uint64_t bytes;
    int32_t requested_res;
    int32_t suggested_res;
} aeros_voxel_plan_t;
int aeros_voxel_plan(const float size[3], int res, uint64_t budget_bytes,
                     aeros_voxel_plan_t* out);

/* ---- readback and post-processing on the device --------------------------------
 * World units of the visualizer: the fields stay on the device, the host
 * arrays below are optional (NULL: not copied). */
typedef struct aeros_world_params {
    float flow_speed;        /* freestream speed, m/s (flowSpeed)                    */
    float air_density;       /* kg/m^3 (airDensity)                                   */
    float min[3];            /* world position of the grid origin (lbmMinX..)         */
    float cell[3];           /* world cell size (lbmCellSizeX..)                      */
    int32_t reserved[4];
} aeros_world_params;

typedef struct aeros_world_stats {
    float pressure_min, pressure_max;   /* lbmPressureMin / lbmPressureMax (strided) */
    float residual_rho;                 /* lbmResidualRho: RMS of rho change since the last call */
    float residual_u;                   /* lbmResidualU: change of max |u| since the last call */
    int64_t pressure_non_finite;        /* lbmPressureNonFinite                      */
} aeros_world_stats;

/* Replaces the readback prep at the end of stepLBMCPU (aeros/src/lbm.cpp:1602-1705)
 * for the state of the last step: world velocity u * flow_speed / |u_in|
 * and pressure rho0 cs2 (rho - 1) scale^2 (zero on body and ground cells),
 * pressure min / max over at most 262,144 strided cells, the density
 * residual against the previous call and the change of max |u|. */
int aeros_lbm_world_fields(aeros_lbm* h, const aeros_world_params* wp, float* ux, float* uy, float* uz,
                           float* pressure, aeros_world_stats* stats);
/* Replaces computeLBMVorticityAndQ (aeros/src/lbm.cpp:2005-2093): |curl u|,
 * the Q criterion and sqrt(2 S:S) from the world velocity of the last
 * aeros_lbm_world_fields call (central differences, interior cells; the
 * strain also replaces the step's |S| there, as in the reference). */
int aeros_lbm_vorticity_q(aeros_lbm* h, float* vorticity, float* q, float* strain);

enum {
    AEROS_FIELD_VELOCITY_LB = 0,   /* getLBMVelocityLB (lbm.cpp:1782-1840): 3 values per point */
    AEROS_FIELD_DENSITY = 1,       /* sampleFieldTrilinear (lbm.cpp:1881-1933) of lbmRho   */
    AEROS_FIELD_PRESSURE = 2,      /* ... of lbmPressure                                    */
    AEROS_FIELD_VORTICITY = 3,
    AEROS_FIELD_Q = 4,
    AEROS_FIELD_STRAIN = 5,
    AEROS_FIELD_TKE = 6,
    AEROS_FIELD_SOLID = 7          /* isLBMSolidWorld (lbm.cpp:1954-1969): 1 or 0          */
};
/* Samples a field at n world points (xyz each) on the device, with the
 * reference's trilinear rules (solid corners skipped, weights renormalised).
 * out: n values (3n for the velocity); valid (optional): 1 where the
 * reference's sampler reports data. */
int aeros_lbm_sample(aeros_lbm* h, const aeros_world_params* wp, int field, const float* points, int64_t n,
                     float* out, uint8_t* valid);

/* ---- surface-pressure lift and drag ------------------------------------------------
 * Replaces computeLiftDrag (aeros/src/forces.cpp:401-688) with the LBM branch
 * of its per-triangle pass (the analytic-flow branch is not on the solver
 * path): the pressure of the last aeros_lbm_world_fields call is sampled per
 * triangle 0.6 LBM cells out along the triangle's normal (wallSamplePoint,
 * forces.cpp:75-90), Cp with the Karman-Tsien correction, pressure force,
 * Blasius / Schlichting skin friction, moment about the quarter chord and the
 * pressure-weighted centre; then base, induced and wave drag, ground effect
 * and the frontal reference area as the reference. The per-triangle pass runs
 * on the device (sums in FP64, a fixed reduction order); the scalar set-up and
 * the closing formulas run on the host in FP32 as the reference's. */
typedef struct aeros_surface_mesh aeros_surface_mesh;
/* Uploads a triangle soup: vertices 9 floats per triangle (g_vertices) and
 * per-vertex normals 9 floats per triangle (g_normals; the pass reads the
 * first vertex's normal of each triangle, as the reference). ntri may be 0
 * (no model: the pass returns AEROS_SURFACE_NOT_RUN). */
int aeros_surface_mesh_create(const float* vertices, const float* normals, int64_t ntri,
                              aeros_surface_mesh** out);
int aeros_surface_mesh_destroy(aeros_surface_mesh* mesh);

typedef struct aeros_surface_params {
    float velocity[3];          /* flowParams.vx, vy, vz (m/s)                              */
    float air_temperature;      /* flowParams.airTemperature (K), Sutherland viscosity       */
    float air_density;          /* flowParams.airDensity (kg/m^3)                            */
    int32_t use_real_density;   /* useRealDensity: else 1.225                                */
    float speed_of_sound;       /* speedOfSound (m/s)                                        */
    int32_t mach_effects;       /* aeroMachEffects: Karman-Tsien for 0.3 < M < 0.85, wave drag */
    int32_t auto_ref_area;      /* aeroAutoRefArea: projected area from the flow angles       */
    float ref_area;             /* aeroRefArea when auto_ref_area is 0                        */
    float flow_azimuth_deg;     /* flowAzimuth (computeLBMRefArea's direction, lbm.cpp:2111)  */
    float flow_elevation_deg;   /* flowElevation                                              */
    float bb_min[3], bb_max[3]; /* minBB, maxBB: model bounds (span and chord estimates)      */
    float center[3];            /* center: model centre                                       */
    float max_dim;              /* maxDim                                                     */
    float reynolds;             /* aeroReNumber (open-base correction above 1e6)              */
    int32_t ground_effect;      /* aeroGroundEffect                                           */
    float ground_height;        /* aeroGroundHeight, above vox_min_y                          */
    float vox_min_y;            /* g_voxMinY                                                  */
    int32_t reserved[4];
} aeros_surface_params;

enum {
    AEROS_SURFACE_NOT_RUN = 0,   /* the reference returns before writing (no usable mesh)  */
    AEROS_SURFACE_NO_FLOW = 1,   /* flow direction undefined: lift, drag and L/D are 0     */
    AEROS_SURFACE_DONE = 2
};

typedef struct aeros_surface_forces {
    int32_t status;             /* AEROS_SURFACE_*                                          */
    int32_t reserved0;
    float drag, lift;           /* dragMagnitude, liftMagnitude (N)                         */
    float lift_to_drag;         /* liftToDragRatio                                          */
    float moment_magnitude;     /* momentMagnitude (N m)                                    */
    float drag_vector[3], lift_vector[3], moment[3];
    float center_of_pressure[3];
    float ref_area;             /* aeroRefArea after the call                               */
    float ref_area_used;        /* the area the coefficients used                           */
    int64_t cp_non_finite;      /* aeroCpNonFinite                                          */
    /* per-triangle sums of the pass (FP64): force xyz, pressure-weighted centre
     * xyz, moment xyz, area, pressure weight, frontal, base area, base force,
     * projected area of computeLBMRefArea */
    double sums[15];
} aeros_surface_forces;

/* cp: optional host array, one value per triangle (the Cp the pass used;
 * 0 for skipped triangles). d_sdf / sdf_grid: the voxel grid's distance
 * field on the device (both NULL: no field, the sample point is never held
 * back). A mesh holds the pass's scratch: passes that share a mesh must not
 * run at the same time (one host thread, or one mesh per thread). Returns
 * after the pass, on the handle's stream. */
int aeros_lbm_surface_forces(aeros_lbm* h, const aeros_world_params* wp, const aeros_surface_params* sp,
                             const aeros_surface_mesh* mesh, const float* d_sdf, const aeros_voxel_grid* sdf_grid,
                             aeros_surface_forces* out, float* cp);

/* ---- timing helper for benches ------------------------------------------------ */
/* Milliseconds of the step kernels enqueued by the last aeros_lbm_step*/
/* call, measured with CUDA events on the handle's stream. */
int aeros_lbm_last_step_ms(aeros_lbm* h, float* ms);
/* Number of kernels the last aeros_lbm_step* call launched. */
int aeros_lbm_last_launch_count(aeros_lbm* h, int64_t* n);
/* Bytes of device memory the handle holds. */
int aeros_lbm_device_bytes(aeros_lbm* h, uint64_t* bytes);

#ifdef __cplusplus
}
#endif
#endif /* AEROS_LBM_H */
