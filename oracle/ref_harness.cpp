// ref_harness.cpp — drives the reference's OWN solver sources (TEST
// INFRASTRUCTURE ONLY). oracle/Makefile compiles this translation unit
// together with the reference sources where they lie (never copied into this
// repository) into oracle/_ref/libaeros_ref.so; tests/golden/make_golden.py
// uses it to pin the C restatement (lbm_oracle.c) and to write the golden
// fixtures under tests/golden/.
//
// The solver's state (f, fNext, lbmWallDist, the thermal populations) is
// file-static in the reference, so the two solver files are included into
// this unit, the way the reference's own headless tests link them with stubs
// for GL/GLFW/CUDA (aeros/tests/physics_ref_headless.cpp:40-45).
#include "lbm.cpp"
#include "thermal_lbm.cpp"
#include "forces.cpp"

#include <cstdint>
#include <omp.h>
#include <cstring>

#include "mesh_bvh.h"
#include "stl_format.h"
#include "stl_loader.h"

extern "C" double glfwGetTime(void) { static double t = 0.0; return (t += 1.0 / 60.0); }
extern "C" void setVoxelData(const int*, const float*, int, int, int, float, float, float, float, float, float) {}
extern "C" int cudaConsumeError(char* buf, int sz) { if (buf && sz > 0) buf[0] = 0; return 0; }
void drawModel() {}
extern "C" void computeVertexPressureCUDA(const std::vector<float>&, const std::vector<float>&, std::vector<float>&, int,
                                          const FlowParams&) {}

// forces.cpp (computeLiftDrag) is included as well. Its vertex-colour and
// arrow uploads are GL calls behind glBackendActive(); reporting the Vulkan
// backend keeps them off, and the function pointers it names are null
// stubs, as in the reference's headless test builds.
bool isRendererVulkan() { return true; }
PFNGLBINDBUFFERPROC glad_glBindBuffer = nullptr;
PFNGLBINDVERTEXARRAYPROC glad_glBindVertexArray = nullptr;
PFNGLBUFFERDATAPROC glad_glBufferData = nullptr;
PFNGLBUFFERSUBDATAPROC glad_glBufferSubData = nullptr;
PFNGLENABLEVERTEXATTRIBARRAYPROC glad_glEnableVertexAttribArray = nullptr;
PFNGLGENBUFFERSPROC glad_glGenBuffers = nullptr;
PFNGLGENVERTEXARRAYSPROC glad_glGenVertexArrays = nullptr;
PFNGLVERTEXATTRIBPOINTERPROC glad_glVertexAttribPointer = nullptr;

extern "C" {

// Grid of one cell per world unit starting at 0, domain padding 0: the solver
// grid equals the mask grid (dimensions >= 8, lbm.cpp:505). Ground: rows
// y <= ground_rows-1 (lbm.cpp:624-643). Flow direction from axis/sign via the
// reference's own azimuth/elevation path. u0 = |inlet| (the reference forces
// 0.08 when u0 < 1e-6, lbm.cpp:196). Returns 0 on success and writes the
// inlet velocity the reference derived.
int ref_lbm_setup(int nx, int ny, int nz, const uint8_t* solid, int ground_rows,
                  float tau, float u0, float smag, int les, int trt,
                  int periodic_x, int periodic_z, int convective, int flow_axis, int flow_sign,
                  const float* body_force, float flow_speed, float* u_in_out) {
    g_voxNx = nx; g_voxNy = ny; g_voxNz = nz;
    g_voxMinX = 0.0f; g_voxMinY = 0.0f; g_voxMinZ = 0.0f;
    g_voxMaxX = (float)nx; g_voxMaxY = (float)ny; g_voxMaxZ = (float)nz;
    g_voxelData.assign((size_t)nx * ny * nz, 0);
    g_distanceField.assign((size_t)nx * ny * nz, 0.0f);
    for (size_t i = 0; i < (size_t)nx * ny * nz; ++i) g_voxelData[i] = solid[i] ? 1 : 0;
    minBB = glm::vec3(0.0f); maxBB = glm::vec3((float)nx, (float)ny, (float)nz);
    center = 0.5f * maxBB; maxDim = (float)std::max(nx, std::max(ny, nz));
    voxelResolution = nx;
    flowSpeed = flow_speed;
    flowAzimuth = 0.0f; flowElevation = 0.0f;
    if (flow_axis == 0 && flow_sign < 0) flowAzimuth = 180.0f;
    if (flow_axis == 2) flowAzimuth = flow_sign > 0 ? 90.0f : -90.0f;
    if (flow_axis == 1) flowElevation = flow_sign > 0 ? 90.0f : -90.0f;
    altitude = 0.0f; timeScale = 1.0f; aeroMachEffects = false; aeroGroundEffect = false;
    lbmParams.enabled = true;
    lbmParams.useGPU = false;
    lbmParams.U0 = u0;
    lbmParams.stepsPerFrame = 1;
    lbmParams.tau = tau;
    lbmParams.smagorinskyC = smag;
    lbmParams.useTurbulence = les != 0;
    lbmParams.useTRT = trt != 0;
    lbmParams.useGround = ground_rows > 0;
    lbmParams.groundHeight = ground_rows > 0 ? (float)ground_rows - 0.5f : 0.0f;
    lbmParams.inletTurbulence = 0.0f;
    lbmParams.domainPadding = 0.0f;
    lbmParams.autoViscosity = false;
    lbmParams.useConvectiveOutlet = convective != 0;
    lbmParams.periodicX = periodic_x != 0;
    lbmParams.periodicZ = periodic_z != 0;
    lbmParams.bodyForceX = body_force[0];
    lbmParams.bodyForceY = body_force[1];
    lbmParams.bodyForceZ = body_force[2];
    lbmParams.convergenceThreshold = 1e-5f;
    thermalParams.enabled = false;   // thermal is attached by ref_thermal_setup
    shutdownLBM();
    initLBM();
    if (!lbmInitialized) return -1;
    if (lbmNx != nx || lbmNy != ny || lbmNz != nz) return -2;
    float ux, uy, uz;
    computeInletVelocityLB(ux, uy, uz);
    u_in_out[0] = ux; u_in_out[1] = uy; u_in_out[2] = uz;
    return 0;
}

// Thermal module on the current grid (thermalInit through initLBM's call
// site, lbm.cpp:876-885).
int ref_thermal_setup(float rayleigh, float prandtl, int fixed, float hot, float cold, float perturbation) {
    thermalParams.enabled = true;
    thermalParams.rayleigh = rayleigh;
    thermalParams.prandtl = prandtl;
    thermalParams.fixedWallTemps = fixed != 0;
    thermalParams.hotTemp = hot;
    thermalParams.coldTemp = cold;
    thermalParams.perturbation = perturbation;
    std::vector<char> m(lbmIsSolid.begin(), lbmIsSolid.end());
    for (size_t i = 0; i < m.size(); ++i) if (lbmIsGround[i]) m[i] = 1;
    return thermalInit(lbmNx, lbmNy, lbmNz, m, lbmParams.viscosity) ? 0 : -1;
}

void ref_thermal_disable() { thermalParams.enabled = false; thermalShutdown(); }

int ref_thermal_upload(const float* T) {
    std::vector<float> v(T, T + (size_t)lbmNx * lbmNy * lbmNz);
    return thermalUpload(v) ? 0 : -1;
}

void ref_thermal_get(float* T, float* buoy, float* nusselt, float* mean_t) {
    const size_t n = (size_t)lbmNx * lbmNy * lbmNz;
    if (T) std::memcpy(T, thermalT.data(), n * sizeof(float));
    if (buoy) std::memcpy(buoy, thermalBuoyancyY.data(), n * sizeof(float));
    if (nusselt) *nusselt = thermalNusselt;
    if (mean_t) *mean_t = thermalMeanT;
}

// Overwrite the initial populations with the equilibrium at u_init for fluid
// cells (the reference cannot start from rest: lbm.cpp:196).
void ref_lbm_set_uniform(float ux, float uy, float uz) {
    const int total = lbmNx * lbmNy * lbmNz;
    float usqr = ux * ux + uy * uy + uz * uz;
    for (int c = 0; c < total; ++c) {
        if (lbmIsSolid[c] || lbmIsGround[c]) continue;
        for (int q = 0; q < Q; ++q) f[(size_t)c * Q + q] = computeEquilibriumFast(q, 1.0f, ux, uy, uz, usqr);
    }
}

// One call per step: stepLBMCPU(n) with n > 1 keeps the raw population
// pointers taken before its first swap (lbm.cpp:937-938 vs :1546), so only
// single-step calls advance the lattice correctly; every reference test and
// the reference bench call it with 1.
void ref_lbm_step(int n) { for (int i = 0; i < n; ++i) stepLBMCPU(1); }

void ref_lbm_get_fields(float* rho, float* ux, float* uy, float* uz, float* strain, float* tke) {
    const size_t n = (size_t)lbmNx * lbmNy * lbmNz;
    if (rho) std::memcpy(rho, lbmRho.data(), n * 4);
    if (ux) std::memcpy(ux, lbmUx.data(), n * 4);
    if (uy) std::memcpy(uy, lbmUy.data(), n * 4);
    if (uz) std::memcpy(uz, lbmUz.data(), n * 4);
    if (strain) std::memcpy(strain, lbmStrainMag.data(), n * 4);
    if (tke) std::memcpy(tke, lbmTKEField.data(), n * 4);
}

// Pre-collision populations, written SoA [19][cells].
void ref_lbm_get_populations(float* out) {
    const size_t n = (size_t)lbmNx * lbmNy * lbmNz;
    for (size_t c = 0; c < n; ++c)
        for (int q = 0; q < Q; ++q) out[(size_t)q * n + c] = f[c * Q + q];
}

void ref_lbm_set_populations(const float* in) {
    const size_t n = (size_t)lbmNx * lbmNy * lbmNz;
    for (size_t c = 0; c < n; ++c)
        for (int q = 0; q < Q; ++q) f[c * Q + q] = in[(size_t)q * n + c];
}

void ref_lbm_get_wall_dist(uint8_t* out) {
    std::memcpy(out, lbmWallDist.data(), lbmWallDist.size());
}

// Scalars of the last step: avgRho, KE, maxU, TKE, convergence, converged,
// step, negPops, badPops, rhoOut, rhoNonFin, uLim.
void ref_lbm_stats(float* fs, long long* is) {
    fs[0] = lbmAvgRho; fs[1] = lbmAvgKineticEnergy; fs[2] = lbmMaxVelocityLB; fs[3] = lbmTKE;
    fs[4] = lbmConvergence; fs[5] = lbmConverged ? 1.0f : 0.0f;
    is[0] = lbmCurrentStep; is[1] = lbmNegativePops; is[2] = lbmBadPops; is[3] = lbmRhoOutOfRange;
    is[4] = lbmRhoNonFinite; is[5] = lbmULimited;
}

void ref_lbm_cv_force(float hx, float hy, float hz, float* out) {
    glm::vec3 F = lbmControlVolumeForce(hx, hy, hz);
    out[0] = F.x; out[1] = F.y; out[2] = F.z;
}

float ref_lbm_projected_area(int axis) { return lbmProjectedAreaCells(axis); }

int ref_equilibrium_moments(float rho, float ux, float uy, float uz, float* out4) {
    return lbmEquilibriumMoments(rho, ux, uy, uz, &out4[0], &out4[1], &out4[2], &out4[3]) ? 1 : 0;
}

// The voxelizer's mask loop (voxel_grid.cpp:313-351) at explicit cell centres.
int ref_voxelize(const float* tris, long long ntri, int nx, int ny, int nz,
                 const float* mn, const float* cs, uint8_t* mask) {
    std::vector<meshbvh::Triangle> tv;
    tv.reserve((size_t)ntri);
    for (long long i = 0; i < ntri; ++i) {
        const float* v = tris + 9 * i;
        const glm::vec3 a(v[0], v[1], v[2]), b(v[3], v[4], v[5]), c(v[6], v[7], v[8]);
        if (!std::isfinite(a.x) || !std::isfinite(a.y) || !std::isfinite(a.z) ||
            !std::isfinite(b.x) || !std::isfinite(b.y) || !std::isfinite(b.z) ||
            !std::isfinite(c.x) || !std::isfinite(c.y) || !std::isfinite(c.z)) continue;
        meshbvh::Triangle t = meshbvh::makeTriangle(a, b, c);
        if (meshbvh::isDegenerate(t)) continue;
        tv.push_back(t);
    }
    meshbvh::BVH bvh;
    if (!tv.empty()) bvh.build(tv);
    const glm::vec3 cell(cs[0], cs[1], cs[2]);
    std::memset(mask, 0, (size_t)nx * ny * nz);
    if (tv.empty()) return 0;
#pragma omp parallel for collapse(3) schedule(dynamic, 4)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const glm::vec3 p(mn[0] + (i + 0.5f) * cs[0], mn[1] + (j + 0.5f) * cs[1], mn[2] + (k + 0.5f) * cs[2]);
                if (bvh.inside(p, cell)) mask[((size_t)k * ny + j) * nx + i] = 1;
            }
    return (int)bvh.nodeCount();
}

int ref_count_hits(const float* tris, long long ntri, const float* o, int axis) {
    std::vector<meshbvh::Triangle> tv;
    for (long long i = 0; i < ntri; ++i) {
        const float* v = tris + 9 * i;
        meshbvh::Triangle t = meshbvh::makeTriangle(glm::vec3(v[0], v[1], v[2]), glm::vec3(v[3], v[4], v[5]),
                                                    glm::vec3(v[6], v[7], v[8]));
        if (meshbvh::isDegenerate(t)) continue;
        tv.push_back(t);
    }
    meshbvh::BVH bvh;
    bvh.build(tv);
    glm::vec3 d(axis == 0 ? 1.0f : 0.0f, axis == 1 ? 1.0f : 0.0f, axis == 2 ? 1.0f : 0.0f);
    return bvh.countIntersections(glm::vec3(o[0], o[1], o[2]), d);
}

void ref_voxel_plan(const float* size, int res, unsigned long long budget, int* out6) {
    VoxelPlan p = voxelPlan(glm::vec3(size[0], size[1], size[2]), res, budget);
    out6[0] = p.nx; out6[1] = p.ny; out6[2] = p.nz; out6[3] = p.fits ? 1 : 0;
    out6[4] = p.suggestedRes; out6[5] = (int)p.cells;
}

// The validation case set-up of aeros/tests/validation_headless.cpp:57-81 and
// :99-129 (sphere / cylinder voxel mask on a [-3,3]^3 box of res^3 cells,
// padded domain, BGK, convective outlet), restated here to export the solver
// grid the reference builds from it. Writes nx, ny, nz, the tau the solver
// uses and the inlet velocity.
int ref_validation_setup(int shape, int res, float radius, int diameter_cells, float re_lat, float pad,
                         float u0, int* dims, float* tau_out, float* uin_out) {
    flowSpeed = 20.0f; flowAzimuth = 0.0f; flowElevation = 0.0f;
    altitude = 0.0f; timeScale = 1.0f; aeroMachEffects = false; aeroGroundEffect = false;
    lbmParams = LBMParams();
    lbmParams.enabled = true;
    lbmParams.useGPU = false;
    lbmParams.U0 = u0;
    lbmParams.stepsPerFrame = 1;
    lbmParams.useTurbulence = false;
    lbmParams.useGround = false;
    lbmParams.inletTurbulence = 0.0f;
    lbmParams.domainPadding = pad;
    lbmParams.autoViscosity = false;
    voxelResolution = res;
    float tau = 0.5f + 3.0f * u0 * (float)diameter_cells / re_lat;
    tau = std::max(0.505f, std::min(tau, 1.4f));
    lbmParams.tau = tau;
    g_voxNx = g_voxNy = g_voxNz = res;
    g_voxMinX = g_voxMinY = g_voxMinZ = -3.0f;
    g_voxMaxX = g_voxMaxY = g_voxMaxZ = 3.0f;
    const float cs = 6.0f / (float)res;
    g_voxelData.assign((size_t)res * res * res, 0);
    g_distanceField.assign((size_t)res * res * res, 0.0f);
    for (int z = 0; z < res; ++z)
        for (int y = 0; y < res; ++y)
            for (int x = 0; x < res; ++x) {
                const float px = g_voxMinX + (x + 0.5f) * cs;
                const float py = g_voxMinY + (y + 0.5f) * cs;
                const float pz = g_voxMinZ + (z + 0.5f) * cs;
                const float d = shape == 0 ? std::sqrt(px * px + py * py + pz * pz) - radius
                                           : std::sqrt(py * py + pz * pz) - radius;
                const size_t i = (size_t)(z * res + y) * res + x;
                g_voxelData[i] = (d <= 0.0f) ? 1 : 0;
                g_distanceField[i] = d / cs;
            }
    minBB = glm::vec3(-radius); maxBB = glm::vec3(radius);
    center = glm::vec3(0.0f); maxDim = 2.0f * radius;
    thermalParams.enabled = false;
    shutdownLBM();
    initLBM();
    if (!lbmInitialized) return -1;
    dims[0] = lbmNx; dims[1] = lbmNy; dims[2] = lbmNz;
    *tau_out = lbmParams.tau;
    float ux, uy, uz;
    computeInletVelocityLB(ux, uy, uz);
    uin_out[0] = ux; uin_out[1] = uy; uin_out[2] = uz;
    return 0;
}

// The reference's whole voxel grid build (voxel_grid.cpp:224-553) of a mesh
// whose bounds are set as the model loader sets them: grid plan from the
// mesh box with a margin of 14 % of its diagonal, BVH mask, distance field. Returns
// the cell count (0 when the build refused); ref_voxel_get reads the result:
// dims3, the grid minimum, the cell sizes, the mask and the distance field.
long long ref_build_voxel_grid(const float* verts, long long nfloats, int res) {
    std::vector<float> v(verts, verts + nfloats);
    glm::vec3 lo(1e30f), hi(-1e30f);
    for (long long i = 0; i + 2 < nfloats; i += 3) {
        lo = glm::min(lo, glm::vec3(v[i], v[i + 1], v[i + 2]));
        hi = glm::max(hi, glm::vec3(v[i], v[i + 1], v[i + 2]));
    }
    // bounds as the model loader sets them (model.cpp:47-66)
    minBB = lo; maxBB = hi; center = (lo + hi) * 0.5f;
    maxDim = glm::length(hi - lo);
    if (maxDim < 0.0001f || !std::isfinite(maxDim)) maxDim = 1.0f;
    g_voxelData.clear();
    g_distanceField.clear();
    buildVoxelGrid(v, res);
    if (!g_voxelBuildError.empty()) return 0;
    return (long long)g_voxelData.size();
}

void ref_voxel_get(int* dims3, float* min3, float* cs3, uint8_t* mask, float* sdf) {
    dims3[0] = g_voxNx; dims3[1] = g_voxNy; dims3[2] = g_voxNz;
    min3[0] = g_voxMinX; min3[1] = g_voxMinY; min3[2] = g_voxMinZ;
    cs3[0] = (g_voxMaxX - g_voxMinX) / g_voxNx;
    cs3[1] = (g_voxMaxY - g_voxMinY) / g_voxNy;
    cs3[2] = (g_voxMaxZ - g_voxMinZ) / g_voxNz;
    const size_t n = g_voxelData.size();
    for (size_t i = 0; i < n; ++i) {
        if (mask) mask[i] = (uint8_t)g_voxelData[i];
        if (sdf) sdf[i] = g_distanceField[i];
    }
}

// sampleSDFCPU / sdfNormalCPU (voxel_grid.cpp:32-123) on the last grid, with
// the flow field's cell size set to the grid's.
void ref_sdf_sample(const float* pts, long long n, float* dist, float* normal) {
    flowParams.cellSizeX = (g_voxMaxX - g_voxMinX) / g_voxNx;
    flowParams.cellSizeY = (g_voxMaxY - g_voxMinY) / g_voxNy;
    flowParams.cellSizeZ = (g_voxMaxZ - g_voxMinZ) / g_voxNz;
    for (long long i = 0; i < n; ++i) {
        const glm::vec3 p(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        dist[i] = sampleSDFCPU(p);
        const glm::vec3 nn = sdfNormalCPU(p);
        normal[3 * i] = nn.x; normal[3 * i + 1] = nn.y; normal[3 * i + 2] = nn.z;
    }
}

// stlformat::detect (stl_format.h:86-140): out4 = format (0 unknown, 1
// binary, 2 ascii), declared triangles, payload bytes, trailing bytes.
void ref_stl_detect(const unsigned char* data, unsigned long long size, unsigned long long* out4) {
    const stlformat::Detection d = stlformat::detect(data, (std::size_t)size);
    out4[0] = d.format == stlformat::Format::Binary ? 1 : (d.format == stlformat::Format::Ascii ? 2 : 0);
    out4[1] = d.declaredTriangles;
    out4[2] = d.payloadBytes;
    out4[3] = d.trailingBytes;
}

// loadSTL (stl_loader.cpp:30-223): returns the triangle count (-1 when it
// returned false); ref_stl_get copies the arrays of the last load.
static std::vector<float> s_stl_v, s_stl_n;
long long ref_stl_load(const char* path) {
    s_stl_v.clear();
    s_stl_n.clear();
    if (!loadSTL(path, s_stl_v, s_stl_n)) return -1;
    return (long long)(s_stl_v.size() / 9);
}
void ref_stl_get(float* v, float* n) {
    std::memcpy(v, s_stl_v.data(), s_stl_v.size() * sizeof(float));
    std::memcpy(n, s_stl_n.data(), s_stl_n.size() * sizeof(float));
}

// Solver mask: 0 fluid, 1 solid, 2 ground.
void ref_get_mask(uint8_t* out) {
    const size_t n = lbmIsSolid.size();
    for (size_t i = 0; i < n; ++i) out[i] = lbmIsSolid[i] ? 1 : (lbmIsGround[i] ? 2 : 0);
}

// The readback prep of the last stepLBMCPU call (lbm.cpp:1602-1705): world
// velocity, pressure, stats4 = {pressure min, max, residual rho, residual u},
// and the world parameters it used: wp8 = {flowSpeed, airDensity, lbmMin xyz,
// lbmCellSize xyz}.
void ref_world_get(float* uxw, float* uyw, float* uzw, float* p, float* stats4, long long* pbad, float* wp8) {
    const size_t n = lbmUxWorld.size();
    for (size_t i = 0; i < n; ++i) {
        uxw[i] = lbmUxWorld[i]; uyw[i] = lbmUyWorld[i]; uzw[i] = lbmUzWorld[i]; p[i] = lbmPressure[i];
    }
    stats4[0] = lbmPressureMin; stats4[1] = lbmPressureMax; stats4[2] = lbmResidualRho; stats4[3] = lbmResidualU;
    *pbad = lbmPressureNonFinite;
    wp8[0] = flowSpeed; wp8[1] = airDensity;
    wp8[2] = lbmMinX; wp8[3] = lbmMinY; wp8[4] = lbmMinZ;
    wp8[5] = lbmCellSizeX; wp8[6] = lbmCellSizeY; wp8[7] = lbmCellSizeZ;
}

// computeLBMVorticityAndQ (lbm.cpp:2005-2093) and its three fields.
void ref_vorticity_q(float* vort, float* q, float* strain) {
    computeLBMVorticityAndQ();
    const size_t n = lbmVorticityMag.size();
    for (size_t i = 0; i < n; ++i) { vort[i] = lbmVorticityMag[i]; q[i] = lbmQCriterion[i]; strain[i] = lbmStrainMag[i]; }
}

// The reference's samplers at n world points: field 0 getLBMVelocityLB (3
// values), 1..6 sampleFieldTrilinear of rho / pressure / vorticity / Q /
// strain / TKE with solid corners skipped, 7 isLBMSolidWorld.
void ref_sample(int field, const float* pts, long long n, float* out, uint8_t* valid) {
    const std::vector<float>* fields[7] = {nullptr, &lbmRho, &lbmPressure, &lbmVorticityMag, &lbmQCriterion,
                                           &lbmStrainMag, &lbmTKEField};
    for (long long i = 0; i < n; ++i) {
        const glm::vec3 w(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        if (field == 0) {
            const glm::vec3 v = getLBMVelocityLB(w);
            out[3 * i] = v.x; out[3 * i + 1] = v.y; out[3 * i + 2] = v.z;
            valid[i] = 0;
        } else if (field == 7) {
            out[i] = isLBMSolidWorld(w) ? 1.0f : 0.0f;
            valid[i] = 0;
        } else {
            float v = 0.0f;
            valid[i] = sampleFieldTrilinear(*fields[field], w, true, &v) ? 1 : 0;
            out[i] = v;
        }
    }
}

// computeLBMRefArea (lbm.cpp:2111-2160) of a triangle soup and settings.
float ref_ref_area(const float* v, long long ntri, float az, float el, int auto_area, float area_in, const float* bbmin,
                   const float* bbmax, float max_dim) {
    g_vertices.assign(v, v + 9 * ntri);
    flowAzimuth = az;
    flowElevation = el;
    aeroAutoRefArea = auto_area != 0;
    aeroRefArea = area_in;
    minBB = glm::vec3(bbmin[0], bbmin[1], bbmin[2]);
    maxBB = glm::vec3(bbmax[0], bbmax[1], bbmax[2]);
    maxDim = max_dim;
    return computeLBMRefArea();
}

// computeLBMRe (lbm.cpp:2094-2108) with the globals it reads.
float ref_lbm_re(float T, float rho, float speed, float max_dim, float re_prev) {
    airTemperature = T;
    airDensity = rho;
    flowSpeed = speed;
    maxDim = max_dim;
    aeroReNumber = re_prev;
    return computeLBMRe();
}

// Overwrites one cell of the last step's world pressure (lbmPressure).
void ref_poke_pressure(long long cell, float value) { lbmPressure[(size_t)cell] = value; }

// The atmosphere global the readback's pressure scale uses; computeLiftDrag's
// updateFlowParams rewrites it from the altitude (atmosphere.cpp:175-190).
void ref_set_air_density(float rho) { airDensity = rho; }

// computeLiftDrag (forces.cpp:401-688) on the LBM state of the last step,
// with the world pressure of that step. One OpenMP thread, so that the
// per-triangle sums run in triangle order. sdf: a field on the solver's voxel
// grid (NULL: no field). Globals the call leaves unchanged keep the
// sentinel 7.
struct RefAeroIn {
    float flow_speed, azimuth, elevation, altitude;
    int use_real_density, auto_ref_area;
    float ref_area;
    int mach_effects, ground_effect;
    float ground_height, re_number;
    float bb_min[3], bb_max[3], center[3], max_dim;
};
struct RefAeroOut {
    float drag, lift, ld, moment_mag, drag_vec[3], lift_vec[3], moment[3], cop[3], ref_area;
    long long cp_bad;
    float vel[3], air_temperature, air_density, speed_of_sound, vox_min_y, re_number;
};
void ref_lift_drag(const float* v, const float* n, long long ntri, const float* sdf, const RefAeroIn* in,
                   RefAeroOut* out) {
    g_vertices.assign(v, v + 9 * ntri);
    g_normals.assign(n, n + 9 * ntri);
    if (sdf) g_distanceField.assign(sdf, sdf + (size_t)g_voxNx * g_voxNy * g_voxNz);
    else g_distanceField.clear();
    flowSpeed = in->flow_speed; flowAzimuth = in->azimuth; flowElevation = in->elevation; altitude = in->altitude;
    useRealDensity = in->use_real_density != 0;
    aeroAutoRefArea = in->auto_ref_area != 0;
    aeroRefArea = in->ref_area;
    aeroMachEffects = in->mach_effects != 0;
    aeroGroundEffect = in->ground_effect != 0;
    aeroGroundHeight = in->ground_height;
    aeroReNumber = in->re_number;
    minBB = glm::vec3(in->bb_min[0], in->bb_min[1], in->bb_min[2]);
    maxBB = glm::vec3(in->bb_max[0], in->bb_max[1], in->bb_max[2]);
    center = glm::vec3(in->center[0], in->center[1], in->center[2]);
    maxDim = in->max_dim;
    const glm::vec3 s7(7.0f);
    dragMagnitude = liftMagnitude = liftToDragRatio = momentMagnitude = 7.0f;
    dragVector = liftVector = momentVector = centerOfPressure = s7;
    aeroCpNonFinite = 7;
    const int prev = omp_get_max_threads();
    omp_set_num_threads(1);
    computeLiftDrag();
    omp_set_num_threads(prev);
    out->drag = dragMagnitude; out->lift = liftMagnitude; out->ld = liftToDragRatio; out->moment_mag = momentMagnitude;
    for (int k = 0; k < 3; ++k) {
        out->drag_vec[k] = dragVector[k]; out->lift_vec[k] = liftVector[k];
        out->moment[k] = momentVector[k]; out->cop[k] = centerOfPressure[k];
    }
    out->ref_area = aeroRefArea;
    out->cp_bad = aeroCpNonFinite;
    out->vel[0] = flowParams.vx; out->vel[1] = flowParams.vy; out->vel[2] = flowParams.vz;
    out->air_temperature = flowParams.airTemperature;
    out->air_density = flowParams.airDensity;
    out->speed_of_sound = speedOfSound;
    out->vox_min_y = g_voxMinY;
    out->re_number = aeroReNumber;   // updateFlowParams recomputes it
}

}  // extern "C"
