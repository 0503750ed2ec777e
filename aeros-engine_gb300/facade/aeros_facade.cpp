// aeros_facade.cpp — globals and functions of aeros_facade.h over the C ABI.
// Errors are not exceptions: a failed call leaves lbmInitialized false (as
// the reference's initLBM refusals, aeros/src/lbm.cpp:543-563) or returns
// false / zero, and keeps the C ABI's message in lbmFacadeLastError().
#include "aeros_facade.h"

#include <algorithm>
#include <cmath>
#include <initializer_list>

std::vector<int> g_voxelData;
int g_voxNx = 0, g_voxNy = 0, g_voxNz = 0;
float lbmInletVelocityLB[3] = {0.0f, 0.0f, 0.0f};
float lbmVelocityScale = 1.0f;
int lbmStorage = AEROS_STORE_FP32;
bool lbmFacadeReadbackFields = true;

LBMParams lbmParams;
bool lbmInitialized = false;
bool lbmConverged = false;
int lbmCurrentStep = 0;
float lbmAvgRho = 1.0f;
float lbmAvgKineticEnergy = 0.0f;
float lbmMaxVelocityLB = 0.0f;
float lbmConvergence = 0.0f;
long long lbmNegativePops = 0;
long long lbmBadPops = 0;
long long lbmRhoOutOfRange = 0;
long long lbmRhoNonFinite = 0;
long long lbmULimited = 0;
float lbmTimeMs = 0.0f;
float lbmTKE = 0.0f;
int lbmNx = 0, lbmNy = 0, lbmNz = 0;
std::vector<float> lbmRho;
std::vector<float> lbmUx, lbmUy, lbmUz;
std::vector<float> lbmTKEField;
std::vector<float> lbmStrainMag;
std::vector<char> lbmIsSolid;
std::vector<char> lbmIsGround;

float lbmMinX = 0.0f, lbmMinY = 0.0f, lbmMinZ = 0.0f;
float lbmCellSizeX = 1.0f, lbmCellSizeY = 1.0f, lbmCellSizeZ = 1.0f;
float lbmMaxX = 0.0f, lbmMaxY = 0.0f, lbmMaxZ = 0.0f;
float lbmFacadeFlowSpeed = 1.0f;
float lbmFacadeAirDensity = 1.225f;
float lbmFacadeAirPressure = 101325.0f;
float lbmFacadeSpeedOfSound = 340.0f;
float lbmFacadeFreestream[3] = {0.0f, 0.0f, 0.0f};
std::vector<float> lbmUxWorld, lbmUyWorld, lbmUzWorld;
std::vector<float> lbmPressure;
std::vector<float> lbmVorticityMag;
std::vector<float> lbmQCriterion;
float lbmPressureMin = 0.0f, lbmPressureMax = 0.0f, lbmResidualRho = 0.0f, lbmResidualU = 0.0f;
long long lbmPressureNonFinite = 0;

float g_voxMinX = 0.0f, g_voxMinY = 0.0f, g_voxMinZ = 0.0f, g_voxMaxX = 0.0f, g_voxMaxY = 0.0f, g_voxMaxZ = 0.0f;
std::vector<float> g_distanceField;
std::string g_voxelBuildError;
long long g_voxelSolidCells = 0;
int g_voxelUsedRes = 0;

ThermalParams thermalParams;
std::vector<float> thermalT;
std::vector<float> thermalBuoyancyY;
bool thermalReady = false;
float thermalNusselt = 0.0f;
float thermalMeanT = 0.0f;

namespace {
aeros_lbm* g_handle = nullptr;
std::string g_error;
bool g_world_read = false;   // the device holds world fields of the current state
float g_uin[3] = {0.0f, 0.0f, 0.0f};   // the solver's inlet velocity (lattice units)

bool ok(int status) {
    if (status == AEROS_OK) return true;
    char buf[1024] = {0};
    aeros_consume_error(buf, sizeof(buf));
    g_error = buf;
    return false;
}

size_t cells() { return (size_t)lbmNx * (size_t)lbmNy * (size_t)lbmNz; }

void pull_stats() {
    aeros_lbm_stats s{};
    if (!ok(aeros_lbm_get_stats(g_handle, &s))) return;
    lbmCurrentStep = (int)s.step;
    lbmAvgRho = s.avg_rho;
    lbmAvgKineticEnergy = s.avg_kinetic;
    lbmTKE = s.avg_tke;
    lbmMaxVelocityLB = s.max_velocity_lb;
    lbmConvergence = s.convergence;
    lbmConverged = s.converged != 0;
    lbmNegativePops = s.negative_pops;
    lbmBadPops = s.bad_pops;
    lbmRhoOutOfRange = s.rho_out_of_range;
    lbmRhoNonFinite = s.rho_non_finite;
    lbmULimited = s.u_limited;
    if (thermalReady) {
        thermalNusselt = s.nusselt;
        thermalMeanT = s.mean_t;
    }
}

aeros_world_params world_params() {
    aeros_world_params w{};
    w.flow_speed = lbmFacadeFlowSpeed;
    w.air_density = lbmFacadeAirDensity;
    w.min[0] = lbmMinX; w.min[1] = lbmMinY; w.min[2] = lbmMinZ;
    w.cell[0] = lbmCellSizeX; w.cell[1] = lbmCellSizeY; w.cell[2] = lbmCellSizeZ;
    return w;
}

// The world-unit readback of the reference's stepLBMCPU end (lbm.cpp:1602-1705).
bool read_world() {
    const size_t n = cells();
    lbmUxWorld.resize(n);
    lbmUyWorld.resize(n);
    lbmUzWorld.resize(n);
    lbmPressure.resize(n);
    const aeros_world_params w = world_params();
    aeros_world_stats st{};
    if (!ok(aeros_lbm_world_fields(g_handle, &w, lbmUxWorld.data(), lbmUyWorld.data(), lbmUzWorld.data(),
                                   lbmPressure.data(), &st)))
        return false;
    lbmPressureMin = st.pressure_min;
    lbmPressureMax = st.pressure_max;
    lbmResidualRho = st.residual_rho;
    lbmResidualU = st.residual_u;
    lbmPressureNonFinite = st.pressure_non_finite;
    g_world_read = true;
    return true;
}
}  // namespace

namespace {
aeros_sdf_field* g_sdf = nullptr;   // the device copy of g_distanceField
aeros_voxel_grid g_sdf_grid{};      // its grid
}  // namespace

bool loadSTL(const std::string& filename, std::vector<float>& vertices, std::vector<float>& normals) {
    aeros_stl_info info{};
    if (!ok(aeros_stl_read_file(filename.c_str(), 0, nullptr, nullptr, 0, &info))) return false;
    const size_t base = vertices.size();
    vertices.resize(base + (size_t)info.triangles * 9);
    normals.resize(normals.size() + (size_t)info.triangles * 9);
    return ok(aeros_stl_read_file(filename.c_str(), 0, vertices.data() + base,
                                  normals.data() + normals.size() - (size_t)info.triangles * 9, info.triangles, &info));
}

void buildVoxelGrid(const std::vector<float>& verts, int res) {
    g_voxelBuildError.clear();
    g_voxelSolidCells = 0;
    g_voxelUsedRes = 0;
    if (verts.empty()) {
        g_voxelBuildError = "no vertices";
        return;
    }
    res = std::min(std::max(res, 8), 256);
    // bounds as the model loader computes them (model.cpp:47-66)
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    bool any = false;
    for (size_t i = 0; i + 2 < verts.size(); i += 3) {
        if (!std::isfinite(verts[i]) || !std::isfinite(verts[i + 1]) || !std::isfinite(verts[i + 2])) continue;
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], verts[i + a]);
            hi[a] = std::max(hi[a], verts[i + a]);
        }
        any = true;
    }
    if (!any) {
        g_voxelBuildError = "no finite vertex";
        return;
    }
    const float ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
    const float diag = std::sqrt(ex * ex + ey * ey + ez * ez);
    if (!(diag >= 1e-6f)) {   // voxel_grid.cpp:241-244
        g_voxelBuildError = "invalid bounding box";
        return;
    }
    const float maxDim = (diag < 0.0001f || !std::isfinite(diag)) ? 1.0f : diag;
    // grid box and plan (voxel_grid.cpp:246-288)
    float margin = 0.14f * maxDim;
    if (!std::isfinite(margin) || margin < 0.001f) margin = 0.1f;
    float mn[3], mx[3], size[3];
    for (int a = 0; a < 3; ++a) {
        mn[a] = lo[a] - margin;
        mx[a] = hi[a] + margin;
        size[a] = mx[a] - mn[a];
        if (size[a] < 1e-6f) size[a] = 1.0f;
    }
    aeros_voxel_plan_t plan{};
    if (!ok(aeros_voxel_plan(size, res, 0, &plan))) {
        g_voxelBuildError = g_error;
        return;
    }
    aeros_voxel_grid grid{};
    grid.nx = plan.nx;
    grid.ny = plan.ny;
    grid.nz = plan.nz;
    for (int a = 0; a < 3; ++a) {
        const int n = a == 0 ? plan.nx : (a == 1 ? plan.ny : plan.nz);
        grid.min[a] = mn[a];
        grid.cell[a] = size[a] / n;
        if (grid.cell[a] < 1e-6f) grid.cell[a] = 0.1f;
    }
    const long long total = (long long)grid.nx * grid.ny * grid.nz;
    if (total <= 0 || total > 20ll * 1024 * 1024) {
        g_voxelBuildError = "cell count " + std::to_string(total) + " outside 1 .. 20 M";
        return;
    }
    std::vector<uint8_t> mask((size_t)total);
    if (!ok(aeros_voxelize(verts.data(), (int64_t)(verts.size() / 9), &grid, mask.data()))) {
        g_voxelBuildError = g_error;
        return;
    }
    aeros_sdf_field* f = nullptr;
    if (!ok(aeros_sdf_field_create(mask.data(), &grid, &f))) {
        g_voxelBuildError = g_error;
        return;
    }
    g_distanceField.resize((size_t)total);
    if (!ok(aeros_sdf_field_read(f, g_distanceField.data()))) {
        aeros_sdf_field_destroy(f);
        g_voxelBuildError = g_error;
        return;
    }
    aeros_sdf_field_destroy(g_sdf);
    g_sdf = f;
    g_sdf_grid = grid;
    g_voxNx = grid.nx;
    g_voxNy = grid.ny;
    g_voxNz = grid.nz;
    g_voxMinX = mn[0]; g_voxMinY = mn[1]; g_voxMinZ = mn[2];
    g_voxMaxX = mx[0]; g_voxMaxY = mx[1]; g_voxMaxZ = mx[2];
    g_voxelData.assign(mask.begin(), mask.end());
    g_voxelSolidCells = 0;
    for (uint8_t v : mask) g_voxelSolidCells += v != 0;
    g_voxelUsedRes = grid.nx;
}

bool voxelFacadeSampleSDF(const float* points, long long n, float* dist, float* normal) {
    if (!g_sdf) {   // no field: the reference's 1000 and (0, 1, 0)
        for (long long i = 0; i < n; ++i) {
            if (dist) dist[i] = 1000.0f;
            if (normal) { normal[3 * i] = 0.0f; normal[3 * i + 1] = 1.0f; normal[3 * i + 2] = 0.0f; }
        }
        return true;
    }
    return ok(aeros_sdf_field_sample(g_sdf, points, n, dist, normal));
}

float sampleSDFCPU(const LbmVec3& p) {
    const float pt[3] = {p.x, p.y, p.z};
    float d = 1000.0f;
    if (!voxelFacadeSampleSDF(pt, 1, &d, nullptr)) return 1000.0f;
    return d;
}

LbmVec3 sdfNormalCPU(const LbmVec3& p) {
    const float pt[3] = {p.x, p.y, p.z};
    float n[3] = {0.0f, 1.0f, 0.0f};
    LbmVec3 r;
    if (!voxelFacadeSampleSDF(pt, 1, nullptr, n)) n[0] = 0.0f, n[1] = 1.0f, n[2] = 0.0f;
    r.x = n[0]; r.y = n[1]; r.z = n[2];
    return r;
}

aeros_lbm* lbmFacadeHandle() { return g_handle; }
const std::string& lbmFacadeLastError() { return g_error; }

bool lbmFacadeReadFields() {
    if (!g_handle) return false;
    const size_t n = cells();
    lbmRho.resize(n);
    lbmUx.resize(n);
    lbmUy.resize(n);
    lbmUz.resize(n);
    lbmStrainMag.resize(n);
    lbmTKEField.resize(n);
    if (!ok(aeros_lbm_read_fields(g_handle, lbmRho.data(), lbmUx.data(), lbmUy.data(), lbmUz.data(),
                                  lbmStrainMag.data(), lbmTKEField.data())))
        return false;
    if (thermalReady) {
        thermalT.resize(n);
        thermalBuoyancyY.resize(n);
        return ok(aeros_lbm_thermal_read(g_handle, thermalT.data(), thermalBuoyancyY.data()));
    }
    return true;
}

void shutdownLBM() {
    if (g_handle) aeros_lbm_destroy(g_handle);
    g_handle = nullptr;
    lbmInitialized = false;
    thermalReady = false;
}

void initLBM() {
    shutdownLBM();
    g_error.clear();
    const long long n = (long long)g_voxNx * g_voxNy * g_voxNz;
    if (g_voxNx < 4 || g_voxNy < 4 || g_voxNz < 4 || (long long)g_voxelData.size() != n) {
        g_error = "initLBM: g_voxelData does not hold g_voxNx*g_voxNy*g_voxNz cells";
        return;
    }
    lbmNx = g_voxNx;
    lbmNy = g_voxNy;
    lbmNz = g_voxNz;
    std::vector<uint8_t> mask((size_t)n);
    lbmIsSolid.assign((size_t)n, 0);
    lbmIsGround.assign((size_t)n, 0);
    for (long long c = 0; c < n; ++c) {
        const int v = g_voxelData[(size_t)c];
        mask[(size_t)c] = v == 0 ? AEROS_CELL_FLUID : (v == 2 ? AEROS_CELL_GROUND : AEROS_CELL_SOLID);
        lbmIsSolid[(size_t)c] = v != 0;
        lbmIsGround[(size_t)c] = v == 2;
    }
    aeros_lbm_params p{};
    p.nx = lbmNx;
    p.ny = lbmNy;
    p.nz = lbmNz;
    p.tau = lbmParams.tau;
    p.smagorinsky_c = lbmParams.smagorinskyC;
    p.use_les = lbmParams.useTurbulence;
    p.use_trt = lbmParams.useTRT;
    p.periodic_x = lbmParams.periodicX;
    p.periodic_z = lbmParams.periodicZ;
    p.convective_outlet = lbmParams.useConvectiveOutlet;
    p.flow_axis = 0;
    p.flow_sign = 1;
    const bool given = lbmInletVelocityLB[0] != 0.0f || lbmInletVelocityLB[1] != 0.0f || lbmInletVelocityLB[2] != 0.0f;
    for (int i = 0; i < 3; ++i) {
        p.u_in[i] = given ? lbmInletVelocityLB[i] : (i == 0 ? lbmParams.U0 : 0.0f);
        p.u_init[i] = p.u_in[i];
        g_uin[i] = p.u_in[i];
    }
    p.body_force[0] = lbmParams.bodyForceX;
    p.body_force[1] = lbmParams.bodyForceY;
    p.body_force[2] = lbmParams.bodyForceZ;
    p.vel_scale = lbmVelocityScale;
    p.convergence_threshold = lbmParams.convergenceThreshold;
    p.storage = lbmStorage;
    p.lateral_bc = AEROS_LATERAL_COPY;
    p.outlet_bc = AEROS_OUTLET_REFERENCE;
    if (!ok(aeros_lbm_create(&p, mask.data(), &g_handle))) {
        g_handle = nullptr;
        return;
    }
    lbmInitialized = true;
    lbmCurrentStep = 0;
    g_world_read = false;
    lbmMaxX = lbmMinX + lbmNx * lbmCellSizeX;
    lbmMaxY = lbmMinY + lbmNy * lbmCellSizeY;
    lbmMaxZ = lbmMinZ + lbmNz * lbmCellSizeZ;
    // the derived fields start at zero, as the reference allocates them (lbm.cpp:566-580)
    for (std::vector<float>* v : {&lbmUxWorld, &lbmUyWorld, &lbmUzWorld, &lbmPressure, &lbmVorticityMag, &lbmQCriterion})
        v->assign((size_t)n, 0.0f);
    pull_stats();
    if (lbmFacadeReadbackFields) lbmFacadeReadFields();
}

void resetLBM() { initLBM(); }

void stepLBMCPU(int steps) {
    if (!g_handle || steps <= 0) return;
    if (!ok(aeros_lbm_step(g_handle, steps))) return;
    g_world_read = false;
    float ms = 0.0f;
    if (ok(aeros_lbm_last_step_ms(g_handle, &ms))) lbmTimeMs = ms;
    pull_stats();
    if (lbmFacadeReadbackFields && lbmFacadeReadFields()) read_world();
}

void computeLBMVorticityAndQ() {
    if (!g_handle) return;
    const size_t n = cells();
    lbmVorticityMag.resize(n);
    lbmQCriterion.resize(n);
    lbmStrainMag.resize(n);
    if (!g_world_read && !read_world()) return;
    ok(aeros_lbm_vorticity_q(g_handle, lbmVorticityMag.data(), lbmQCriterion.data(), lbmStrainMag.data()));
}

std::vector<float> g_vertices, g_normals;
float lbmFacadeAirTemperature = 288.15f;
bool useRealDensity = true;
float flowAzimuth = 0.0f, flowElevation = 0.0f;
LbmVec3 minBB, maxBB, center;
float maxDim = 1.0f;
float aeroRefArea = 1.0f;
bool aeroAutoRefArea = true, aeroMachEffects = false, aeroGroundEffect = false;
float aeroGroundHeight = 0.0f, aeroReNumber = 0.0f;
float liftMagnitude = 0.0f, dragMagnitude = 0.0f, liftToDragRatio = 0.0f, momentMagnitude = 0.0f;
LbmVec3 liftVector, dragVector, momentVector, centerOfPressure;
long long aeroCpNonFinite = 0;

float computeLBMRefArea() {
    if (!aeroAutoRefArea) return (!std::isfinite(aeroRefArea) || aeroRefArea < 1e-6f) ? 1.0f : aeroRefArea;
    const float az = flowAzimuth * 0.01745329251994329576923690768489f;
    const float el = flowElevation * 0.01745329251994329576923690768489f;
    const float ce = cosf(el), se = sinf(el), ca = cosf(az), sa = sinf(az);
    float fd[3] = {ce * ca, se, ce * sa};
    const float fl = sqrtf((fd[0] * fd[0] + fd[1] * fd[1]) + fd[2] * fd[2]);
    if (fl > 1e-6f) {
        fd[0] /= fl; fd[1] /= fl; fd[2] /= fl;
    } else {
        fd[0] = 1.0f; fd[1] = 0.0f; fd[2] = 0.0f;
    }
    if (g_vertices.size() >= 9) {
        float proj = 0.0f;
        const size_t ntri = g_vertices.size() / 9;
        for (size_t t = 0; t < ntri; ++t) {
            const float* v = g_vertices.data() + 9 * t;
            const float e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
            const float e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
            const float c[3] = {e1[1] * e2[2] - e2[1] * e1[2], e1[2] * e2[0] - e2[2] * e1[0],
                                e1[0] * e2[1] - e2[0] * e1[1]};
            const float d = (c[0] * c[0] + c[1] * c[1]) + c[2] * c[2];
            const float area = 0.5f * sqrtf(d);
            if (!std::isfinite(area) || area < 1e-12f) continue;
            const float inv = 1.0f / sqrtf(d);   // glm::normalize: v * inversesqrt(dot(v, v))
            const float n[3] = {c[0] * inv, c[1] * inv, c[2] * inv};
            proj += area * fabsf((n[0] * fd[0] + n[1] * fd[1]) + n[2] * fd[2]);
        }
        const float frontal = proj * 0.5f;
        if (std::isfinite(frontal) && frontal > 1e-6f && frontal < 1e6f) return frontal;
    }
    float sy = maxBB.y - minBB.y, sz = maxBB.z - minBB.z, sx = maxBB.x - minBB.x;
    if (!std::isfinite(sy) || sy < 0.01f) sy = maxDim;
    if (!std::isfinite(sz) || sz < 0.01f) sz = maxDim;
    if (!std::isfinite(sx) || sx < 0.01f) sx = maxDim;
    float area = (fabsf(fd[0]) * sy * sz + fabsf(fd[1]) * sx * sz + fabsf(fd[2]) * sx * sy);
    if (!std::isfinite(area) || area < 1e-6f) area = maxDim * maxDim * 0.5f;
    return area;
}

float computeLBMRe() {
    float T = lbmFacadeAirTemperature;   // airSutherlandViscosity, flow_field.h:46-54
    if (!std::isfinite(T) || T < 50.0f) T = 288.15f;
    if (T > 2000.0f) T = 2000.0f;
    const float T0 = 273.15f, S = 110.4f, mu0 = 1.716e-5f;
    float mu = mu0 * powf(T / T0, 1.5f) * (T0 + S) / (T + S);
    if (!std::isfinite(mu) || mu < 1e-7f) mu = 1.81e-5f;
    float L = maxDim;
    if (L < 1e-6f) L = 1.0f;
    float re = lbmFacadeAirDensity * lbmFacadeFlowSpeed * L / mu;
    if (!std::isfinite(re)) re = aeroReNumber;
    if (re > 1e9f) re = 1e9f;
    return re;
}

float lbmReynolds = 0.0f;

void computeLBMForcesFromLBM() {
    lbmReynolds = computeLBMRe();
    aeroReNumber = lbmReynolds;
}

void computeLiftDrag() {
    if (!g_handle || g_vertices.size() < 9 || g_normals.size() != g_vertices.size()) return;   // forces.cpp:403-406
    if (!g_world_read && !read_world()) return;
    aeros_surface_params sp{};
    for (int a = 0; a < 3; ++a) sp.velocity[a] = lbmFacadeFreestream[a];
    sp.air_temperature = lbmFacadeAirTemperature;
    sp.air_density = lbmFacadeAirDensity;
    sp.use_real_density = useRealDensity;
    sp.speed_of_sound = lbmFacadeSpeedOfSound;
    sp.mach_effects = aeroMachEffects;
    sp.auto_ref_area = aeroAutoRefArea;
    sp.ref_area = aeroRefArea;
    sp.flow_azimuth_deg = flowAzimuth;
    sp.flow_elevation_deg = flowElevation;
    const LbmVec3* bv[3] = {&minBB, &maxBB, &center};
    float* dv[3] = {sp.bb_min, sp.bb_max, sp.center};
    for (int i = 0; i < 3; ++i) {
        dv[i][0] = bv[i]->x;
        dv[i][1] = bv[i]->y;
        dv[i][2] = bv[i]->z;
    }
    sp.max_dim = maxDim;
    sp.reynolds = aeroReNumber;
    sp.ground_effect = aeroGroundEffect;
    sp.ground_height = aeroGroundHeight;
    sp.vox_min_y = g_voxMinY;
    aeros_surface_mesh* mesh = nullptr;
    if (!ok(aeros_surface_mesh_create(g_vertices.data(), g_normals.data(), (int64_t)(g_vertices.size() / 9), &mesh)))
        return;
    const aeros_world_params w = world_params();
    aeros_surface_forces out{};
    const bool done = ok(aeros_lbm_surface_forces(g_handle, &w, &sp, mesh, g_sdf ? aeros_sdf_field_device(g_sdf) : nullptr,
                                                  g_sdf ? &g_sdf_grid : nullptr, &out, nullptr));
    aeros_surface_mesh_destroy(mesh);
    if (!done || out.status == AEROS_SURFACE_NOT_RUN) return;
    liftMagnitude = out.lift;
    dragMagnitude = out.drag;
    liftToDragRatio = out.lift_to_drag;
    if (out.status == AEROS_SURFACE_NO_FLOW) return;   // forces.cpp:412: only these three
    momentMagnitude = out.moment_magnitude;
    LbmVec3* vs[4] = {&dragVector, &liftVector, &momentVector, &centerOfPressure};
    const float* src[4] = {out.drag_vector, out.lift_vector, out.moment, out.center_of_pressure};
    for (int i = 0; i < 4; ++i) {
        vs[i]->x = src[i][0];
        vs[i]->y = src[i][1];
        vs[i]->z = src[i][2];
    }
    aeroRefArea = out.ref_area;
    aeroCpNonFinite = out.cp_non_finite;
}

bool lbmFacadeSample(int field, const float* points, long long n, float* out, uint8_t* valid) {
    if (!g_handle) return false;
    const aeros_world_params w = world_params();
    return ok(aeros_lbm_sample(g_handle, &w, field, points, n, out, valid));
}

namespace {
bool sample_one(int field, const LbmVec3& p, float* out) {
    const float pt[3] = {p.x, p.y, p.z};
    uint8_t valid = 0;
    if (!lbmFacadeSample(field, pt, 1, out, &valid)) return false;
    return valid != 0;
}
float sample_or(int field, const LbmVec3& p, float fallback) {
    float v = 0.0f;
    return sample_one(field, p, &v) ? v : fallback;
}
}  // namespace

LbmVec3 getLBMVelocityLB(const LbmVec3& worldPos) {   // the value is the answer: no validity flag
    const float pt[3] = {worldPos.x, worldPos.y, worldPos.z};
    float v[3] = {0.0f, 0.0f, 0.0f};
    uint8_t valid = 0;
    LbmVec3 r;
    if (!lbmFacadeSample(AEROS_FIELD_VELOCITY_LB, pt, 1, v, &valid)) v[0] = v[1] = v[2] = 0.0f;
    r.x = v[0]; r.y = v[1]; r.z = v[2];
    return r;
}
float getLBMDensityWorld(const LbmVec3& worldPos) {   // lbm.cpp:1948-1952
    float rho = 1.0f;
    if (sample_one(AEROS_FIELD_DENSITY, worldPos, &rho)) return std::min(std::max(rho, 0.8f), 1.2f);
    return 1.0f;
}
bool getLBMPressureWorldChecked(const LbmVec3& worldPos, float* outPa) {
    if (!outPa) return false;
    *outPa = 0.0f;
    return sample_one(AEROS_FIELD_PRESSURE, worldPos, outPa);
}
float getLBMPressureWorld(const LbmVec3& worldPos) { return sample_or(AEROS_FIELD_PRESSURE, worldPos, 0.0f); }
float getLBMVorticityWorld(const LbmVec3& worldPos) { return sample_or(AEROS_FIELD_VORTICITY, worldPos, 0.0f); }
float getLBMQWorld(const LbmVec3& worldPos) { return sample_or(AEROS_FIELD_Q, worldPos, 0.0f); }
float getLBMTKEWorld(const LbmVec3& worldPos) { return sample_or(AEROS_FIELD_TKE, worldPos, 0.0f); }
float getLBMStrainWorld(const LbmVec3& worldPos) { return sample_or(AEROS_FIELD_STRAIN, worldPos, 0.0f); }
bool isLBMSolidWorld(const LbmVec3& worldPos) {   // the value is the answer: no validity flag
    const float pt[3] = {worldPos.x, worldPos.y, worldPos.z};
    float v = 0.0f;
    uint8_t valid = 0;
    return lbmFacadeSample(AEROS_FIELD_SOLID, pt, 1, &v, &valid) && v != 0.0f;
}

namespace {
LbmVec3 vec3(float x, float y, float z) {
    LbmVec3 v;
    v.x = x; v.y = y; v.z = z;
    return v;
}
float length3(const LbmVec3& v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
// flowSpeed / |u_in| with the reference's fallbacks (lbm.cpp:1857-1862)
float velocity_scale() {
    float u0 = std::sqrt(g_uin[0] * g_uin[0] + g_uin[1] * g_uin[1] + g_uin[2] * g_uin[2]);
    if (!std::isfinite(u0) || u0 < 1e-6f) u0 = 0.08f;
    float scale = lbmFacadeFlowSpeed / u0;
    if (!std::isfinite(scale) || scale > 1000.0f) scale = 20.0f;
    return scale;
}
}  // namespace

LbmVec3 getLBMVelocityWorld(const LbmVec3& p) {   // lbm.cpp:1847-1870
    const LbmVec3 fs = vec3(lbmFacadeFreestream[0], lbmFacadeFreestream[1], lbmFacadeFreestream[2]);
    if (!lbmInitialized || !g_handle) return fs;
    if (p.x < lbmMinX || p.x > lbmMaxX || p.y < lbmMinY || p.y > lbmMaxY || p.z < lbmMinZ || p.z > lbmMaxZ) return fs;
    if (isLBMSolidWorld(p)) return vec3(0.0f, 0.0f, 0.0f);
    const LbmVec3 v = getLBMVelocityLB(p);
    const float mag2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (mag2 < 1e-12f) return vec3(0.0f, 0.0f, 0.0f);
    const float scale = velocity_scale();
    LbmVec3 w = vec3(v.x * scale, v.y * scale, v.z * scale);
    if (!std::isfinite(w.x)) return fs;
    const float maxV = lbmFacadeFlowSpeed * 2.0f;
    const float mag = length3(w);
    if (mag > maxV) {
        const float k = maxV / mag;
        w = vec3(w.x * k, w.y * k, w.z * k);
    }
    return w;
}

float getLBMVelocityMagWorld(const LbmVec3& p) {   // lbm.cpp:1992-1996
    const float m = length3(getLBMVelocityWorld(p));
    return std::isfinite(m) ? m : 0.0f;
}

float getLBMMachWorld(const LbmVec3& p) {   // lbm.cpp:2319-2326
    const float mag = length3(getLBMVelocityWorld(p));
    if (!std::isfinite(mag)) return 0.0f;
    float a = lbmFacadeSpeedOfSound;
    if (a < 1.0f) a = 340.0f;
    return mag / a;
}

// lbm.cpp:2328-2356: normalized helicity from the world velocity at the point
// and the central-difference vorticity of the cell (the world fields of the
// last readback, held on the host by this layer).
float getLBMHelicityWorld(const LbmVec3& p) {
    if (!lbmInitialized) return 0.0f;
    const float fx = (p.x - lbmMinX) / lbmCellSizeX;
    const float fy = (p.y - lbmMinY) / lbmCellSizeY;
    const float fz = (p.z - lbmMinZ) / lbmCellSizeZ;
    const int ix = (int)std::floor(fx), iy = (int)std::floor(fy), iz = (int)std::floor(fz);
    if (ix <= 0 || ix >= lbmNx - 1 || iy <= 0 || iy >= lbmNy - 1 || iz <= 0 || iz >= lbmNz - 1) return 0.0f;
    const long long cell = ((long long)iz * lbmNy + iy) * lbmNx + ix;
    const long long total = (long long)lbmNx * lbmNy * lbmNz;
    if ((long long)lbmVorticityMag.size() != total || (long long)lbmUxWorld.size() != total) return 0.0f;
    const LbmVec3 vel = getLBMVelocityWorld(p);
    const long long xm = cell - 1, xp = cell + 1;
    const long long ym = cell - lbmNx, yp = cell + lbmNx;
    const long long zm = cell - (long long)lbmNx * lbmNy, zp = cell + (long long)lbmNx * lbmNy;
    const float duz_dy = (lbmUzWorld[yp] - lbmUzWorld[ym]) * 0.5f;
    const float duy_dz = (lbmUyWorld[zp] - lbmUyWorld[zm]) * 0.5f;
    const float dux_dz = (lbmUxWorld[zp] - lbmUxWorld[zm]) * 0.5f;
    const float duz_dx = (lbmUzWorld[xp] - lbmUzWorld[xm]) * 0.5f;
    const float duy_dx = (lbmUyWorld[xp] - lbmUyWorld[xm]) * 0.5f;
    const float dux_dy = (lbmUxWorld[yp] - lbmUxWorld[ym]) * 0.5f;
    const LbmVec3 om = vec3(duz_dy - duy_dz, dux_dz - duz_dx, duy_dx - dux_dy);
    const float h = vel.x * om.x + vel.y * om.y + vel.z * om.z;
    if (!std::isfinite(h)) return 0.0f;
    const float vm = length3(vel), om_m = length3(om);
    if (vm < 1e-6f || om_m < 1e-6f) return 0.0f;
    return h / (vm * om_m);
}

float getLBMTotalPressureWorld(const LbmVec3& p) {   // lbm.cpp:2358-2372
    const LbmVec3 v = getLBMVelocityWorld(p);
    const float mag2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (!std::isfinite(mag2)) return lbmFacadeAirPressure;
    float pStatic = lbmFacadeAirPressure;
    float lbmP = 0.0f;
    getLBMPressureWorldChecked(p, &lbmP);
    pStatic += lbmP;
    const float pt = pStatic + 0.5f * lbmFacadeAirDensity * mag2;
    return std::isfinite(pt) ? pt : lbmFacadeAirPressure;
}

float lbmLatticeDtWorld() {   // lbm.cpp:1717-1732
    if (!lbmInitialized) return 0.0f;
    const float dx = lbmCellSizeX;
    if (!std::isfinite(dx) || dx <= 0.0f) return 0.0f;
    float u0 = std::sqrt(g_uin[0] * g_uin[0] + g_uin[1] * g_uin[1] + g_uin[2] * g_uin[2]);
    if (!std::isfinite(u0) || u0 < 1e-6f) u0 = 0.08f;
    float vs = lbmFacadeFlowSpeed / u0;
    if (!std::isfinite(vs) || vs > 1000.0f) vs = 20.0f;
    if (vs < 0.01f) vs = 0.01f;
    float dt = dx / vs;
    if (!std::isfinite(dt) || dt <= 0.0f) return 0.0f;
    return dt > 1.0f ? 1.0f : dt;
}

void updateLBM(float deltaTime, int forceSteps) {   // lbm.cpp:1734-1780
    if (!lbmParams.enabled) return;
    // a new voxel grid re-initializes the solver (lbm.cpp:1740-1762)
    if (!lbmInitialized || g_voxNx != lbmNx || g_voxNy != lbmNy || g_voxNz != lbmNz) {
        initLBM();
        return;
    }
    int steps;
    if (forceSteps >= 0) {
        steps = std::min(forceSteps, 64);
    } else {
        steps = lbmParams.stepsPerFrame;
        if (steps <= 0) steps = 1;
        if (steps > 50) steps = 50;
        if (deltaTime > 0.02f) steps = std::min(steps * 2, 50);
    }
    if (steps <= 0) return;
    stepLBMCPU(steps);
    if (lbmCurrentStep % 30 == 0) computeLBMVorticityAndQ();
}

bool lbmEquilibriumMoments(float rho, float ux, float uy, float uz, float* sumFeq, float* momX, float* momY,
                           float* momZ) {
    if (!sumFeq || !momX || !momY || !momZ) return false;
    const float st[4] = {rho, ux, uy, uz};
    float out[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    uint8_t good = 0;
    if (!ok(aeros_equilibrium_moments(st, 1, out, &good)) || !good) return false;
    *sumFeq = out[0];
    *momX = out[1];
    *momY = out[2];
    *momZ = out[3];
    return true;
}

bool lbmValidateInitialization() {   // lbm.cpp:2263-2270
    if (!lbmInitialized || lbmNx <= 0 || lbmNy <= 0 || lbmNz <= 0) return false;
    if (lbmRho.size() != cells()) return false;
    for (float r : lbmRho)
        if (!std::isfinite(r) || r < 0.5f || r > 1.5f) return false;
    return true;
}

bool lbmValidateConservation() {   // lbm.cpp:2272-2279
    if (!lbmInitialized) return true;
    double sum = 0.0;
    long long n = 0;
    for (float r : lbmRho)
        if (std::isfinite(r)) {
            sum += r;
            ++n;
        }
    if (n == 0) return false;
    return std::fabs(sum / (double)n - 1.0f) <= 0.1f;
}

bool lbmValidateBoundaryConditions() {   // lbm.cpp:2281-2286
    if (!lbmInitialized) return true;
    const float mag = std::sqrt(g_uin[0] * g_uin[0] + g_uin[1] * g_uin[1] + g_uin[2] * g_uin[2]);
    return std::isfinite(mag) && mag >= 1e-6f && mag <= 0.2f;
}

bool lbmValidateSolidHandling() {   // lbm.cpp:2288-2295
    if (!lbmInitialized) return true;
    const size_t n = std::min(lbmIsSolid.size(), lbmUx.size());
    for (size_t i = 0; i < n; ++i)
        if (lbmIsSolid[i] && (std::fabs(lbmUx[i]) > 1e-4f || std::fabs(lbmUy[i]) > 1e-4f || std::fabs(lbmUz[i]) > 1e-4f))
            return false;
    return true;
}

bool lbmValidateRealisticAero() {   // lbm.cpp:2297-2309
    if (!lbmInitialized) return true;
    float maxP = -1e9f, minP = 1e9f;
    for (float p : lbmPressure) {
        if (!std::isfinite(p)) return false;
        maxP = std::max(maxP, p);
        minP = std::min(minP, p);
    }
    const float q = 0.5f * lbmFacadeAirDensity * lbmFacadeFlowSpeed * lbmFacadeFlowSpeed;
    if (std::fabs(maxP) > q * 1.5f || std::fabs(minP) > q * 1.5f) return false;
    for (float t : lbmTKEField)
        if (t < -1e-3f || !std::isfinite(t) || t > 10.0f) return false;
    for (float v : lbmVorticityMag)
        if (v < -1e-3f || !std::isfinite(v) || v > 1e4f) return false;
    return true;
}

bool lbmValidateStability() {   // lbm.cpp:2311-2317
    if (!lbmInitialized) return true;
    if (!std::isfinite(lbmAvgRho) || lbmAvgRho < 0.8f || lbmAvgRho > 1.2f) return false;
    if (!std::isfinite(lbmMaxVelocityLB) || lbmMaxVelocityLB > 0.35f) return false;
    if (!std::isfinite(lbmAvgKineticEnergy) || lbmAvgKineticEnergy > 0.1f) return false;
    return true;
}

LbmVec3 lbmControlVolumeForce(float boxHalfX, float boxHalfY, float boxHalfZ) {
    LbmVec3 r;
    double f[3] = {0.0, 0.0, 0.0};
    if (g_handle && ok(aeros_lbm_cv_force(g_handle, boxHalfX, boxHalfY, boxHalfZ, f))) {
        r.x = (float)f[0];
        r.y = (float)f[1];
        r.z = (float)f[2];
    }
    return r;
}

float lbmProjectedAreaCells(int axis) {
    double a = 0.0;
    if (!g_handle || !ok(aeros_lbm_projected_area(g_handle, axis, &a))) return 0.0f;
    return (float)a;
}

bool thermalInit(int nx, int ny, int nz, const std::vector<char>& solidMask, float nuLB) {
    thermalReady = false;
    if (!g_handle || nx != lbmNx || ny != lbmNy || nz != lbmNz || solidMask.size() != cells()) {
        g_error = "thermalInit: the GPU lattice has another grid (call initLBM first)";
        return false;
    }
    aeros_thermal_params tp{};
    tp.enabled = thermalParams.enabled ? 1 : 0;
    tp.rayleigh = thermalParams.rayleigh;
    tp.prandtl = thermalParams.prandtl;
    tp.fixed_wall_temps = thermalParams.fixedWallTemps ? 1 : 0;
    tp.hot_temp = thermalParams.hotTemp;
    tp.cold_temp = thermalParams.coldTemp;
    tp.perturbation = thermalParams.perturbation;
    tp.nu_lb = nuLB;
    if (!ok(aeros_lbm_thermal_init(g_handle, &tp))) return false;
    thermalReady = thermalParams.enabled;
    if (thermalReady && lbmFacadeReadbackFields) lbmFacadeReadFields();
    return true;
}

void thermalShutdown() { thermalReady = false; }

bool thermalUpload(const std::vector<float>& T) {
    if (!g_handle || T.size() != cells()) return false;
    if (!ok(aeros_lbm_thermal_upload(g_handle, T.data()))) return false;
    if (lbmFacadeReadbackFields) lbmFacadeReadFields();
    return true;
}

void thermalStep(const float*, const float*, const float*) {}
