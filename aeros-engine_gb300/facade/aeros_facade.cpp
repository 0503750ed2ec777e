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
float lbmFacadeFlowSpeed = 1.0f;
float lbmFacadeAirDensity = 1.225f;
std::vector<float> lbmUxWorld, lbmUyWorld, lbmUzWorld;
std::vector<float> lbmPressure;
std::vector<float> lbmVorticityMag;
std::vector<float> lbmQCriterion;
float lbmPressureMin = 0.0f, lbmPressureMax = 0.0f, lbmResidualRho = 0.0f, lbmResidualU = 0.0f;
long long lbmPressureNonFinite = 0;

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

LbmVec3 getLBMVelocityLB(const LbmVec3& worldPos) {
    float v[3] = {0.0f, 0.0f, 0.0f};
    LbmVec3 r;
    if (g_handle) sample_one(AEROS_FIELD_VELOCITY_LB, worldPos, v);
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
bool isLBMSolidWorld(const LbmVec3& worldPos) {
    float v = 0.0f;
    return sample_one(AEROS_FIELD_SOLID, worldPos, &v) && v != 0.0f;
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
