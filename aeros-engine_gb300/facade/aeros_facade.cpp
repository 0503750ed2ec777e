// aeros_facade.cpp — globals and functions of aeros_facade.h over the C ABI.
// Errors are not exceptions: a failed call leaves lbmInitialized false (as
// the reference's initLBM refusals, aeros/src/lbm.cpp:543-563) or returns
// false / zero, and keeps the C ABI's message in lbmFacadeLastError().
#include "aeros_facade.h"

#include <algorithm>
#include <cmath>

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

ThermalParams thermalParams;
std::vector<float> thermalT;
std::vector<float> thermalBuoyancyY;
bool thermalReady = false;
float thermalNusselt = 0.0f;
float thermalMeanT = 0.0f;

namespace {
aeros_lbm* g_handle = nullptr;
std::string g_error;

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
    pull_stats();
    if (lbmFacadeReadbackFields) lbmFacadeReadFields();
}

void resetLBM() { initLBM(); }

void stepLBMCPU(int steps) {
    if (!g_handle || steps <= 0) return;
    if (!ok(aeros_lbm_step(g_handle, steps))) return;
    float ms = 0.0f;
    if (ok(aeros_lbm_last_step_ms(g_handle, &ms))) lbmTimeMs = ms;
    pull_stats();
    if (lbmFacadeReadbackFields) lbmFacadeReadFields();
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
