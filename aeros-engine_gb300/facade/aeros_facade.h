// aeros_facade.h — the reference solver's C++ interface (aeros/src/lbm.h,
// aeros/src/thermal_lbm.h) over the GB300 C ABI (include/aeros_lbm.h).
//
// Drop-in for the solver's callers: the same function names and the same
// globals, which this layer fills from the device after each stepLBMCPU call
// (scalars always, fields when lbmFacadeReadbackFields is true). The grid
// comes from the voxel globals the reference's initLBM reads
// (g_voxelData / g_voxNx.. , aeros/src/globals.h:150-158), taken as the
// solver grid itself (the reference's domainPadding = 0 case). C++17, no
// dependency beyond the C ABI; glm::vec3 is used for the vector results when
// <glm/glm.hpp> is on the include path, a three-float struct otherwise.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/aeros_lbm.h"

#if __has_include(<glm/glm.hpp>)
#include <glm/glm.hpp>
using LbmVec3 = glm::vec3;
#else
struct LbmVec3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
};
#endif

// Solver settings: the fields of the reference's LBMParams (aeros/src/lbm.h:11-75)
// with its defaults, so settings code compiles unchanged. Fields the GPU step
// does not read (frame pacing, world-unit viscosity, domain padding) are kept
// for source compatibility.
struct LBMParams {
    bool enabled = false;
    bool useGPU = false;
    int stepsPerFrame = 3;
    float tau = 0.6f;
    float U0 = 0.1f;
    float viscosity = 0.033f;
    float smagorinskyC = 0.12f;
    bool useTurbulence = true;
    int maxSteps = 10000;
    float convergenceThreshold = 1e-5f;
    bool useGround = false;
    float groundHeight = 0.0f;
    bool useTRT = false;
    bool useConvectiveOutlet = true;
    float inletTurbulence = 0.02f;
    float domainPadding = 0.25f;
    bool autoViscosity = true;
    float bodyForceX = 0.0f;
    float bodyForceY = 0.0f;
    float bodyForceZ = 0.0f;
    bool periodicX = false;
    bool periodicZ = false;
};

// ---- inputs (aeros/src/globals.h:150-158) -----------------------------------
extern std::vector<int> g_voxelData;   // nx*ny*nz, nonzero = solid; 2 = ground
extern int g_voxNx, g_voxNy, g_voxNz;
// Inlet velocity in lattice units (the reference derives it from U0 and the
// flow angles, computeInletVelocityLB, aeros/src/lbm.cpp:186-199); default
// (U0, 0, 0) when all three are zero.
extern float lbmInletVelocityLB[3];
// Velocity scale world / lattice used for TKE in world units (lbm.cpp:1130).
extern float lbmVelocityScale;
// Population storage of the GPU step: AEROS_STORE_FP32 (drop-in, bitwise the
// reference's arithmetic) or AEROS_STORE_FP16 / AEROS_STORE_BF16.
extern int lbmStorage;
// Read the fields back after every stepLBMCPU call (the reference's globals
// always hold the latest fields); false leaves them to lbmFacadeReadFields().
extern bool lbmFacadeReadbackFields;

// ---- state (aeros/src/lbm.h:77-154) -----------------------------------------
extern LBMParams lbmParams;
extern bool lbmInitialized;
extern bool lbmConverged;
extern int lbmCurrentStep;
extern float lbmAvgRho;
extern float lbmAvgKineticEnergy;
extern float lbmMaxVelocityLB;
extern float lbmConvergence;
extern long long lbmNegativePops;
extern long long lbmBadPops;
extern long long lbmRhoOutOfRange;
extern long long lbmRhoNonFinite;
extern long long lbmULimited;
extern float lbmTimeMs;
extern float lbmTKE;
extern int lbmNx, lbmNy, lbmNz;
extern std::vector<float> lbmRho;
extern std::vector<float> lbmUx, lbmUy, lbmUz;
extern std::vector<float> lbmTKEField;
extern std::vector<float> lbmStrainMag;
extern std::vector<char> lbmIsSolid;
extern std::vector<char> lbmIsGround;

// World-unit readback (aeros/src/lbm.h:126-154): filled after every
// stepLBMCPU call when lbmFacadeReadbackFields is true, as the reference's
// stepLBMCPU does at its end (lbm.cpp:1602-1705). The grid's world placement
// and the freestream: the reference keeps flowSpeed and airDensity in other
// modules, so a caller copies them into the two inputs below.
extern float lbmMinX, lbmMinY, lbmMinZ;
extern float lbmCellSizeX, lbmCellSizeY, lbmCellSizeZ;
// lbmMin + lbmN * lbmCellSize, set by initLBM (lbm.cpp:505-507)
extern float lbmMaxX, lbmMaxY, lbmMaxZ;
extern float lbmFacadeFlowSpeed;       // flowSpeed, m/s
extern float lbmFacadeAirDensity;      // airDensity, kg/m^3
extern float lbmFacadeAirPressure;     // airPressure, Pa
extern float lbmFacadeSpeedOfSound;    // speedOfSound, m/s
extern float lbmFacadeFreestream[3];   // flowParams.vx, vy, vz, m/s
extern std::vector<float> lbmUxWorld, lbmUyWorld, lbmUzWorld;
extern std::vector<float> lbmPressure;
extern std::vector<float> lbmVorticityMag;
extern std::vector<float> lbmQCriterion;
extern float lbmPressureMin, lbmPressureMax, lbmResidualRho, lbmResidualU;
extern long long lbmPressureNonFinite;

// ---- solver (aeros/src/lbm.h:156-202) ---------------------------------------
void initLBM();
void resetLBM();
void shutdownLBM();
void stepLBMCPU(int steps = 1);
// updateLBM (lbm.cpp:1734-1780) for a fixed grid: forceSteps >= 0 steps that
// many (at most 64), -1 takes lbmParams.stepsPerFrame (doubled for long
// frames, at most 50); vorticity / Q every 30 steps. Initializes the solver
// when it is not.
void updateLBM(float deltaTime, int forceSteps = -1);
// lbmLatticeDtWorld (lbm.cpp:1717-1732): seconds of physical time per step.
float lbmLatticeDtWorld();
// lbmEquilibriumMoments (lbm.cpp:249-267), evaluated on the device.
bool lbmEquilibriumMoments(float rho, float ux, float uy, float uz, float* sumFeq, float* momX, float* momY,
                           float* momZ);
LbmVec3 lbmControlVolumeForce(float boxHalfX, float boxHalfY, float boxHalfZ);
float lbmProjectedAreaCells(int axis);
// computeLBMVorticityAndQ (lbm.cpp:2005-2093), on the device.
void computeLBMVorticityAndQ();
// The samplers (lbm.cpp:1782-1969), on the device, one point per call.
LbmVec3 getLBMVelocityLB(const LbmVec3& worldPos);
float getLBMDensityWorld(const LbmVec3& worldPos);
float getLBMPressureWorld(const LbmVec3& worldPos);
bool getLBMPressureWorldChecked(const LbmVec3& worldPos, float* outPa);
float getLBMVorticityWorld(const LbmVec3& worldPos);
float getLBMQWorld(const LbmVec3& worldPos);
float getLBMTKEWorld(const LbmVec3& worldPos);
float getLBMStrainWorld(const LbmVec3& worldPos);
bool isLBMSolidWorld(const LbmVec3& worldPos);
// Compositions of the samplers above, as the reference composes them
// (lbm.cpp:1847-1870, 1992-1996, 2319-2372).
LbmVec3 getLBMVelocityWorld(const LbmVec3& worldPos);
float getLBMVelocityMagWorld(const LbmVec3& worldPos);
float getLBMMachWorld(const LbmVec3& worldPos);
float getLBMHelicityWorld(const LbmVec3& worldPos);
float getLBMTotalPressureWorld(const LbmVec3& worldPos);
// Many points at once (xyz each): the way to sample a whole slice or a set
// of streamline seeds without a device round trip per point. field is one of
// AEROS_FIELD_*; out gets n values (3n for the velocity), valid n flags.
bool lbmFacadeSample(int field, const float* points, long long n, float* out, uint8_t* valid);

// The reference's self-checks (lbm.cpp:2263-2317) over the globals above
// (initialisation: density in [0.5, 1.5]; conservation: mean density within
// 10 %; inlet speed in (1e-6, 0.2]; solid cells at rest; pressure within
// 1.5 dynamic pressures, TKE and vorticity bounded; mean density, maximum
// velocity and kinetic energy in range).
bool lbmValidateInitialization();
bool lbmValidateConservation();
bool lbmValidateBoundaryConditions();
bool lbmValidateSolidHandling();
bool lbmValidateRealisticAero();
bool lbmValidateStability();

// ---- thermal (aeros/src/thermal_lbm.h:33-72) --------------------------------
struct ThermalParams {
    bool enabled = false;
    float rayleigh = 1.0e5f;
    float prandtl = 0.71f;
    bool fixedWallTemps = true;
    float hotTemp = 1.0f;
    float coldTemp = 0.0f;
    float perturbation = 0.02f;
};
extern ThermalParams thermalParams;
extern std::vector<float> thermalT;
extern std::vector<float> thermalBuoyancyY;
extern bool thermalReady;
extern float thermalNusselt;
extern float thermalMeanT;
// On the solver's grid (the GPU lattice must exist: call after initLBM). The
// mask argument is the solid mask the solver already holds; nuLB as the
// reference (lattice viscosity).
bool thermalInit(int nx, int ny, int nz, const std::vector<char>& solidMask, float nuLB);
void thermalShutdown();
bool thermalUpload(const std::vector<float>& T);
// The GPU step advances the thermal lattice inside stepLBMCPU (the reference
// calls thermalStep from there too, aeros/src/lbm.cpp:1551-1552); a separate
// call has nothing left to do.
void thermalStep(const float* ux, const float* uy, const float* uz);

// ---- geometry in (aeros/src/stl_loader.h, aeros/src/voxel_grid.h) ---------------
// loadSTL (stl_loader.cpp:30-223): binary or ASCII by content; 9 floats per
// triangle, per-vertex normals. false when the file cannot be used.
bool loadSTL(const std::string& filename, std::vector<float>& vertices, std::vector<float>& normals);
// buildVoxelGrid (voxel_grid.cpp:224-553) on the device: grid plan over the
// mesh bounds (computed from verts as the model loader does, model.cpp:47-66)
// plus 14 % of their diagonal, mask by the BVH three-ray vote, signed
// distance field. Fills the voxel globals below; g_voxelBuildError says why
// when it does not. The memory plan has no byte budget (the reference caps it
// at half of the free RAM).
void buildVoxelGrid(const std::vector<float>& verts, int res);
float sampleSDFCPU(const LbmVec3& p);    // on the device, one point per call
LbmVec3 sdfNormalCPU(const LbmVec3& p);
extern float g_voxMinX, g_voxMinY, g_voxMinZ, g_voxMaxX, g_voxMaxY, g_voxMaxZ;
extern std::vector<float> g_distanceField;
extern std::string g_voxelBuildError;
extern long long g_voxelSolidCells;
extern int g_voxelUsedRes;

// ---- lift and drag from the surface pressure (aeros/src/forces.h, globals.h) -------
// computeLiftDrag (forces.cpp:401-688), LBM branch: the per-triangle pass on the
// device over the pressure of the last step, the closing formulas on the host.
// Inputs: the model (g_vertices / g_normals, 9 floats per triangle each), the
// flow (lbmFacadeFreestream, lbmFacadeAirTemperature, lbmFacadeAirDensity,
// lbmFacadeSpeedOfSound), the aero options and model bounds below, and the
// distance field of the last buildVoxelGrid. Outputs: the globals below, as
// the reference sets them (unchanged when it returns early).
extern std::vector<float> g_vertices, g_normals;
extern float lbmFacadeAirTemperature;   // flowParams.airTemperature, K
extern bool useRealDensity;
extern float flowAzimuth, flowElevation;   // degrees (computeLBMRefArea's direction)
extern LbmVec3 minBB, maxBB, center;
extern float maxDim;
extern float aeroRefArea;
extern bool aeroAutoRefArea, aeroMachEffects, aeroGroundEffect;
extern float aeroGroundHeight, aeroReNumber;
extern float liftMagnitude, dragMagnitude, liftToDragRatio, momentMagnitude;
extern LbmVec3 liftVector, dragVector, momentVector, centerOfPressure;
extern long long aeroCpNonFinite;
void computeLiftDrag();
// computeLBMRefArea (lbm.cpp:2111-2160): with aeroAutoRefArea, the frontal area of g_vertices
// along the flowAzimuth / flowElevation direction (half the sum of area x |cos|), else the
// bounding-box projection; without it, aeroRefArea (1 when not positive). Host FP32, in the
// reference's order.
float computeLBMRefArea();
// computeLBMRe (lbm.cpp:2094-2108): air density x flow speed x maxDim / the Sutherland viscosity
// at lbmFacadeAirTemperature (flow_field.h:46-54); aeroReNumber when not finite; at most 1e9.
float computeLBMRe();
// computeLBMForcesFromLBM (lbm.cpp:2258-2261): lbmReynolds = aeroReNumber = computeLBMRe().
extern float lbmReynolds;
void computeLBMForcesFromLBM();

// ---- extras of this layer ----------------------------------------------------
// The C-ABI handle (NULL before initLBM): for callers that also use the batch
// or the device field pointers.
aeros_lbm* lbmFacadeHandle();
// Reads rho, u, strain and TKE into the globals now.
bool lbmFacadeReadFields();
// Message of the last failed call ("" when none).
const std::string& lbmFacadeLastError();
// Many distance samples at once (xyz each; dist n, normal 3n, either NULL).
bool voxelFacadeSampleSDF(const float* points, long long n, float* dist, float* normal);
