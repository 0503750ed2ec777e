// A caller written against the reference solver interface, built on the
// C++17 facade: the 64x32x32 Poiseuille channel (walls at y = 0 and y = 31,
// periodic x and z, body force 1e-6, tau 0.8, BGK, no LES), placed in world
// space at (-3.2, -1.6, -1.6) with 0.1 m cells. Steps it, prints the globals
// the visualizer reads and writes to the file argv[2], as float32:
// lbmUx, lbmUxWorld, lbmUyWorld, lbmPressure, lbmVorticityMag, lbmQCriterion,
// lbmStrainMag (cells each), then NPTS sample points (xyz) and, for each field
// 0..7 of lbmFacadeSample, its values (3 per point for the velocity) and
// validity flags (as floats); then the box mesh of the lift / drag call
// (vertices, normals: 108 floats each).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "aeros_facade.h"

namespace {
constexpr int NPTS = 64;

void put(FILE* fh, const std::vector<float>& v) { std::fwrite(v.data(), sizeof(float), v.size(), fh); }
}  // namespace

int main(int argc, char** argv) {
    const int steps = argc > 1 ? std::atoi(argv[1]) : 200;
    g_voxNx = 64;
    g_voxNy = 32;
    g_voxNz = 32;
    g_voxelData.assign((size_t)g_voxNx * g_voxNy * g_voxNz, 0);
    for (int z = 0; z < g_voxNz; ++z)
        for (int x = 0; x < g_voxNx; ++x) {
            g_voxelData[(size_t)(z * g_voxNy + 0) * g_voxNx + x] = 1;
            g_voxelData[(size_t)(z * g_voxNy + g_voxNy - 1) * g_voxNx + x] = 1;
        }
    lbmParams.tau = 0.8f;
    lbmParams.useTurbulence = false;
    lbmParams.useTRT = false;
    lbmParams.periodicX = true;
    lbmParams.periodicZ = true;
    lbmParams.bodyForceX = 1e-6f;
    lbmParams.U0 = 0.0f;
    lbmInletVelocityLB[0] = 0.0f;
    lbmMinX = -3.2f;
    lbmMinY = -1.6f;
    lbmMinZ = -1.6f;
    lbmCellSizeX = lbmCellSizeY = lbmCellSizeZ = 0.1f;
    lbmFacadeFlowSpeed = 10.0f;
    lbmFacadeAirDensity = 1.225f;
    initLBM();
    if (!lbmInitialized) {
        std::fprintf(stderr, "initLBM failed: %s\n", lbmFacadeLastError().c_str());
        return 1;
    }
    lbmFacadeFreestream[0] = 10.0f;
    lbmParams.enabled = true;
    for (int i = 0; i < steps / 2; ++i) updateLBM(0.01f, 1);   // frame-loop style
    stepLBMCPU(steps - steps / 2);                               // and one batched call
    computeLBMVorticityAndQ();
    const LbmVec3 F = lbmControlVolumeForce(0.3f, 0.3f, 0.3f);
    std::printf("step %d avg_rho %.9g avg_ke %.9g max_u %.9g fx %.9g area %.1f\n", lbmCurrentStep, lbmAvgRho,
                lbmAvgKineticEnergy, lbmMaxVelocityLB, F.x, lbmProjectedAreaCells(0));
    std::printf("pmin %.9g pmax %.9g res_rho %.9g res_u %.9g nonfinite %lld\n", lbmPressureMin, lbmPressureMax,
                lbmResidualRho, lbmResidualU, lbmPressureNonFinite);
    // points on a diagonal through the channel, some outside it and some in the walls
    std::vector<float> pts(3 * NPTS);
    for (int i = 0; i < NPTS; ++i) {
        const float t = (float)i / (float)(NPTS - 1);
        pts[3 * i + 0] = -3.4f + 6.8f * t;
        pts[3 * i + 1] = -1.7f + 3.4f * t;
        pts[3 * i + 2] = 0.37f - 0.5f * t;
    }
    LbmVec3 mid;
    mid.x = pts[3 * 20];
    mid.y = pts[3 * 20 + 1];
    mid.z = pts[3 * 20 + 2];
    float pa = 0.0f;
    const bool pok = getLBMPressureWorldChecked(mid, &pa);
    const LbmVec3 u = getLBMVelocityLB(mid);
    std::printf("probe p %.9g ok %d ux %.9g rho %.9g q %.9g vort %.9g strain %.9g tke %.9g solid %d %d\n", pa, (int)pok,
                u.x, getLBMDensityWorld(mid), getLBMQWorld(mid), getLBMVorticityWorld(mid), getLBMStrainWorld(mid),
                getLBMTKEWorld(mid), (int)isLBMSolidWorld(mid), (int)isLBMSolidWorld(LbmVec3{-3.0f, -1.58f, 0.0f}));
    const LbmVec3 vw = getLBMVelocityWorld(mid);
    std::printf("world ux %.9g uy %.9g mag %.9g mach %.9g dt %.9g outside %.9g\n", vw.x, vw.y, getLBMVelocityMagWorld(mid),
                getLBMMachWorld(mid), lbmLatticeDtWorld(), getLBMVelocityWorld(LbmVec3{9.0f, 0.0f, 0.0f}).x);
    // the equilibrium moments of the reference's own test states
    const float eq[7][4] = {{1.0f, 0.0f, 0.0f, 0.0f},    {1.0f, 0.05f, 0.0f, 0.0f},  {0.7f, 0.04f, -0.03f, 0.02f},
                            {1.35f, -0.02f, 0.05f, 0.01f}, {0.55f, 0.1f, 0.1f, 0.0f}, {1.6f, 0.0f, 0.0f, -0.08f},
                            {1.1f, 0.28f, 0.0f, 0.0f}};
    for (const auto& c : eq) {
        float m = 0.0f, px = 0.0f, py = 0.0f, pz = 0.0f;
        const bool good = lbmEquilibriumMoments(c[0], c[1], c[2], c[3], &m, &px, &py, &pz);
        std::printf("eq %d %.9g %.9g %.9g %.9g\n", (int)good, m, px, py, pz);
    }
    std::printf("validate %d %d %d %d %d %d\n", (int)lbmValidateInitialization(), (int)lbmValidateConservation(),
                (int)lbmValidateBoundaryConditions(), (int)lbmValidateSolidHandling(), (int)lbmValidateRealisticAero(),
                (int)lbmValidateStability());
    // lift and drag on a 1 m box around the origin (12 triangles, face normals)
    g_vertices.clear();
    g_normals.clear();
    for (int a = 0; a < 3; ++a)
        for (int sgn = -1; sgn <= 1; sgn += 2) {
            const int b = (a + 1) % 3, c = (a + 2) % 3;
            const float q[4][2] = {{-0.5f, -0.5f}, {0.5f, -0.5f}, {0.5f, 0.5f}, {-0.5f, 0.5f}};
            const int tri[2][3] = {{0, 1, 2}, {0, 2, 3}};
            for (const auto& t : tri)
                for (int k = 0; k < 3; ++k) {
                    float v[3], n[3] = {0.0f, 0.0f, 0.0f};
                    v[a] = 0.5f * (float)sgn;
                    v[b] = q[t[k]][0];
                    v[c] = q[t[k]][1];
                    n[a] = (float)sgn;
                    g_vertices.insert(g_vertices.end(), v, v + 3);
                    g_normals.insert(g_normals.end(), n, n + 3);
                }
        }
    minBB = LbmVec3{-0.5f, -0.5f, -0.5f};
    maxBB = LbmVec3{0.5f, 0.5f, 0.5f};
    center = LbmVec3{0.0f, 0.0f, 0.0f};
    maxDim = 1.7320508f;
    aeroReNumber = 3e5f;
    computeLiftDrag();
    std::printf("forces drag %.9g lift %.9g ld %.9g moment %.9g cop %.9g %.9g %.9g area %.9g bad %lld\n",
                dragMagnitude, liftMagnitude, liftToDragRatio, momentMagnitude, centerOfPressure.x, centerOfPressure.y,
                centerOfPressure.z, aeroRefArea, aeroCpNonFinite);
    if (argc > 2) {
        FILE* fh = std::fopen(argv[2], "wb");
        if (!fh) return 2;
        for (const std::vector<float>* v : {&lbmUx, &lbmUxWorld, &lbmUyWorld, &lbmPressure, &lbmVorticityMag,
                                            &lbmQCriterion, &lbmStrainMag})
            put(fh, *v);
        put(fh, pts);
        for (int f = AEROS_FIELD_VELOCITY_LB; f <= AEROS_FIELD_SOLID; ++f) {
            std::vector<float> out((size_t)NPTS * (f == AEROS_FIELD_VELOCITY_LB ? 3 : 1));
            std::vector<uint8_t> valid(NPTS);
            if (!lbmFacadeSample(f, pts.data(), NPTS, out.data(), valid.data())) return 4;
            put(fh, out);
            put(fh, std::vector<float>(valid.begin(), valid.end()));
        }
        put(fh, g_vertices);
        put(fh, g_normals);
        std::fclose(fh);
    }
    shutdownLBM();
    return lbmCurrentStep == steps ? 0 : 3;
}
