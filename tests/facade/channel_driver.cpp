// A caller written against the reference solver interface, built on the
// C++17 facade: the 64x32x32 Poiseuille channel (walls at y = 0 and y = 31,
// periodic x and z, body force 1e-6, tau 0.8, BGK, no LES). Steps it, prints
// the globals the visualizer reads and writes lbmUx to the file argv[2].
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "aeros_facade.h"

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
    initLBM();
    if (!lbmInitialized) {
        std::fprintf(stderr, "initLBM failed: %s\n", lbmFacadeLastError().c_str());
        return 1;
    }
    for (int i = 0; i < steps / 2; ++i) stepLBMCPU(1);   // frame-loop style
    stepLBMCPU(steps - steps / 2);                          // and one batched call
    const LbmVec3 F = lbmControlVolumeForce(0.3f, 0.3f, 0.3f);
    std::printf("step %d avg_rho %.9g avg_ke %.9g max_u %.9g fx %.9g area %.1f\n", lbmCurrentStep, lbmAvgRho,
                lbmAvgKineticEnergy, lbmMaxVelocityLB, F.x, lbmProjectedAreaCells(0));
    if (argc > 2) {
        FILE* fh = std::fopen(argv[2], "wb");
        if (!fh) return 2;
        std::fwrite(lbmUx.data(), sizeof(float), lbmUx.size(), fh);
        std::fclose(fh);
    }
    shutdownLBM();
    return lbmCurrentStep == steps ? 0 : 3;
}
