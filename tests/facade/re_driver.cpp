// computeLBMRe through the C++17 facade: argv = air temperature (K), air
// density, flow speed, maxDim, previous aeroReNumber; prints the number, then
// lbmReynolds and aeroReNumber after computeLBMForcesFromLBM.
#include <cstdio>
#include <cstdlib>

#include "aeros_facade.h"

int main(int argc, char** argv) {
    if (argc < 6) return 2;
    lbmFacadeAirTemperature = std::strtof(argv[1], nullptr);
    lbmFacadeAirDensity = std::strtof(argv[2], nullptr);
    lbmFacadeFlowSpeed = std::strtof(argv[3], nullptr);
    maxDim = std::strtof(argv[4], nullptr);
    aeroReNumber = std::strtof(argv[5], nullptr);
    const float re = computeLBMRe();
    computeLBMForcesFromLBM();
    std::printf("%.9g %.9g %.9g\n", re, lbmReynolds, aeroReNumber);
    return 0;
}
