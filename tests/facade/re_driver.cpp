// computeLBMRe through the C++17 facade: argv = air temperature (K), air
// density, flow speed, maxDim, previous aeroReNumber; prints the number.
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
    std::printf("%.9g\n", computeLBMRe());
    return 0;
}
