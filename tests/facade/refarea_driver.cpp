// computeLBMRefArea through the C++17 facade: a triangle soup (float32, 9 per
// triangle) from the file argv[1], then azimuth, elevation, auto (0/1), the
// fixed area, bbox min xyz, bbox max xyz and maxDim; prints the area.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "aeros_facade.h"

int main(int argc, char** argv) {
    if (argc < 13) return 2;
    FILE* fh = std::fopen(argv[1], "rb");
    if (!fh) return 3;
    std::vector<float> v;
    float buf[9];
    while (std::fread(buf, sizeof(float), 9, fh) == 9) v.insert(v.end(), buf, buf + 9);
    std::fclose(fh);
    g_vertices = v;
    flowAzimuth = std::strtof(argv[2], nullptr);
    flowElevation = std::strtof(argv[3], nullptr);
    aeroAutoRefArea = std::atoi(argv[4]) != 0;
    aeroRefArea = std::strtof(argv[5], nullptr);
    minBB = LbmVec3{std::strtof(argv[6], nullptr), std::strtof(argv[7], nullptr), std::strtof(argv[8], nullptr)};
    maxBB = LbmVec3{std::strtof(argv[9], nullptr), std::strtof(argv[10], nullptr), std::strtof(argv[11], nullptr)};
    maxDim = std::strtof(argv[12], nullptr);
    std::printf("%.9g\n", computeLBMRefArea());
    return 0;
}
