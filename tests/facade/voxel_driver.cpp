// A caller written against the reference's stl_loader.h / voxel_grid.h names,
// built on the C++17 facade: loads the STL file argv[1], builds the voxel
// grid at resolution argv[2] and writes to argv[3]: int32 nx ny nz, float32
// grid min (3) and max (3), the mask (nx*ny*nz uint8), the distance field
// (float32), then for the NPTS points read from argv[4] (float32 xyz) the
// distances and normals of sampleSDFCPU / sdfNormalCPU.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "aeros_facade.h"

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    std::vector<float> v, n;
    if (!loadSTL(argv[1], v, n)) {
        std::fprintf(stderr, "loadSTL: %s\n", lbmFacadeLastError().c_str());
        return 1;
    }
    buildVoxelGrid(v, std::atoi(argv[2]));
    if (!g_voxelBuildError.empty()) {
        std::fprintf(stderr, "buildVoxelGrid: %s\n", g_voxelBuildError.c_str());
        return 1;
    }
    std::vector<float> pts;
    if (FILE* fp = std::fopen(argv[4], "rb")) {
        float b[3];
        while (std::fread(b, sizeof(float), 3, fp) == 3) pts.insert(pts.end(), b, b + 3);
        std::fclose(fp);
    }
    FILE* fo = std::fopen(argv[3], "wb");
    if (!fo) return 2;
    const int dims[3] = {g_voxNx, g_voxNy, g_voxNz};
    const float box[6] = {g_voxMinX, g_voxMinY, g_voxMinZ, g_voxMaxX, g_voxMaxY, g_voxMaxZ};
    std::fwrite(dims, sizeof(int), 3, fo);
    std::fwrite(box, sizeof(float), 6, fo);
    std::vector<unsigned char> mask(g_voxelData.begin(), g_voxelData.end());
    std::fwrite(mask.data(), 1, mask.size(), fo);
    std::fwrite(g_distanceField.data(), sizeof(float), g_distanceField.size(), fo);
    for (size_t i = 0; i + 2 < pts.size(); i += 3) {
        LbmVec3 p;
        p.x = pts[i]; p.y = pts[i + 1]; p.z = pts[i + 2];
        const float d = sampleSDFCPU(p);
        const LbmVec3 nn = sdfNormalCPU(p);
        const float rec[4] = {d, nn.x, nn.y, nn.z};
        std::fwrite(rec, sizeof(float), 4, fo);
    }
    std::fclose(fo);
    std::printf("triangles %zu grid %dx%dx%d solid %lld\n", v.size() / 9, g_voxNx, g_voxNy, g_voxNz, g_voxelSolidCells);
    return 0;
}
