// forces.cuh — control-volume momentum balance (aeros/src/lbm.cpp:2183-2232)
// and projected area (lbm.cpp:2236-2256) on the device.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace aeros {

struct ForceArgs {
    int nx, ny, nz;
    const uint32_t* desc;
    const float* rho;
    const float4* u;          // (ux, uy, uz, 0) per cell
    int box[6];              // x0 x1 y0 y1 z0 z1, inclusive
    double* partials;        // 3 per block
    double* out;             // 3 sums (not negated)
    unsigned int* counter;   // last-block ticket, left at zero
};

constexpr int FORCE_BLOCK = 256;

// Blocks needed for one box (at most `max_blocks`).
int cv_force_blocks(const int box[6], int max_blocks);
cudaError_t launch_cv_force(const ForceArgs& a, int blocks, cudaStream_t s);
// Counts (a, b) columns with a body cell along `axis`; `count` is zeroed first.
cudaError_t launch_projected_area(int nx, int ny, int nz, const uint32_t* desc, int axis,
                                  unsigned long long* count, cudaStream_t s);

}  // namespace aeros
