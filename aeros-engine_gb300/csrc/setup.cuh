// setup.cuh — device-side descriptor construction (see setup.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace aeros {

struct DescArgs {
    int nx, ny, nz;
    int flow_axis;
    int inlet_pos, outlet_pos, ic, ic2;   // coordinates along the flow axis
    int outlet_mode;                      // outlet side buffer in use
};

// mask: AEROS_CELL_* bytes on the device; tmp0/tmp1: ncell bytes of scratch.
cudaError_t build_descriptors(const DescArgs& a, const uint8_t* d_mask, uint8_t* d_tmp0, uint8_t* d_tmp1,
                              uint32_t* d_desc, cudaStream_t s);

}  // namespace aeros
