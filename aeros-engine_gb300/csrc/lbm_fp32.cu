// FP32 populations: the drop-in form. Compiled with --fmad=false so every
// float operation rounds separately, as the reference's x86-64 build does.
#include "lbm_aux.cuh"

namespace aeros {
AEROS_DEFINE_LAUNCHERS(launchers_fp32, StoreF32)
}
