// FP16 / BF16 shifted populations (f_i - w_i), FP32 arithmetic. Compiled with
// FMA contraction on: this form is measured against the FP64 run, not
// bit-matched.
#include "lbm_aux.cuh"

namespace aeros {
AEROS_DEFINE_LAUNCHERS(launchers_fp16, StoreF16)
AEROS_DEFINE_LAUNCHERS(launchers_bf16, StoreBF16)
}
