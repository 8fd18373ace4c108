// Paired FP32 step passes (pass_x2.cuh) on the alternative plans, N in {128, 192, 384}.
#include "pass_x2_launch.cuh"

namespace gpe {
GPE_INST_PASS_X2(128, 1) GPE_INST_PASS_X2(192, 1) GPE_INST_PASS_X2(384, 1)
}  // namespace gpe
