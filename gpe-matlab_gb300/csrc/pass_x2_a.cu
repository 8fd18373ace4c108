// Paired FP32 step passes (pass_x2.cuh) on the alternative plans, N in {256, 512}.
#include "pass_x2_launch.cuh"

namespace gpe {
GPE_INST_PASS_X2(256, 1) GPE_INST_PASS_X2(512, 1)
}  // namespace gpe
