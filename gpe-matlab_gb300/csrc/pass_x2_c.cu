// Paired FP32 step passes (pass_x2.cuh) on the default plans, N in {128, 256}.
#include "pass_x2_launch.cuh"

namespace gpe {
GPE_INST_PASS_X2(128, 0) GPE_INST_PASS_X2(256, 0)
}  // namespace gpe
