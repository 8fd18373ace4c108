// Paired FP32 step passes (pass_x2.cuh) on the default plan, N = 512.
#include "pass_x2_launch.cuh"

namespace gpe {
GPE_INST_PASS_X2(512, 0)
}  // namespace gpe
