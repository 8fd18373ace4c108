// Paired FP32 step passes (pass_x2.cuh), N in {128, 192, 384}.
#include "pass_x2_launch.cuh"

namespace gpe {
GPE_INST_PASS_X2(128) GPE_INST_PASS_X2(192) GPE_INST_PASS_X2(384)
}  // namespace gpe
