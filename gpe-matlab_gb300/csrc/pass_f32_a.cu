// Axis-pass kernels, float, N in {8, 12, 16, 24, 32, 48, 64, 96}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(float, 8)
GPE_INST_PLAN(8)
GPE_INST_PASS(float, 12)
GPE_INST_PLAN(12)
GPE_INST_PASS(float, 16)
GPE_INST_PLAN(16)
GPE_INST_PASS(float, 24)
GPE_INST_PLAN(24)
GPE_INST_PASS(float, 32)
GPE_INST_PLAN(32)
GPE_INST_PASS(float, 48)
GPE_INST_PLAN(48)
GPE_INST_PASS(float, 64)
GPE_INST_PLAN(64)
GPE_INST_PASS(float, 96)
GPE_INST_PLAN(96)
}  // namespace gpe
