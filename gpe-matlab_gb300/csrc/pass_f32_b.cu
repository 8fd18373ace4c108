// Axis-pass kernels, float, N in {128, 192}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(float, 128)
GPE_INST_PLAN(128)
GPE_INST_PASS(float, 192)
GPE_INST_PLAN(192)
}  // namespace gpe
