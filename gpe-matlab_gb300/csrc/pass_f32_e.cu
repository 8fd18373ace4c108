// Axis-pass kernels, float, N in {512}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(float, 512)
GPE_INST_PLAN(512)
}  // namespace gpe
