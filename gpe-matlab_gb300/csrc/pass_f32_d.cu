// Axis-pass kernels, float, N in {384}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(float, 384)
GPE_INST_PLAN(384)
}  // namespace gpe
