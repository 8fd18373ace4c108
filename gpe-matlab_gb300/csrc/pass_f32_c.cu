// Axis-pass kernels, float, N in {256}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(float, 256)
GPE_INST_PLAN(256)
}  // namespace gpe
