// Axis-pass kernels, float, N in {768, 1024}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(float, 768)
GPE_INST_PLAN(768)
GPE_INST_PASS(float, 1024)
GPE_INST_PLAN(1024)
}  // namespace gpe
