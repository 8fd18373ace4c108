// Axis-pass kernels, double, N in {512}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(double, 512)
}  // namespace gpe
