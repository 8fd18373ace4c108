// Axis-pass kernels, double, N in {384}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(double, 384)
}  // namespace gpe
