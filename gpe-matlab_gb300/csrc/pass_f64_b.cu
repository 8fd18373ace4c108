// Axis-pass kernels, double, N in {128, 192}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(double, 128)
GPE_INST_PASS(double, 192)
}  // namespace gpe
