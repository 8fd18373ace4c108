// Axis-pass kernels, double, N in {256}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(double, 256)
}  // namespace gpe
