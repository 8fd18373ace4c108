// Axis-pass kernels, double, N in {768, 1024}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(double, 768)
GPE_INST_PASS(double, 1024)
}  // namespace gpe
