// Axis-pass kernels, double, N in {8, 12, 16, 24, 32, 48, 64, 96}.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS(double, 8)
GPE_INST_PASS(double, 12)
GPE_INST_PASS(double, 16)
GPE_INST_PASS(double, 24)
GPE_INST_PASS(double, 32)
GPE_INST_PASS(double, 48)
GPE_INST_PASS(double, 64)
GPE_INST_PASS(double, 96)
}  // namespace gpe
