// Axis-pass kernels with the alternative plans (plans.cuh PlanAlt), float.
#include "pass_launch.cuh"

namespace gpe {
GPE_INST_PASS_ALT(256)
}  // namespace gpe
