// FP32 step kernels along the radix-8 path.
#include "launch2d.cuh"

namespace tara {
TARA_STEP_R8_INSTANCES(, float)
}  // namespace tara
