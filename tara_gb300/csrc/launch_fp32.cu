// FP32 instantiations of the 2D launchers (FP32 transforms and products; the
// radix-8 step kernels compile in launch_fp32_r8.cu).
#include "launch2d.cuh"

namespace tara {
TARA_STEP_R8_INSTANCES(extern, float)
template struct Launch2D<float>;
}  // namespace tara
