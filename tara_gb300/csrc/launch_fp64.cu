// FP64 instantiations of the 2D launchers (the radix-4 path; the radix-8 step
// kernels compile in launch_fp64_r8.cu).
#include "launch2d.cuh"

namespace tara {
TARA_STEP_R8_INSTANCES(extern, double)
template struct Launch2D<double>;
}  // namespace tara
