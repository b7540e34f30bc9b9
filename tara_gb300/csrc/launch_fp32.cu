// FP32 instantiations of the 2D launchers (FP32 transforms and products).
#include "launch2d.cuh"

namespace tara {
template struct Launch2D<float>;
}  // namespace tara
