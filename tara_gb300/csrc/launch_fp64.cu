// FP64 instantiations of the 2D launchers.
#include "launch2d.cuh"

namespace tara {
template struct Launch2D<double>;
}  // namespace tara
