// Double-float instantiations of the RHS launchers (transforms and products in
// FP32 pairs of about 48 significant bits; the state update stays FP64).  Only
// the three RHS passes are instantiated: the plain transforms, diagnostics and
// initial conditions of a double-float solver run in FP64.
#include "launch2d.cuh"

namespace tara {
template int Launch2D<df64>::col_inverse(int, int, const double2*, void*, const Grid2D&, const RhsParams&,
                                         const void*, cudaStream_t, int, int);
template int Launch2D<df64>::row_nl(int, int, const void*, void*, const Grid2D&, const void*, cudaStream_t, int,
                                    int);
template int Launch2D<df64>::col_forward(int, int, const void*, const StepBufs&, const Grid2D&, const RhsParams&,
                                         int, const void*, cudaStream_t, int, int);
template bool Launch2D<df64>::tile_fits(int, int, int);
}  // namespace tara
