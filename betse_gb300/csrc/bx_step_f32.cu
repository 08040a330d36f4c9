// FP32/FP64-split form of the fused cell step (instantiations): fluxes and
// pumps in FP32, segment sums, concentrations and Vmem in FP64.
#include "bx_launch.cuh"
namespace bx {
BX_DEFINE_CELL_STEP_LAUNCHER(float, 128)
BX_DEFINE_CELL_STEP_LAUNCHER(float, 256)
}  // namespace bx
