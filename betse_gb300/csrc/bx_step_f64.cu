// Plain FP64 form of the fused cell step (instantiations).
#include "bx_launch.cuh"
namespace bx {
BX_DEFINE_CELL_STEP_LAUNCHER(double, 128)
BX_DEFINE_CELL_STEP_LAUNCHER(double, 256)
}  // namespace bx
