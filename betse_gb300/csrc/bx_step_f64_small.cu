// Plain FP64 form of the fused cell step, small CTAs and the one-lane-per-ion
// kernel (instantiations; a unit of its own so that it compiles in parallel
// with the larger ones).
#include "bx_launch.cuh"
namespace bx {
BX_DEFINE_CELL_STEP_LAUNCHER(double, 32)
BX_DEFINE_CELL_STEP_LAUNCHER(double, 64)
BX_DEFINE_CELL_STEP_ION_LAUNCHER(8)
BX_DEFINE_CELL_STEP_ION_LAUNCHER(16)
BX_DEFINE_CELL_STEP_ION_LAUNCHER(32)
BX_DEFINE_CELL_STEP_ION_LAUNCHER(64)
}  // namespace bx
