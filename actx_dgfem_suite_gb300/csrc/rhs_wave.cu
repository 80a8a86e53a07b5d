// FP64 RHS kernels for the wave equation, orders 1..4.
#include "rhs_instantiate.cuh"

namespace dg {
cudaError_t fp64_shape_wave(int order, LaunchShape* out) {
  return shape_any<DG_WAVE>(order, out);
}
cudaError_t fp64_launch_wave(int order, const RhsArgs& a, int grid,
                               cudaStream_t s) {
  return launch_any<DG_WAVE>(order, a, grid, s);
}
}  // namespace dg
