// FP64 RHS kernels for the maxwell equation, orders 1..4.
#include "rhs_instantiate.cuh"

namespace dg {
cudaError_t fp64_shape_maxwell(int order, LaunchShape* out) {
  return shape_any<DG_MAXWELL>(order, out);
}
cudaError_t fp64_launch_maxwell(int order, const RhsArgs& a, int grid,
                               cudaStream_t s) {
  return launch_any<DG_MAXWELL>(order, a, grid, s);
}
}  // namespace dg
