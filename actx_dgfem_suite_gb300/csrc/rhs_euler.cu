// FP64 RHS kernels for the euler equation, orders 1..4.
#include "rhs_instantiate.cuh"

namespace dg {
cudaError_t fp64_shape_euler(int order, LaunchShape* out) {
  return shape_any<DG_EULER>(order, out);
}
cudaError_t fp64_launch_euler(int order, const RhsArgs& a, int grid,
                               cudaStream_t s) {
  return launch_any<DG_EULER>(order, a, grid, s);
}
}  // namespace dg
