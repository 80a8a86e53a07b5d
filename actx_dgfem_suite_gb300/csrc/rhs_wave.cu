// RHS kernels for the wave equation: orders 1..4, FP64 and mixed
// precision, plain RHS and fused RK stage; face-shared FP64 forms with FP64
// or tensor-core contractions; mixed precision on tcgen05.
#include "rhs_instantiate.cuh"

namespace dg {
cudaError_t shape_wave(int order, int precision, int mode, LaunchShape* out) {
  return shape_any<DG_WAVE>(order, precision, mode, out);
}
cudaError_t launch_wave(int order, int precision, int mode, const RhsArgs& a,
                         int grid, cudaStream_t s) {
  return launch_any<DG_WAVE>(order, precision, mode, a, grid, s);
}
cudaError_t face_blocks_wave(int order, int* blocks_per_sm) {
  return face_blocks_any<DG_WAVE>(order, blocks_per_sm);
}
cudaError_t face_launch_wave(int order, const FaceArgs& a, int grid, int aux_grid,
                           cudaStream_t s) {
  return face_launch_any<DG_WAVE>(order, a, grid, aux_grid, s);
}
cudaError_t tc_shape_wave(int order, int mode, LaunchShape* out) {
  return tc_shape_any<DG_WAVE>(order, mode, out);
}
cudaError_t tc_launch_wave(int order, int mode, const RhsArgs& a, int grid,
                        cudaStream_t s) {
  return tc_launch_any<DG_WAVE>(order, mode, a, grid, s);
}
cudaError_t tcm_shape_wave(int order, int mode, LaunchShape* out) {
  return tcm_shape_any<DG_WAVE>(order, mode, out);
}
cudaError_t tcm_launch_wave(int order, int mode, const RhsArgs& a, int grid,
                        cudaStream_t s) {
  return tcm_launch_any<DG_WAVE>(order, mode, a, grid, s);
}
}  // namespace dg
