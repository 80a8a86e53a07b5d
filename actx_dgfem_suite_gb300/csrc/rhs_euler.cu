// RHS kernels for the euler equation: orders 1..4, FP64 and mixed
// precision, plain RHS and fused RK stage; face-shared FP64 forms with FP64
// or tensor-core contractions; mixed precision on tcgen05.
#include "rhs_instantiate.cuh"

namespace dg {
cudaError_t shape_euler(int order, int precision, int mode, LaunchShape* out) {
  return shape_any<DG_EULER>(order, precision, mode, out);
}
cudaError_t launch_euler(int order, int precision, int mode, const RhsArgs& a,
                         int grid, cudaStream_t s) {
  return launch_any<DG_EULER>(order, precision, mode, a, grid, s);
}
cudaError_t face_blocks_euler(int order, int* blocks_per_sm) {
  return face_blocks_any<DG_EULER>(order, blocks_per_sm);
}
cudaError_t face_launch_euler(int order, const FaceArgs& a, int grid, int aux_grid,
                           cudaStream_t s) {
  return face_launch_any<DG_EULER>(order, a, grid, aux_grid, s);
}
cudaError_t tc_shape_euler(int order, int mode, LaunchShape* out) {
  return tc_shape_any<DG_EULER>(order, mode, out);
}
cudaError_t tc_launch_euler(int order, int mode, const RhsArgs& a, int grid,
                        cudaStream_t s) {
  return tc_launch_any<DG_EULER>(order, mode, a, grid, s);
}
cudaError_t tcm_shape_euler(int order, int mode, LaunchShape* out) {
  return tcm_shape_any<DG_EULER>(order, mode, out);
}
cudaError_t tcm_launch_euler(int order, int mode, const RhsArgs& a, int grid,
                        cudaStream_t s) {
  return tcm_launch_any<DG_EULER>(order, mode, a, grid, s);
}

// Mixed-precision Euler: the pressure of every node, recovered from total
// energy in FP64 with the mixed kernels' reciprocal (FP32 estimate refined
// by one Newton step) and stored as FP32, the flux arithmetic's type.  Once
// per node, where the kernels would otherwise recover it for every node and
// again for the exterior side of every face point on the FP64 pipe.
__global__ void __launch_bounds__(kFaceBlock)
    dg_euler_pressure_f32_kernel(const double* __restrict__ q, float* __restrict__ pres,
                                 int64_t nelnp, double gamma) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nelnp;
       idx += stride) {
    const double rho = __ldg(q + idx);
    const double en = __ldg(q + nelnp + idx);
    const double m0 = __ldg(q + 2 * nelnp + idx);
    const double m1 = __ldg(q + 3 * nelnp + idx);
    const double m2 = __ldg(q + 4 * nelnp + idx);
    const double rinv = rcp64_fast(rho);
    pres[idx] = d2f_alu((gamma - 1.0) * (en - 0.5 * (m0 * m0 + m1 * m1 + m2 * m2) * rinv));
  }
}

cudaError_t pressure_launch_euler(const double* q, float* pres, int64_t nelnp,
                                  double gamma, int grid, cudaStream_t s) {
  dg_euler_pressure_f32_kernel<<<grid, kFaceBlock, 0, s>>>(q, pres, nelnp, gamma);
  return cudaGetLastError();
}
}  // namespace dg
