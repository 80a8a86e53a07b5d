// Transposed Jacobian (vector-Jacobian product) of the FP64 Euler RHS,
// orders 1..4: see dg_adjoint_euler.cuh.
#include "dg_adjoint_euler.cuh"
#include "dg_launch.h"

namespace dg {
namespace {

template <int N>
cudaError_t vjp_shape_n(LaunchShape* out) {
  using T = VjpTile<N>;
  cudaError_t err = cudaFuncSetAttribute(
      dg_euler_vjp_volume<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, T::SMEM_BYTES);
  if (err != cudaSuccess) return err;
  int nb = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, dg_euler_vjp_volume<N>, kBlock,
                                                      T::SMEM_BYTES);
  out->smem_bytes = T::SMEM_BYTES;
  out->blocks_per_sm = nb;
  out->elems_per_tile = T::E;
  out->ops_bytes = AdjOpsLayout<N>::SIZE;
  return err;
}

template <int N>
cudaError_t vjp_launch_n(const VjpArgs& a, int grid, int nsm, bool stage, cudaStream_t s) {
  constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP;
  const int64_t nodes = a.nel * NP;
  const int64_t cap = (int64_t)nsm * 16;
  int64_t nb = (nodes + kBlock - 1) / kBlock;
  if (nb > cap) nb = cap;
  dg_euler_aux_kernel<DG_EULER><<<(int)nb, kFaceBlock, 0, s>>>(
      a.q, const_cast<double*>(a.aux), (uint32_t)nodes, a.gamma);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  dg_euler_vjp_volume<N><<<grid, kBlock, VjpTile<N>::SMEM_BYTES, s>>>(a);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  int64_t fb = (a.nowned * NFP + kFaceBlock - 1) / kFaceBlock;
  if (fb > cap) fb = cap;
  if (fb < 1) fb = 1;
  dg_euler_vjp_face<N><<<(int)fb, kFaceBlock, 0, s>>>(a);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  if (stage)
    dg_vjp_node_gather<N, 5, true><<<(int)nb, kBlock, 0, s>>>(a);
  else
    dg_vjp_node_gather<N, 5><<<(int)nb, kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t vjp_shape_euler(int order, LaunchShape* out) {
  switch (order) {
    case 1: return vjp_shape_n<1>(out);
    case 2: return vjp_shape_n<2>(out);
    case 3: return vjp_shape_n<3>(out);
    case 4: return vjp_shape_n<4>(out);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t vjp_launch_euler(int order, const VjpArgs& a, int grid, int nsm, bool stage,
                             cudaStream_t s) {
  switch (order) {
    case 1: return vjp_launch_n<1>(a, grid, nsm, stage, s);
    case 2: return vjp_launch_n<2>(a, grid, nsm, stage, s);
    case 3: return vjp_launch_n<3>(a, grid, nsm, stage, s);
    case 4: return vjp_launch_n<4>(a, grid, nsm, stage, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dg
