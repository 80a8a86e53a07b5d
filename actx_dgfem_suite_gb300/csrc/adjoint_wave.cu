// Adjoint (transpose) kernels of the FP64 wave RHS, orders 1..4.
#include "dg_adjoint.cuh"
#include "dg_launch.h"

namespace dg {
namespace {

template <int N>
cudaError_t adj_shape_n(LaunchShape* out) {
  using T = AdjTile<N>;
  cudaError_t err = cudaFuncSetAttribute(
      dg_wave_adjoint_volume<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      T::SMEM_BYTES);
  if (err != cudaSuccess) return err;
  int nb = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &nb, dg_wave_adjoint_volume<N>, kBlock, T::SMEM_BYTES);
  out->smem_bytes = T::SMEM_BYTES;
  out->blocks_per_sm = nb;
  out->elems_per_tile = T::E;
  out->ops_bytes = AdjOpsLayout<N>::SIZE;
  return err;
}

template <int N>
cudaError_t adj_launch_n(const AdjArgs& a, int grid, int nsm, cudaStream_t s) {
  dg_wave_adjoint_volume<N><<<grid, kBlock, AdjTile<N>::SMEM_BYTES, s>>>(a);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  const int64_t nodes = a.nel * Shape<N>::NP;
  int64_t blocks = (nodes + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)nsm * 16;
  if (blocks > cap) blocks = cap;
  dg_wave_adjoint_surface<N><<<(int)blocks, kBlock, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t adjoint_shape_wave(int order, LaunchShape* out) {
  switch (order) {
    case 1: return adj_shape_n<1>(out);
    case 2: return adj_shape_n<2>(out);
    case 3: return adj_shape_n<3>(out);
    case 4: return adj_shape_n<4>(out);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t adjoint_launch_wave(int order, const AdjArgs& a, int grid, int nsm,
                                cudaStream_t s) {
  switch (order) {
    case 1: return adj_launch_n<1>(a, grid, nsm, s);
    case 2: return adj_launch_n<2>(a, grid, nsm, s);
    case 3: return adj_launch_n<3>(a, grid, nsm, s);
    case 4: return adj_launch_n<4>(a, grid, nsm, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dg
