// Adjoint (transpose) kernels of the FP64 wave RHS, orders 1..4.
#include "dg_adjoint.cuh"
#include "dg_launch.h"

namespace dg {
namespace {

template <int N>
cudaError_t adj_shape_n(LaunchShape* out) {
  using T = AdjTile<N>;
  int nb = 0;
  for (int stage = 0; stage < 2; ++stage) {  // both forms, the smaller occupancy
    auto* fn = stage ? dg_wave_adjoint_volume<N, true> : dg_wave_adjoint_volume<N, false>;
    cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           T::SMEM_BYTES);
    if (err != cudaSuccess) return err;
    int b = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, kBlock, T::SMEM_BYTES);
    if (err != cudaSuccess) return err;
    nb = stage == 0 || b < nb ? b : nb;
  }
  out->smem_bytes = T::SMEM_BYTES;
  out->blocks_per_sm = nb;
  out->elems_per_tile = T::E;
  out->ops_bytes = AdjOpsLayout<N>::SIZE;
  return cudaSuccess;
}

template <int N, bool STAGE>
cudaError_t adj_launch_n(const AdjArgs& a, int grid, int nsm, cudaStream_t s) {
  dg_wave_adjoint_volume<N, STAGE><<<grid, kBlock, AdjTile<N>::SMEM_BYTES, s>>>(a);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  const int64_t nodes = a.nel * Shape<N>::NP;
  int64_t blocks = (nodes + kBlock - 1) / kBlock;
  const int64_t cap = (int64_t)nsm * 16;
  if (blocks > cap) blocks = cap;
  dg_wave_adjoint_surface<N, STAGE><<<(int)blocks, kBlock, 0, s>>>(a);
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
    case 1: return adj_launch_n<1, false>(a, grid, nsm, s);
    case 2: return adj_launch_n<2, false>(a, grid, nsm, s);
    case 3: return adj_launch_n<3, false>(a, grid, nsm, s);
    case 4: return adj_launch_n<4, false>(a, grid, nsm, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t adjoint_stage_launch_wave(int order, const AdjArgs& a, int grid, int nsm,
                                      cudaStream_t s) {
  switch (order) {
    case 1: return adj_launch_n<1, true>(a, grid, nsm, s);
    case 2: return adj_launch_n<2, true>(a, grid, nsm, s);
    case 3: return adj_launch_n<3, true>(a, grid, nsm, s);
    case 4: return adj_launch_n<4, true>(a, grid, nsm, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dg
