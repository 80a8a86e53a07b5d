// Instantiates the FP64 RHS kernel of one equation for orders 1..4 and
// defines its shape/launch entry points.  Included by exactly one .cu file
// per equation with DG_EQ and DG_NAME defined.
#pragma once

#include "dg_launch.h"
#include "dg_rhs_fp64.cuh"

namespace dg {
namespace {

template <int N, int EQ>
cudaError_t shape_impl(LaunchShape* out) {
  using T = Tile<N, EQ>;
  auto kern = dg_rhs_fp64_kernel<N, EQ>;
  cudaError_t err = cudaFuncSetAttribute(
      kern, cudaFuncAttributeMaxDynamicSharedMemorySize, T::SMEM_BYTES);
  if (err != cudaSuccess) return err;
  int nb = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kBlock,
                                                      T::SMEM_BYTES);
  out->smem_bytes = T::SMEM_BYTES;
  out->blocks_per_sm = nb;
  out->elems_per_tile = T::E;
  out->ops_doubles = OpsLayout<N>::SIZE;
  return err;
}

template <int N, int EQ>
cudaError_t launch_impl(const RhsArgs& a, int grid, cudaStream_t s) {
  using T = Tile<N, EQ>;
  dg_rhs_fp64_kernel<N, EQ><<<grid, kBlock, T::SMEM_BYTES, s>>>(a);
  return cudaGetLastError();
}

template <int EQ>
cudaError_t shape_any(int order, LaunchShape* out) {
  switch (order) {
    case 1: return shape_impl<1, EQ>(out);
    case 2: return shape_impl<2, EQ>(out);
    case 3: return shape_impl<3, EQ>(out);
    case 4: return shape_impl<4, EQ>(out);
    default: return cudaErrorInvalidValue;
  }
}

template <int EQ>
cudaError_t launch_any(int order, const RhsArgs& a, int grid, cudaStream_t s) {
  switch (order) {
    case 1: return launch_impl<1, EQ>(a, grid, s);
    case 2: return launch_impl<2, EQ>(a, grid, s);
    case 3: return launch_impl<3, EQ>(a, grid, s);
    case 4: return launch_impl<4, EQ>(a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace
}  // namespace dg
