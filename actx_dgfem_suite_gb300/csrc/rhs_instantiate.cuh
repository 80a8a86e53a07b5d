// Instantiates the RHS kernel of one equation for orders 1..4, FP64 and
// mixed precision, plain RHS and fused RK stage, and defines the equation's
// shape/launch entry points.  Included by exactly one .cu file per equation.
#pragma once

#include "dg_launch.h"
#include "dg_rhs.cuh"

namespace dg {
namespace {

template <int N, int EQ, typename Real, int MODE>
cudaError_t shape_impl(LaunchShape* out) {
  using T = Tile<N, EQ, Real>;
  auto kern = dg_rhs_kernel<N, EQ, Real, MODE>;
  cudaError_t err = cudaFuncSetAttribute(
      kern, cudaFuncAttributeMaxDynamicSharedMemorySize, T::SMEM_BYTES);
  if (err != cudaSuccess) return err;
  int nb = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kBlock,
                                                      T::SMEM_BYTES);
  out->smem_bytes = T::SMEM_BYTES;
  out->blocks_per_sm = nb;
  out->elems_per_tile = T::E;
  out->ops_bytes = OpsLayout<N, Real>::SIZE;
  return err;
}

template <int N, int EQ, typename Real, int MODE>
cudaError_t launch_impl(const RhsArgs& a, int grid, cudaStream_t s) {
  using T = Tile<N, EQ, Real>;
  dg_rhs_kernel<N, EQ, Real, MODE><<<grid, kBlock, T::SMEM_BYTES, s>>>(a);
  return cudaGetLastError();
}

template <int N, int EQ>
cudaError_t shape_n(int precision, int mode, LaunchShape* out) {
  if (precision == 0)
    return mode == 0 ? shape_impl<N, EQ, double, MODE_RHS>(out)
                     : shape_impl<N, EQ, double, MODE_STAGE>(out);
  return mode == 0 ? shape_impl<N, EQ, float, MODE_RHS>(out)
                   : shape_impl<N, EQ, float, MODE_STAGE>(out);
}

template <int N, int EQ>
cudaError_t launch_n(int precision, int mode, const RhsArgs& a, int grid,
                     cudaStream_t s) {
  if (precision == 0)
    return mode == 0 ? launch_impl<N, EQ, double, MODE_RHS>(a, grid, s)
                     : launch_impl<N, EQ, double, MODE_STAGE>(a, grid, s);
  return mode == 0 ? launch_impl<N, EQ, float, MODE_RHS>(a, grid, s)
                   : launch_impl<N, EQ, float, MODE_STAGE>(a, grid, s);
}

template <int EQ>
cudaError_t shape_any(int order, int precision, int mode, LaunchShape* out) {
  if ((precision != 0 && precision != 1) || (mode != 0 && mode != 1))
    return cudaErrorInvalidValue;
  switch (order) {
    case 1: return shape_n<1, EQ>(precision, mode, out);
    case 2: return shape_n<2, EQ>(precision, mode, out);
    case 3: return shape_n<3, EQ>(precision, mode, out);
    case 4: return shape_n<4, EQ>(precision, mode, out);
    default: return cudaErrorInvalidValue;
  }
}

template <int EQ>
cudaError_t launch_any(int order, int precision, int mode, const RhsArgs& a,
                       int grid, cudaStream_t s) {
  if ((precision != 0 && precision != 1) || (mode != 0 && mode != 1))
    return cudaErrorInvalidValue;
  switch (order) {
    case 1: return launch_n<1, EQ>(precision, mode, a, grid, s);
    case 2: return launch_n<2, EQ>(precision, mode, a, grid, s);
    case 3: return launch_n<3, EQ>(precision, mode, a, grid, s);
    case 4: return launch_n<4, EQ>(precision, mode, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace
}  // namespace dg
