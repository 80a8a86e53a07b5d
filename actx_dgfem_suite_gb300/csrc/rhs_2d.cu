// RHS kernels on triangle meshes (2D): wave, euler and maxwell (TM) at
// orders 1..4, FP64, plain RHS and fused RK stage; shape/launch entry points
// and the operator block layout of dg_rhs2d_kernel.
#include <cstring>

#include "dg_launch.h"
#include "dg_rhs2d.cuh"

namespace dg {
namespace {

template <int N, int EQ, int MODE>
cudaError_t shape2_impl(LaunchShape* out) {
  using T = Tile2<N, EQ>;
  auto kern = dg_rhs2d_kernel<N, EQ, MODE>;
  cudaError_t err = cudaFuncSetAttribute(
      kern, cudaFuncAttributeMaxDynamicSharedMemorySize, T::SMEM_BYTES);
  if (err != cudaSuccess) return err;
  int nb = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kBlock, T::SMEM_BYTES);
  out->smem_bytes = T::SMEM_BYTES;
  out->blocks_per_sm = nb;
  out->elems_per_tile = T::E;
  out->ops_bytes = Ops2<N>::SIZE;
  out->threads = kBlock;
  return err;
}

template <int N, int EQ, int MODE>
cudaError_t launch2_impl(const RhsArgs& a, int grid, cudaStream_t s) {
  dg_rhs2d_kernel<N, EQ, MODE><<<grid, kBlock, Tile2<N, EQ>::SMEM_BYTES, s>>>(a);
  return cudaGetLastError();
}

template <int N, int EQ>
cudaError_t shape2_n(int mode, LaunchShape* out) {
  return mode == MODE_RHS ? shape2_impl<N, EQ, MODE_RHS>(out)
                          : shape2_impl<N, EQ, MODE_STAGE>(out);
}

template <int N, int EQ>
cudaError_t launch2_n(int mode, const RhsArgs& a, int grid, cudaStream_t s) {
  return mode == MODE_RHS ? launch2_impl<N, EQ, MODE_RHS>(a, grid, s)
                          : launch2_impl<N, EQ, MODE_STAGE>(a, grid, s);
}

template <int EQ>
cudaError_t shape2_eq(int order, int mode, LaunchShape* out) {
  switch (order) {
    case 1: return shape2_n<1, EQ>(mode, out);
    case 2: return shape2_n<2, EQ>(mode, out);
    case 3: return shape2_n<3, EQ>(mode, out);
    case 4: return shape2_n<4, EQ>(mode, out);
    default: return cudaErrorInvalidValue;
  }
}

template <int EQ>
cudaError_t launch2_eq(int order, int mode, const RhsArgs& a, int grid, cudaStream_t s) {
  switch (order) {
    case 1: return launch2_n<1, EQ>(mode, a, grid, s);
    case 2: return launch2_n<2, EQ>(mode, a, grid, s);
    case 3: return launch2_n<3, EQ>(mode, a, grid, s);
    case 4: return launch2_n<4, EQ>(mode, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t shape_2d(int eq, int order, int mode, LaunchShape* out) {
  if (mode != MODE_RHS && mode != MODE_STAGE) return cudaErrorInvalidValue;
  switch (eq) {
    case DG_WAVE: return shape2_eq<DG_WAVE>(order, mode, out);
    case DG_EULER: return shape2_eq<DG_EULER>(order, mode, out);
    case DG_MAXWELL: return shape2_eq<DG_MAXWELL>(order, mode, out);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_2d(int eq, int order, int mode, const RhsArgs& a, int grid,
                      cudaStream_t s) {
  if (mode != MODE_RHS && mode != MODE_STAGE) return cudaErrorInvalidValue;
  switch (eq) {
    case DG_WAVE: return launch2_eq<DG_WAVE>(order, mode, a, grid, s);
    case DG_EULER: return launch2_eq<DG_EULER>(order, mode, a, grid, s);
    case DG_MAXWELL: return launch2_eq<DG_MAXWELL>(order, mode, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

int pack_ops_2d(int order, const double* diff, const double* lift,
                const int32_t* face_nodes, unsigned char* out, int out_bytes) {
  const int np = (order + 1) * (order + 2) / 2, nfpt = 3 * (order + 1);
  const int l_off = pad16(2 * np * np * 8), fn_off = l_off + pad16(nfpt * np * 8);
  const int size = fn_off + pad16(nfpt * 4);
  if (!out) return size;
  if (out_bytes < size) return -1;
  std::memset(out, 0, size);
  double* w = reinterpret_cast<double*>(out);
  double* l = reinterpret_cast<double*>(out + l_off);
  int32_t* fn = reinterpret_cast<int32_t*>(out + fn_off);
  for (int r = 0; r < 2; ++r)
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j) w[(r * np + j) * np + i] = diff[(r * np + i) * np + j];
  for (int i = 0; i < np; ++i)
    for (int fj = 0; fj < nfpt; ++fj) l[fj * np + i] = lift[i * nfpt + fj];
  for (int k = 0; k < nfpt; ++k) fn[k] = face_nodes[k];
  return size;
}

}  // namespace dg
