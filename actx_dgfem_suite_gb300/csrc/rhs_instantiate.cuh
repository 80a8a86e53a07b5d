// Instantiates the RHS kernel of one equation for orders 1..4, FP64 and
// mixed precision, plain RHS and fused RK stage (FP64 also in the
// face-shared split form, with its face kernel; mixed precision also with
// the contractions on mma.sync tensor cores at three tile shapes, and on
// tcgen05), and defines the equation's shape/launch entry points.  Included
// by exactly one .cu file per equation.
#pragma once

#include <type_traits>

#include "dg_face.cuh"
#include "dg_tc.cuh"
#include "dg_tcm.cuh"
#include "dg_launch.h"
#include "dg_rhs.cuh"

namespace dg {
namespace {

template <int N, int EQ, typename Real, int MODE>
constexpr int smem_of() {
  using T = Tile<N, EQ, Real, (MODE & MODE_SPLIT) != 0, block_of(MODE)>;
  return (MODE & MODE_TC) ? T::SMEM_BYTES_TC : T::SMEM_BASE;
}

// dynamic shared memory a CTA may request (227 KB on sm_100 / sm_103)
constexpr int kMaxDynSmem = 227 * 1024;

// A tile shape whose shared memory exceeds the CTA limit is reported with
// blocks_per_sm = 0 (not supported) instead of an error, and never launched.
template <int N, int EQ, typename Real, int MODE>
cudaError_t shape_impl(LaunchShape* out) {
  using T = Tile<N, EQ, Real, (MODE & MODE_SPLIT) != 0, block_of(MODE)>;
  constexpr int SMEM = smem_of<N, EQ, Real, MODE>();
  out->smem_bytes = SMEM;
  out->blocks_per_sm = 0;
  out->elems_per_tile = T::E;
  out->ops_bytes = OpsLayout<N, Real>::SIZE;
  out->threads = block_of(MODE);
  if constexpr (SMEM > kMaxDynSmem) {
    return cudaSuccess;
  } else {
    auto kern = dg_rhs_kernel<N, EQ, Real, MODE>;
    cudaError_t err = cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (err != cudaSuccess) return err;
    int nb = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, block_of(MODE), SMEM);
    out->blocks_per_sm = nb;
    return err;
  }
}

template <int N, int EQ, typename Real, int MODE>
cudaError_t launch_impl(const RhsArgs& a, int grid, cudaStream_t s) {
  constexpr int SMEM = smem_of<N, EQ, Real, MODE>();
  if constexpr (SMEM > kMaxDynSmem) {
    return cudaErrorInvalidConfiguration;
  } else {
    dg_rhs_kernel<N, EQ, Real, MODE><<<grid, block_of(MODE), SMEM, s>>>(a);
    return cudaGetLastError();
  }
}

template <int N, int EQ, typename Real>
cudaError_t shape_mode(int mode, LaunchShape* out) {
  switch (mode) {
    case MODE_RHS: return shape_impl<N, EQ, Real, MODE_RHS>(out);
    case MODE_STAGE: return shape_impl<N, EQ, Real, MODE_STAGE>(out);
    default: break;
  }
  if constexpr (std::is_same<Real, double>::value) {
    switch (mode) {
      case MODE_SPLIT: return shape_impl<N, EQ, Real, MODE_SPLIT>(out);
      case MODE_SPLIT | MODE_STAGE:
        return shape_impl<N, EQ, Real, MODE_SPLIT | MODE_STAGE>(out);
      default: break;
    }
  } else {
    constexpr int T1 = MODE_TC | MODE_B128, T5 = MODE_TC | MODE_B512;
    switch (mode) {
      case MODE_TC: return shape_impl<N, EQ, Real, MODE_TC>(out);
      case MODE_TC | MODE_STAGE: return shape_impl<N, EQ, Real, MODE_TC | MODE_STAGE>(out);
      case T1: return shape_impl<N, EQ, Real, T1>(out);
      case T1 | MODE_STAGE: return shape_impl<N, EQ, Real, T1 | MODE_STAGE>(out);
      case T5: return shape_impl<N, EQ, Real, T5>(out);
      case T5 | MODE_STAGE: return shape_impl<N, EQ, Real, T5 | MODE_STAGE>(out);
      default: break;
    }
  }
  return cudaErrorInvalidValue;
}

template <int N, int EQ, typename Real>
cudaError_t launch_mode(int mode, const RhsArgs& a, int grid, cudaStream_t s) {
  switch (mode) {
    case MODE_RHS: return launch_impl<N, EQ, Real, MODE_RHS>(a, grid, s);
    case MODE_STAGE: return launch_impl<N, EQ, Real, MODE_STAGE>(a, grid, s);
    default: break;
  }
  if constexpr (std::is_same<Real, double>::value) {
    switch (mode) {
      case MODE_SPLIT: return launch_impl<N, EQ, Real, MODE_SPLIT>(a, grid, s);
      case MODE_SPLIT | MODE_STAGE:
        return launch_impl<N, EQ, Real, MODE_SPLIT | MODE_STAGE>(a, grid, s);
      default: break;
    }
  } else {
    constexpr int T1 = MODE_TC | MODE_B128, T5 = MODE_TC | MODE_B512;
    switch (mode) {
      case MODE_TC: return launch_impl<N, EQ, Real, MODE_TC>(a, grid, s);
      case MODE_TC | MODE_STAGE:
        return launch_impl<N, EQ, Real, MODE_TC | MODE_STAGE>(a, grid, s);
      case T1: return launch_impl<N, EQ, Real, T1>(a, grid, s);
      case T1 | MODE_STAGE: return launch_impl<N, EQ, Real, T1 | MODE_STAGE>(a, grid, s);
      case T5: return launch_impl<N, EQ, Real, T5>(a, grid, s);
      case T5 | MODE_STAGE: return launch_impl<N, EQ, Real, T5 | MODE_STAGE>(a, grid, s);
      default: break;
    }
  }
  return cudaErrorInvalidValue;
}

template <int N, int EQ>
cudaError_t shape_n(int precision, int mode, LaunchShape* out) {
  return precision == 0 ? shape_mode<N, EQ, double>(mode, out)
                        : shape_mode<N, EQ, float>(mode, out);
}

template <int N, int EQ>
cudaError_t launch_n(int precision, int mode, const RhsArgs& a, int grid,
                     cudaStream_t s) {
  return precision == 0 ? launch_mode<N, EQ, double>(mode, a, grid, s)
                        : launch_mode<N, EQ, float>(mode, a, grid, s);
}

template <int EQ>
cudaError_t shape_any(int order, int precision, int mode, LaunchShape* out) {
  if ((precision != 0 && precision != 1) || mode < 0 || mode > 31)
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
  if ((precision != 0 && precision != 1) || mode < 0 || mode > 31)
    return cudaErrorInvalidValue;
  switch (order) {
    case 1: return launch_n<1, EQ>(precision, mode, a, grid, s);
    case 2: return launch_n<2, EQ>(precision, mode, a, grid, s);
    case 3: return launch_n<3, EQ>(precision, mode, a, grid, s);
    case 4: return launch_n<4, EQ>(precision, mode, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

// {{{ face-shared path: the face kernel (and, for Euler, the per-node table)

template <int N, int EQ>
cudaError_t face_blocks_n(int* blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      blocks_per_sm, dg_face_flux_kernel<N, EQ>, kFaceBlock, 0);
}

template <int EQ>
cudaError_t face_blocks_any(int order, int* blocks_per_sm) {
  switch (order) {
    case 1: return face_blocks_n<1, EQ>(blocks_per_sm);
    case 2: return face_blocks_n<2, EQ>(blocks_per_sm);
    case 3: return face_blocks_n<3, EQ>(blocks_per_sm);
    case 4: return face_blocks_n<4, EQ>(blocks_per_sm);
    default: return cudaErrorInvalidValue;
  }
}

template <int EQ>
cudaError_t face_launch_any(int order, const FaceArgs& a, int grid, int aux_grid,
                            cudaStream_t s) {
  if constexpr (EQ == DG_EULER) {
    dg_euler_aux_kernel<EQ><<<aux_grid, kFaceBlock, 0, s>>>(
        a.q, const_cast<double*>(a.aux),
        (uint32_t)(a.nel * ((order + 1) * (order + 2) * (order + 3) / 6)), a.p0);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  switch (order) {
    case 1: dg_face_flux_kernel<1, EQ><<<grid, kFaceBlock, 0, s>>>(a); break;
    case 2: dg_face_flux_kernel<2, EQ><<<grid, kFaceBlock, 0, s>>>(a); break;
    case 3: dg_face_flux_kernel<3, EQ><<<grid, kFaceBlock, 0, s>>>(a); break;
    case 4: dg_face_flux_kernel<4, EQ><<<grid, kFaceBlock, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// }}}

// {{{ FP64 with tensor-core contractions (face-shared path only)

template <int N, int EQ, int MODE>
cudaError_t tc_shape_impl(LaunchShape* out) {
  using P = tc::Plan<N, EQ>;
  auto kern = dg_rhs_tc_kernel<N, EQ, MODE>;
  cudaError_t err = cudaFuncSetAttribute(
      kern, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM_BYTES);
  if (err != cudaSuccess) return err;
  int nb = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, tc::kTcBlock, P::SMEM_BYTES);
  out->smem_bytes = P::SMEM_BYTES;
  out->blocks_per_sm = nb;
  out->elems_per_tile = P::E;
  out->ops_bytes = P::OPS_BYTES;
  out->threads = tc::kTcBlock;
  return err;
}

template <int N, int EQ>
cudaError_t tc_shape_n(int mode, LaunchShape* out) {
  return mode == 0 ? tc_shape_impl<N, EQ, MODE_SPLIT>(out)
                   : tc_shape_impl<N, EQ, MODE_SPLIT | MODE_STAGE>(out);
}

template <int N, int EQ>
cudaError_t tc_launch_n(int mode, const RhsArgs& a, int grid, cudaStream_t s) {
  using P = tc::Plan<N, EQ>;
  if (mode == 0)
    dg_rhs_tc_kernel<N, EQ, MODE_SPLIT><<<grid, tc::kTcBlock, P::SMEM_BYTES, s>>>(a);
  else
    dg_rhs_tc_kernel<N, EQ, MODE_SPLIT | MODE_STAGE><<<grid, tc::kTcBlock, P::SMEM_BYTES, s>>>(a);
  return cudaGetLastError();
}

// orders 3 and 4 only (the tensor-core products need the work of high orders)
template <int EQ>
cudaError_t tc_shape_any(int order, int mode, LaunchShape* out) {
  if (mode != 0 && mode != 1) return cudaErrorInvalidValue;
  switch (order) {
    case 3: return tc_shape_n<3, EQ>(mode, out);
    case 4: return tc_shape_n<4, EQ>(mode, out);
    default: return cudaErrorInvalidValue;
  }
}

template <int EQ>
cudaError_t tc_launch_any(int order, int mode, const RhsArgs& a, int grid,
                          cudaStream_t s) {
  if (mode != 0 && mode != 1) return cudaErrorInvalidValue;
  switch (order) {
    case 3: return tc_launch_n<3, EQ>(mode, a, grid, s);
    case 4: return tc_launch_n<4, EQ>(mode, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

// }}}


// {{{ mixed precision with tcgen05 contractions (fused face fluxes)

template <int N, int EQ, int MODE, bool TF, bool ALT = false>
cudaError_t tcm_shape_impl(LaunchShape* out) {
  using P = tcm::MPlan<N, EQ, TF, ALT>;
  auto kern = dg_rhs_tcm_kernel<N, EQ, MODE, TF, ALT>;
  cudaError_t err = cudaFuncSetAttribute(
      kern, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM_BYTES);
  if (err != cudaSuccess) return err;
  // resident CTAs per SM from the kernel's registers and shared memory (the
  // occupancy query reports one CTA for kernels that allocate tensor
  // memory), capped by the SM's 512 tensor-memory columns
  cudaFuncAttributes fa;
  err = cudaFuncGetAttributes(&fa, kern);
  if (err != cudaSuccess) return err;
  int dev = 0, regs_sm = 0, smem_sm = 0, smem_rsv = 0, thr_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  const int warps = P::THREADS / 32;
  const int regs_warp = ((fa.numRegs * 32 + 255) / 256) * 256;  // 256-register units
  int nb = regs_sm / (regs_warp * warps);
  const int smem_blk = P::SMEM_BYTES + (int)fa.sharedSizeBytes + smem_rsv;
  if (smem_sm / smem_blk < nb) nb = smem_sm / smem_blk;
  if (thr_sm / P::THREADS < nb) nb = thr_sm / P::THREADS;
  if (nb > 512 / P::TMEM_COLS) nb = 512 / P::TMEM_COLS;
  out->smem_bytes = P::SMEM_BYTES;
  out->blocks_per_sm = nb;
  out->elems_per_tile = P::E;
  out->ops_bytes = P::OPS_BYTES;
  out->threads = P::THREADS;
  return err;
}

// mode bit 0: fused RK stage; bit 1: 3xTF32 products instead of exact
// digits; bit 2 (3xTF32 only): the other CTA size (MPlan::ALT)
constexpr bool tcm_mode_ok(int mode) { return mode >= 0 && mode <= 7 && (mode < 4 || (mode & 2)); }

template <int N, int EQ>
cudaError_t tcm_shape_n(int mode, LaunchShape* out) {
  switch (mode) {
    case 0: return tcm_shape_impl<N, EQ, MODE_RHS, false>(out);
    case 1: return tcm_shape_impl<N, EQ, MODE_STAGE, false>(out);
    case 2: return tcm_shape_impl<N, EQ, MODE_RHS, true>(out);
    case 3: return tcm_shape_impl<N, EQ, MODE_STAGE, true>(out);
    case 6: return tcm_shape_impl<N, EQ, MODE_RHS, true, true>(out);
    default: return tcm_shape_impl<N, EQ, MODE_STAGE, true, true>(out);
  }
}

template <int N, int EQ, int MODE, bool TF, bool ALT = false>
cudaError_t tcm_launch_impl(const RhsArgs& a, int grid, cudaStream_t s) {
  using P = tcm::MPlan<N, EQ, TF, ALT>;
  dg_rhs_tcm_kernel<N, EQ, MODE, TF, ALT><<<grid, P::THREADS, P::SMEM_BYTES, s>>>(a);
  return cudaGetLastError();
}

template <int N, int EQ>
cudaError_t tcm_launch_n(int mode, const RhsArgs& a, int grid, cudaStream_t s) {
  switch (mode) {
    case 0: return tcm_launch_impl<N, EQ, MODE_RHS, false>(a, grid, s);
    case 1: return tcm_launch_impl<N, EQ, MODE_STAGE, false>(a, grid, s);
    case 2: return tcm_launch_impl<N, EQ, MODE_RHS, true>(a, grid, s);
    case 3: return tcm_launch_impl<N, EQ, MODE_STAGE, true>(a, grid, s);
    case 6: return tcm_launch_impl<N, EQ, MODE_RHS, true, true>(a, grid, s);
    default: return tcm_launch_impl<N, EQ, MODE_STAGE, true, true>(a, grid, s);
  }
}

template <int EQ>
cudaError_t tcm_shape_any(int order, int mode, LaunchShape* out) {
  if (!tcm_mode_ok(mode)) return cudaErrorInvalidValue;
  switch (order) {
    case 1: return tcm_shape_n<1, EQ>(mode, out);
    case 2: return tcm_shape_n<2, EQ>(mode, out);
    case 3: return tcm_shape_n<3, EQ>(mode, out);
    case 4: return tcm_shape_n<4, EQ>(mode, out);
    default: return cudaErrorInvalidValue;
  }
}

template <int EQ>
cudaError_t tcm_launch_any(int order, int mode, const RhsArgs& a, int grid,
                           cudaStream_t s) {
  if (!tcm_mode_ok(mode)) return cudaErrorInvalidValue;
  switch (order) {
    case 1: return tcm_launch_n<1, EQ>(mode, a, grid, s);
    case 2: return tcm_launch_n<2, EQ>(mode, a, grid, s);
    case 3: return tcm_launch_n<3, EQ>(mode, a, grid, s);
    case 4: return tcm_launch_n<4, EQ>(mode, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

// }}}

}  // namespace
}  // namespace dg
