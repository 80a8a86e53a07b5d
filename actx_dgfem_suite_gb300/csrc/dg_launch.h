// Host-side launch interface between the C ABI (abi.cu) and the per-equation
// kernel translation units (rhs_wave.cu, rhs_euler.cu, rhs_maxwell.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace dg {

struct RhsArgs;
struct AdjArgs;
struct FaceArgs;
struct VjpArgs;

struct LaunchShape {
  int smem_bytes = 0;      // dynamic shared memory per CTA
  int blocks_per_sm = 0;   // resident CTAs per SM at that footprint
  int elems_per_tile = 0;  // elements per CTA tile
  int ops_bytes = 0;       // size of the staged operator block
  int threads = 256;       // threads per CTA
};

// Byte layout of the operator block, shared by host packing and the kernels'
// OpsLayout<N, Real>: [Wt (3 Np Np) | Lt (4 Nfp Np) | int32 face_nodes],
// each segment padded to 16 bytes; `rs` = sizeof(Real).
struct OpsOffsets {
  int w, l, fn, size;
};
inline int pad16_host(int n) { return (n + 15) & ~15; }
// same rule as the kernels' odd4(): multiple of 4 with an odd quotient
inline int pitch_host(int n) {
  const int m = (n + 3) & ~3;
  return (m / 4) % 2 == 0 ? m + 4 : m;
}
// rs = 8: FP64 layout Wt[r][j][i], Lt[fj][i]; rs = 4: mixed layout
// W[r][i][j] with pitch pitch_host(np), L[i][fj] with pitch pitch_host(4 nfp)
inline OpsOffsets ops_offsets(int np, int nfp, int rs) {
  OpsOffsets o;
  const bool mixed = rs == 4;
  o.w = 0;
  o.l = o.w + pad16_host((mixed ? 3 * np * pitch_host(np) : 3 * np * np) * rs);
  o.fn = o.l + pad16_host((mixed ? np * pitch_host(4 * nfp) : 4 * nfp * np) * rs);
  o.size = o.fn + pad16_host(4 * nfp * 4);
  return o;
}

// Per equation: shape query (also raises the kernel's shared-memory limit on
// the current device) and launch, for precision 0 (FP64) or 1 (FP32
// arithmetic, FP64 state) and mode bits MODE_STAGE (fused RK stage) and
// MODE_SPLIT (face values from the face-shared kernels, FP64 only).  Return
// cudaErrorInvalidValue for a combination that is not compiled in.
// face_blocks_*: resident CTAs per SM of the face kernel; face_launch_*:
// (Euler: the per-node table, then) the face kernel of the face-shared path.
// tc_shape_* / tc_launch_*: the face-shared volume/LIFT kernel with the
// contractions on the tensor cores (mode 0 RHS, 1 RK stage).
// tcm_shape_* / tcm_launch_*: the mixed-precision kernel with its
// contractions on tcgen05 (mode bit 0: RK stage; bit 1: 3xTF32 products,
// else exact digit-pair products; bit 2, with bit 1: the other CTA size).
#define DG_DECLARE_EQ(name)                                                   \
  cudaError_t shape_##name(int order, int precision, int mode,               \
                           LaunchShape* out);                                \
  cudaError_t launch_##name(int order, int precision, int mode,              \
                            const RhsArgs& a, int grid, cudaStream_t s);     \
  cudaError_t face_blocks_##name(int order, int* blocks_per_sm);             \
  cudaError_t face_launch_##name(int order, const FaceArgs& a, int grid,     \
                                 int aux_grid, cudaStream_t s);              \
  cudaError_t tc_shape_##name(int order, int mode, LaunchShape* out);        \
  cudaError_t tc_launch_##name(int order, int mode, const RhsArgs& a,        \
                               int grid, cudaStream_t s);                    \
  cudaError_t tcm_shape_##name(int order, int mode, LaunchShape* out);       \
  cudaError_t tcm_launch_##name(int order, int mode, const RhsArgs& a,       \
                                int grid, cudaStream_t s);
DG_DECLARE_EQ(wave)
DG_DECLARE_EQ(euler)
DG_DECLARE_EQ(maxwell)
#undef DG_DECLARE_EQ

// Operator block of the tensor-core kernel (layout of tc::Plan<N, EQ> in
// dg_tc.cuh): the volume product [A_0; A_1; A_2] (3 Np x Np, wave and
// maxwell) or [A_0 A_1 A_2] (Np x 3 Np, euler), then LIFT (Np x 4 Nfp).
// Each: 7 FP16 digit slices in the K-major no-swizzle layout of the tcgen05
// descriptors, then one int32 exponent per padded row; blocks padded to 16
// bytes.  Returns the block size (out == NULL: size only).
int pack_tc_ops(int eq, int order, const double* diff, const double* lift,
                unsigned char* out, int out_bytes);

// Operator block of the mixed tcgen05 kernel (tcm::MPlan<N, EQ, tf32> in
// dg_tcm.cuh): [A_0 A_1 A_2] (Np x 3 Np) and LIFT (Np x 4 Nfp) in the K-major
// no-swizzle layout of the tcgen05 descriptors; digits (tf32 false): each
// row scaled to 31-bit integers written as four FP16 digit slices, then the
// FP32 row scales 2^e of each; tf32: two slices, x = hi + lo in TF32.  Then
// the int32 face node table.  Returns the block size (out == NULL: size only).
int pack_tcm_ops(int order, const double* diff, const double* lift,
                 const int32_t* face_nodes, unsigned char* out, int out_bytes,
                 bool tf32);

// Triangle meshes (rhs_2d.cu): shape query and launch of dg_rhs2d_kernel
// for mode MODE_RHS or MODE_STAGE (FP64), and the operator block
// [Wt (2 Np Np) | Lt (3 Nfp Np) | int32 edge nodes (3 Nfp)] packed from the
// host arrays diff (2, Np, Np), lift (Np, 3, Nfp), face_nodes (3, Nfp);
// returns the block size (out == NULL: size only; -1 if out_bytes is short).
cudaError_t shape_2d(int eq, int order, int mode, LaunchShape* out);
cudaError_t launch_2d(int eq, int order, int mode, const RhsArgs& a, int grid,
                      cudaStream_t s);
int pack_ops_2d(int order, const double* diff, const double* lift,
                const int32_t* face_nodes, unsigned char* out, int out_bytes);

// Record `msg` as the calling thread's last error (dg_last_error) and
// return `code`; shared by the translation units behind the C ABI.
int set_error(int code, const char* msg);

// Adjoint of the FP64 wave RHS: shape of the volume kernel, and the two
// launches (volume transpose + lifted face adjoints, then the per-node
// transposed flux/gather); `nsm` caps the second grid.
cudaError_t adjoint_shape_wave(int order, LaunchShape* out);
cudaError_t adjoint_launch_wave(int order, const AdjArgs& a, int grid, int nsm,
                                cudaStream_t s);
// The same two launches as one fused reverse LSRK stage (AdjArgs' stage
// fields: lam += dt L^T rbar, next rbar, c-gradient inner products).
cudaError_t adjoint_stage_launch_wave(int order, const AdjArgs& a, int grid, int nsm,
                                      cudaStream_t s);

// Mixed-precision Euler: the per-node pressure table (FP64 recovery from
// total energy, stored as FP32) that the mixed kernels read; one launch
// before each mixed Euler RHS or RK stage.
cudaError_t pressure_launch_euler(const double* q, float* pres, int64_t nelnp,
                                  double gamma, int grid, cudaStream_t s);

// Transposed Jacobian of the FP64 Euler RHS (dg_adjoint_euler.cuh): shape of
// the volume kernel, and the launches (node table, volume, face, node gather;
// with stage, the gather applies the reverse LSRK stage update instead of
// storing y).
cudaError_t vjp_shape_euler(int order, LaunchShape* out);
cudaError_t vjp_launch_euler(int order, const VjpArgs& a, int grid, int nsm, bool stage,
                             cudaStream_t s);

}  // namespace dg
