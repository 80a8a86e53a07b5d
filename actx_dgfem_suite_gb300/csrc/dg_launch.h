// Host-side launch interface between the C ABI (abi.cu) and the per-equation
// kernel translation units (rhs_wave.cu, rhs_euler.cu, rhs_maxwell.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace dg {

struct RhsArgs;

struct LaunchShape {
  int smem_bytes = 0;      // dynamic shared memory per CTA
  int blocks_per_sm = 0;   // resident CTAs per SM at that footprint
  int elems_per_tile = 0;  // elements per CTA tile
  int ops_doubles = 0;     // size of the staged operator block
};

// Layout of the operator block (in doubles), shared by host packing and the
// kernels' OpsLayout<N>: [Wt (3 Np Np) | Lt (4 Nfp Np) | int32 face_nodes].
struct OpsOffsets {
  int w, l, fn, size;
};
inline int pad2_host(int n) { return (n + 1) & ~1; }
inline OpsOffsets ops_offsets(int np, int nfp) {
  OpsOffsets o;
  o.w = 0;
  o.l = o.w + pad2_host(3 * np * np);
  o.fn = o.l + pad2_host(4 * nfp * np);
  o.size = o.fn + pad2_host((4 * nfp + 1) / 2);
  return o;
}

// Per equation: shape query (also raises the kernel's shared-memory limit on
// the current device) and launch.  Return cudaErrorInvalidValue for an order
// that is not compiled in.
cudaError_t fp64_shape_wave(int order, LaunchShape* out);
cudaError_t fp64_shape_euler(int order, LaunchShape* out);
cudaError_t fp64_shape_maxwell(int order, LaunchShape* out);
cudaError_t fp64_launch_wave(int order, const RhsArgs& a, int grid,
                             cudaStream_t s);
cudaError_t fp64_launch_euler(int order, const RhsArgs& a, int grid,
                              cudaStream_t s);
cudaError_t fp64_launch_maxwell(int order, const RhsArgs& a, int grid,
                                cudaStream_t s);

}  // namespace dg
