// Shared device helpers for the sm_103a DG-FEM kernels: TMA bulk copies into
// shared memory completed on an mbarrier, and bounded waits that report a
// timeout through a device status word instead of spinning forever.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/dgfem_gb300.h"

namespace dg {

constexpr int kBlock = 256;                        // threads per CTA
constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar,
                                                      uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

// 1D TMA bulk copy global -> shared; dst/src 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for phase `parity` of `bar` for at most kWaitLimitNs; false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar,
                                                  uint32_t parity) {
  const unsigned long long t0 = global_ns();
  for (uint32_t it = 0; it < (1u << 30); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u && global_ns() - t0 > kWaitLimitNs) return false;
  }
  return false;
}

__device__ __forceinline__ void raise_status(int* status, int code) {
  if (status) atomicMax(status, code);
}

// FP64 <-> FP32 conversions done with integer ALU instructions.  On GB300 the
// FP64 pipe issues a small fraction of the FP32/INT rate, and conversion
// instructions that touch FP64 compete for it; in the mixed-precision kernels
// the state is converted once per load, so these bit manipulations keep that
// traffic off the FP64 pipe.  Round to nearest even; results below the
// smallest normal float flush to zero, values beyond the float range become
// infinity (the DG states are O(1)).
__device__ __forceinline__ float d2f_alu(double x) {
  const uint32_t lo = (uint32_t)__double2loint(x);
  const uint32_t hi = (uint32_t)__double2hiint(x);
  const uint32_t sign = hi & 0x80000000u;
  const int32_t e = (int32_t)((hi >> 20) & 0x7ffu) - 896;  // float biased exponent
  const uint32_t mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const uint32_t rest = lo & 0x1fffffffu;
  uint32_t bits = ((uint32_t)e << 23) + mant;
  bits += (uint32_t)((rest > 0x10000000u) | ((rest == 0x10000000u) & (mant & 1u)));
  bits = e <= 0 ? 0u : bits;
  bits = e >= 255 ? 0x7f800000u : bits;
  return __uint_as_float(sign | bits);
}

__device__ __forceinline__ double f2d_alu(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t sign = b & 0x80000000u;
  const uint32_t e = (b >> 23) & 0xffu;
  const uint32_t m = b & 0x7fffffu;
  uint32_t hi = sign | ((e + 896u) << 20) | (m >> 3);
  uint32_t lo = m << 29;
  hi = e == 0u ? sign : hi;
  lo = e == 0u ? 0u : lo;
  hi = e == 255u ? (sign | 0x7ff00000u | (m >> 3)) : hi;
  return __hiloint2double((int)hi, (int)lo);
}

}  // namespace dg
