// FP64 RHS with the contractions on the tensor cores: exact FP64 emulation
// by FP16 digit slices (error-free splitting in the manner of Ozaki et al.,
// "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applicability", Numer.
// Algorithms 59, 2012), issued as tcgen05 products with accumulators in
// tensor memory.
//
// GB300 issues FP64 at about 1.25 TFLOP/s but FP16 tensor-core products at
// petaflop rates, and the high-order DG contractions (volume derivatives,
// LIFT) keep the FP64 pipe ~97 % busy.  Here every contraction C = A X
// (A: a reference operator, M x K; X: K x NC columns of FP64 data, one column
// per element and field) is evaluated as
//
//   A = 2^(e_m - 54) A_int,  X = 2^(e_n - 54) X_int   (per-row / per-column
//   exponents, 54-bit integers), each integer written as 7 balanced base-256
//   digits d_1..d_7 in [-128, 127] (exact in FP16);
//   v_l = sum_{i + j = l} D^A_i D^X_j    for l = 2..8: one tcgen05.mma
//   (kind::f16, M = 128, K = 16, FP32 accumulation in tensor memory) per
//   digit pair and k-step (28 pairs), all pairs of a level accumulating into
//   that level's tensor-memory columns -- exactly, because
//   |v_l| <= 7 K 128^2 < 2^24 for K <= 146;
//   C = 2^(e_m + e_n - 60) (G_hi 2^32 + G_lo),  G_hi = sum_{l<=4} v_l 2^(8(4-l)),
//   G_lo = sum_{l>=5} v_l 2^(8(8-l)) in 64-bit integers (exact), read out of
//   tensor memory with tcgen05.ld.
//
// Error: the 54-bit rounding of the inputs (2^-55 of the row or column
// maximum) and the dropped digit pairs (l > 8, below ~2^-51 K max_k |A_mk|
// max_k |X_kn|) -- the order of FP64's own accumulation error.  Splitting
// and recombination are integer work (no FP64 pipe): the level sums are
// folded by 64-bit Horner sums and converted to FP64 with round-to-nearest-
// even built from the bits.
//
// One thread issues all products of a contraction (asynchronous, completion
// signalled on an mbarrier through tcgen05.commit; the wait is bounded);
// operands come from shared memory through matrix descriptors (K-major, no
// swizzle: 8-row x 16-byte core matrices, k-chunks 128 bytes apart, 8-row
// groups SBO bytes apart).  The CTA allocates tensor memory once (8 levels x
// the padded column count, at most 512 columns) and frees it before it exits.
//
// The kernel is the volume/LIFT half of the face-shared path: face values
// come from dg_face_flux_kernel (and, for Euler, pressure and 1/rho from
// dg_euler_aux_kernel), pointwise work (Euler fluxes, metric terms, curl,
// RK epilogue) stays in FP64.  One 512-thread CTA per SM (the order-4
// operator digits take 109 KB of shared memory); where shared memory allows
// a second input buffer (order 3; wave and Euler at order 4) the next tile's
// inputs arrive by 1D TMA bulk copies into it while the current tile
// computes.  Orders 3 and 4 (lower orders have too little contraction work
// for the digit splitting to pay).
#pragma once

#include <cuda_fp16.h>

#include <type_traits>

#include "dg_face.cuh"
#include "dg_ledger.h"
#include "dg_rhs.cuh"

namespace dg {
namespace tc {

constexpr int kS = 7;        // digits per value (balanced, base 256)
constexpr int kFix = 54;     // fixed-point bits (7 balanced base-256 digits hold |x| < 2^54.99)
constexpr int kLevels = 8;   // digit pairs with i + j <= kLevels are kept
constexpr int kTcBlock = 512;  // threads per CTA (one CTA per SM)
static_assert(kLevels == 8 && kS == 7, "the split and recombination are base 256, levels 2..8");

constexpr int r16(int x) { return (x + 15) & ~15; }
constexpr int r8(int x) { return (x + 7) & ~7; }
constexpr int p16(int bytes) { return (bytes + 15) & ~15; }

// One emulated product: operator A (M x K) times NC data columns of length K.
//   operator block (global and shared): 7 FP16 digit slices of A in the
//   K-major canonical layout (element (m, k) at (m/8) SBO_A + (k/8) 128 +
//   (m%8) 16 + (k%8) 2 bytes, SBO_A = KP/8 x 128; rows padded to a multiple of
//   8), then one int32 exponent per padded row;
//   data slices (shared): the same layout for the NPAD (>= NC) data columns.
// The products read 128 operator rows from each slice: rows past the padded
// M belong to the next slice or region and only feed output rows that are
// never read.
template <int M_, int K_, int NC_>
struct Gemm {
  static constexpr int M = M_, K = K_, NC = NC_;
  static constexpr int MR8 = r8(M), KP = r16(K), KC = KP / 8, KT = KP / 16;
  static constexpr int NPAD = r16(NC);
  static constexpr int SBO = KC * 128;
  static constexpr int A_SLICE = (MR8 / 8) * SBO;
  static constexpr int DIGITS = kS * A_SLICE;
  static constexpr int OPS_BYTES = p16(DIGITS + MR8 * 4);
  static constexpr int A_READ = 16 * SBO;             // bytes a product reads per slice
  static constexpr int B_SLICE = (NPAD / 8) * SBO;
  static constexpr int SLICE_BYTES = kS * B_SLICE;
  static constexpr int TMEM_COLS = (kLevels - 1) * NPAD;
  // instruction descriptor: D FP32, A and B FP16, both K-major, N, M = 128
  static constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(NPAD >> 3) << 17) | (8u << 24);
  static_assert(M <= 128, "one 128-row product per contraction");
  static_assert(K <= 146, "exact FP32 level sums need 7 K 128^2 < 2^24");
  static_assert(TMEM_COLS <= 512, "levels x columns must fit in tensor memory");
};

// Elements per CTA tile: at most 64 data columns per contraction so the 8
// level accumulators fit the 512 tensor-memory columns, filling the columns
// the products pad to 16 anyway (wave 4 E, euler and maxwell NF E), within
// the shared memory left beside the FP16 operator digits at order 4.
constexpr int tile_elems(int N, int EQ) {
  return N == 3 ? (EQ == DG_MAXWELL ? 10 : (EQ == DG_EULER ? 12 : 16))
                : (EQ == DG_EULER ? 6 : (EQ == DG_MAXWELL ? 7 : 8));
}

constexpr int pow2_cols(int c) {
  return c <= 32 ? 32 : c <= 64 ? 64 : c <= 128 ? 128 : c <= 256 ? 256 : 512;
}

// Products of one equation at order N (3 or 4).  GV, the volume product:
//   wave, maxwell: stacked rows [A_0; A_1; A_2] (3 Np x Np) applied to
//     columns (field f, element e) at n = f E + e -- maxwell the six fields,
//     wave u and the three metric-combined velocity components (of whose
//     products only the diagonal blocks are used);
//   euler: concatenated columns [A_0 A_1 A_2] (Np x 3 Np) applied to the
//     metric-combined fluxes of each (field, element);
// GL: LIFT (Np x 4 Nfp) applied to the face values of each (field, element).
template <int N, int EQ>
struct Plan {
  static_assert(N >= 3, "tensor-core products are built for orders 3 and 4");
  static constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP, NFPT = Shape<N>::NFPT;
  static constexpr int NF = EqInfo<EQ>::NF;
  static constexpr int E = tile_elems(N, EQ);
  static constexpr bool STACKED = EQ != DG_EULER;
  using GV = typename std::conditional<
      STACKED, Gemm<3 * NP, NP, (EQ == DG_WAVE ? 4 : NF) * E>,
      Gemm<NP, 3 * NP, NF * E>>::type;
  using GL = Gemm<NP, NFPT, NF * E>;
  static constexpr int OPS_GV = 0;
  static constexpr int OPS_GL = GV::OPS_BYTES;
  static constexpr int OPS_BYTES = OPS_GL + GL::OPS_BYTES;

  static constexpr int NAUX = EQ == DG_WAVE ? 3 : (EQ == DG_EULER ? 15 : 0);
  static constexpr int cmax(int x, int y) { return x > y ? x : y; }
  static constexpr int R1_BYTES = p16(cmax(GV::SLICE_BYTES, GL::SLICE_BYTES));
  static constexpr int R2_BYTES = p16(8 * cmax(cmax(NAUX * E * NP, GV::M * GV::NC),
                                               NF * E * NFPT + GL::M * GL::NC));
  static constexpr int NCOLS = cmax(GV::NPAD, GL::NPAD);
  static constexpr int TMEM_ALLOC = pow2_cols(cmax(GV::TMEM_COLS, GL::TMEM_COLS));
  // a tile's inputs: state, face values, metric (FP64)
  static constexpr int IN_Q = p16(NF * E * NP * 8), IN_F = p16(NF * E * NFPT * 8);
  static constexpr int IN_G = p16(9 * E * 8);
  static constexpr int IN_BYTES = IN_Q + IN_F + IN_G;
  // where shared memory allows (order 3), two input buffers: the next tile's
  // inputs arrive by TMA bulk copies while the current tile computes
  static constexpr bool PREFETCH =
      p16(OPS_BYTES) + R1_BYTES + R2_BYTES + p16(NCOLS * 4) + 2 * IN_BYTES <= 227 * 1024;
  // shared memory: ops | state (FP64) | R1 (slices) | R2 (FP64 scratch) |
  // metric | column exponents | (PREFETCH: two input buffers, which then
  // hold the state and metric)
  static constexpr int SM_OPS = 0;
  static constexpr int SM_Q = p16(OPS_BYTES);
  static constexpr int SM_R1 = SM_Q + (PREFETCH ? 0 : IN_Q);
  static constexpr int SM_R2 = SM_R1 + R1_BYTES;
  static constexpr int SM_GEO = SM_R2 + R2_BYTES;
  static constexpr int SM_EXP = SM_GEO + (PREFETCH ? 0 : IN_G);
  static constexpr int SM_IN = SM_EXP + p16(NCOLS * 4);
  static constexpr int SMEM_USED = SM_IN + (PREFETCH ? 2 * IN_BYTES : 0);
  static_assert(!PREFETCH || (E * NP) % 2 == 0, "bulk-copy destinations 16-byte aligned");
  // a CTA that takes all 512 tensor-memory columns must be alone on its SM
  static constexpr int SMEM_BYTES =
      TMEM_ALLOC == 512 && SMEM_USED < 120 * 1024 ? 120 * 1024 : SMEM_USED;
  static_assert(SMEM_BYTES <= 227 * 1024, "tile does not fit in shared memory");
  // every product's reads of 128 operator rows / NPAD data rows stay in the CTA
  static_assert(OPS_GV + 7 * GV::A_SLICE + GV::A_READ <= SMEM_BYTES, "GV operand reads");
  static_assert(OPS_GL + 7 * GL::A_SLICE + GL::A_READ <= SMEM_BYTES, "GL operand reads");
};

// {{{ device helpers

// {{{ tcgen05 helpers

// shared-memory matrix descriptor: start address, leading (k-chunk) and
// stride (8-row group) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3fff) | ((uint64_t)((lbo >> 4) & 0x3fff) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3fff) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b,
                                       uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
      ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// arrive on `bar` once every tcgen05 operation this thread issued has completed
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
      ::"r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_ld8(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tc_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// shared-memory stores of this thread become visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// }}}

// two digits in [-128, 128] -> half2: the bit pattern 0x6600 + d is the half
// 1536 + d, and one HSUB2 removes the 1536 exactly (bits move through the
// __ushort_as_half / __half_as_ushort intrinsics, not pointer punning)
__device__ __forceinline__ uint32_t digits_to_half2(int d0, int d1) {
  const __half2 h = __halves2half2(__ushort_as_half((unsigned short)(0x6600 + d0)),
                                   __ushort_as_half((unsigned short)(0x6600 + d1)));
  const __half2 c = __halves2half2(__ushort_as_half((unsigned short)0x6600u),
                                   __ushort_as_half((unsigned short)0x6600u));
  const __half2 d = __hsub2(h, c);
  return (uint32_t)__half_as_ushort(__low2half(d)) |
         ((uint32_t)__half_as_ushort(__high2half(d)) << 16);
}


// FP32 holding an exact integer |v| < 2^22 -> int32 (FADD + IADD, no conversion unit)
__device__ __forceinline__ int32_t f32_exact_int(float v) {
  return __float_as_int(__fadd_rn(v, 12582912.0f)) - 0x4B400000;
}

// FP32 holding an exact integer |v| < 2^24 -> int32 without a conversion
// instruction (GB300's conversion unit issues at a fraction of the FP32
// rate): the FADD at 1.5 * 2^31, where the float spacing is 256, rounds v to
// hi = 256 round(v / 256), read off the sum's mantissa bits; lo = v - hi is
// exact (|lo| <= 128) and read off the bits of lo + 1.5 * 2^23
__device__ __forceinline__ int32_t f32_exact_int24(float v) {
  const float kBig = 3221225472.0f;  // 1.5 * 2^31
  const float big = __fadd_rn(v, kBig);
  const float lo = __fsub_rn(v, __fsub_rn(big, kBig));
  return (__float_as_int(big) - __float_as_int(kBig)) * 256 +
         (__float_as_int(__fadd_rn(lo, 12582912.0f)) - 0x4B400000);
}

// int64 |g| < 2^51 -> double, exactly (integer add + one DADD)
__device__ __forceinline__ double i64_exact_double(long long g) {
  return __longlong_as_double(g + 0x4338000000000000LL) - 6755399441055744.0;
}

// 2^e as a double, e clamped to the normal range
__device__ __forceinline__ double pow2(int e) {
  e = e < -1022 ? -1022 : (e > 1023 ? 1023 : e);
  return __longlong_as_double((long long)(e + 1023) << 52);
}

// RN(W) 2^s with W = T 2^28 + f (T: int64, |T| < 2^46; f in [0, 2^28)), built
// from integer operations only (GB300 issues FP64 at 1/64 of the integer
// rate).  Magnitude M = A 2^28 + B; M < 2^64 is normalised directly, larger
// M keeps its top 64 bits with the dropped bits jammed into a sticky bit
// (then M >= 2^54, so the sticky bit sits below the rounding bit).  Round to
// nearest, ties to even; the carry of a round-up moves into the exponent.
// Returns false (out untouched) when the result is not a normal double.
__device__ __forceinline__ bool fixed_to_double(long long T, unsigned f, int s, double* out) {
  const bool neg = T < 0;
  unsigned long long A = (unsigned long long)(neg ? -T - (f != 0u) : T);
  const unsigned B = neg && f != 0u ? (1u << 28) - f : f;
  unsigned long long Z;
  int zexp;
  if (A < (1ull << 36)) {
    Z = (A << 28) | B;
    zexp = 0;
  } else {
    Z = (A << 18) | (B >> 10) | (unsigned long long)((B & 1023u) != 0u);
    zexp = 10;
  }
  if (Z == 0) {
    *out = 0.0;
    return true;
  }
  const int n = 63 - __clzll((long long)Z);
  const int eb = n + zexp + s + 1023;
  if (eb < 1 || eb > 2045) return false;
  unsigned long long mant, up = 0;
  if (n <= 52) {
    mant = Z << (52 - n);
  } else {
    const int sh = n - 52;
    mant = Z >> sh;
    const unsigned long long rem = Z & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    up = (rem > half || (rem == half && (mant & 1ull))) ? 1ull : 0ull;
  }
  const unsigned long long bits = ((unsigned long long)eb << 52) + (mant - (1ull << 52)) + up;
  *out = __longlong_as_double((long long)(bits | ((unsigned long long)neg << 63)));
  return true;
}

// biased exponent field of a double (0 for zero and subnormals)
__device__ __forceinline__ int dexp(double x) {
  return (__double2hiint(x) >> 20) & 0x7ff;
}

// x -> round(x 2^(54 - e_n)) as a 64-bit integer, where e_n = emax - 1022 and
// emax is the largest exponent field in x's column (so |result| <= 2^54):
// the 53-bit significand m of x = m 2^(ex - 1075) shifted by ex - emax + 1
__device__ __forceinline__ long long to_fixed(double x, int emax) {
  const long long bits = __double_as_longlong(x);
  int ex = (int)((bits >> 52) & 0x7ff);
  long long m = bits & 0xfffffffffffffLL;
  if (ex != 0) m |= 0x10000000000000LL;
  else ex = 1;
  const int sh = emax - ex - (kFix - 53);  // right shift (>= -1)
  long long r;
  if (sh < 0) r = m << (-sh);
  else if (sh == 0) r = m;
  else if (sh > 60) r = 0;
  else r = (m + (1LL << (sh - 1))) >> sh;
  return bits < 0 ? -r : r;
}

// 7 balanced base-256 digits (each in [-128, 127]) of |x| <= 2^54, most
// significant first, with 32-bit arithmetic: the low 24 bits give digits
// 4..6 (leaving a carry of 0 or 1), the high part (|x >> 24| <= 2^30) plus
// the carry gives digits 0..3
__device__ __forceinline__ void digits7(long long x, int* d) {
  int hi = (int)(x >> 24);
  int lo = (int)(x & 0xffffffLL);
#pragma unroll
  for (int s = 6; s >= 4; --s) {
    const int q = ((lo + 128) & 255) - 128;
    d[s] = q;
    lo = (lo - q) >> 8;
  }
  hi += lo;
#pragma unroll
  for (int s = 3; s >= 0; --s) {
    const int q = ((hi + 128) & 255) - 128;
    d[s] = q;
    hi = (hi - q) >> 8;
  }
}

// }}}

// Split data columns into FP16 digit slices (+ column exponent fields).
// src(n, k) returns the FP64 value of column n < NC, row k < K; columns up to
// NPAD and rows up to KP are written as zero digits.
template <class G, class Src>
__device__ __forceinline__ void split_columns(unsigned char* slices, int* col_emax,
                                              Src src) {
  const int t = threadIdx.x, lane = t & 31;
  // column exponents: one warp per column, lanes split the rows
  for (int n = t >> 5; n < G::NPAD; n += kTcBlock / 32) {
    int em = 0;
    if (n < G::NC)
      for (int k = lane; k < G::K; k += 32) {
        const int ex = dexp(src(n, k));
        em = ex > em ? ex : em;
      }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const int o = __shfl_xor_sync(0xffffffffu, em, off);
      em = o > em ? o : em;
    }
    if (lane == 0) col_emax[n] = em;
  }
  __syncthreads();
  // digits: each warp fills whole 8 x 16-byte core matrices, one 4-byte word
  // (rows k, k + 1 of one column) per lane: stores free of bank conflicts
  constexpr int ITEMS = (G::NPAD / 8) * G::KC * 32;
  for (int idx = t; idx < ITEMS; idx += kTcBlock) {
    const int kp4 = idx & 3, nr = (idx >> 2) & 7;
    const int blk = idx >> 5;                 // n-group * KC + k-chunk
    const int ng = blk / G::KC, kc = blk - ng * G::KC;
    const int n = ng * 8 + nr;
    const int k = kc * 8 + 2 * kp4;
    long long x0 = 0, x1 = 0;
    if (n < G::NC) {
      const int em = col_emax[n];
      if (k < G::K) x0 = to_fixed(src(n, k), em);
      if (k + 1 < G::K) x1 = to_fixed(src(n, k + 1), em);
    }
    int d0[kS], d1[kS];
    digits7(x0, d0);
    digits7(x1, d1);
    unsigned char* dst = slices + ng * G::SBO + kc * 128 + nr * 16 + kp4 * 4;
#pragma unroll
    for (int sl = 0; sl < kS; ++sl)
      *reinterpret_cast<uint32_t*>(dst + sl * G::B_SLICE) = digits_to_half2(d0[sl], d1[sl]);
  }
  fence_async_smem();
}

// Issue every digit-pair product of one contraction (one thread): level l
// accumulates into tensor-memory columns (l - 2) NPAD.., then commit on `bar`.
template <class G>
__device__ __forceinline__ void issue_products(uint32_t a_s, uint32_t b_s, uint32_t tmem,
                                              uint64_t* bar) {
  tc_fence_after();  // order after the barrier that published the slices / freed TMEM
#pragma unroll 1
  for (int l = 2; l <= kLevels; ++l) {
    const int ilo = l - kS > 1 ? l - kS : 1;
    const int ihi = l - 1 < kS ? l - 1 : kS;
    uint32_t acc = 0;
#pragma unroll 1
    for (int i = ilo; i <= ihi; ++i) {
      const int j = l - i;
#pragma unroll
      for (int kt = 0; kt < G::KT; ++kt) {
        const uint64_t da = smem_desc(a_s + (i - 1) * G::A_SLICE + kt * 256, 128, G::SBO);
        const uint64_t db = smem_desc(b_s + (j - 1) * G::B_SLICE + kt * 256, 128, G::SBO);
        tc_mma(tmem + (uint32_t)((l - 2) * G::NPAD), da, db, G::IDESC, acc);
        acc = 1;
      }
    }
  }
  tc_commit(bar);
}

// Read the level sums out of tensor memory and recombine them.  Warp w may
// read tensor-memory lanes 32 (w % 4).. only; lanes (= rows) at or past M and
// columns at or past NC are skipped (warp-uniformly), and the columns of a
// lane quadrant are shared by the warps that can read it.  Per 8 columns the
// 7 level loads are issued before one wait; the recombination is integer
// work.  Writes C (FP64) into out[row * NC + col].
template <class G>
__device__ __forceinline__ void fold_products(uint32_t tmem, const int* row_exp,
                                             const int* col_emax, double* out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = warp & 3;
  if (32 * q >= G::M) return;                    // no real rows in this quadrant
  constexpr int NW = kTcBlock / 32 / 4;            // warps per lane quadrant
  const int row = 32 * q + lane;
  const uint32_t tq = tmem + ((uint32_t)(32 * q) << 16);
  const int e_row = row < G::M ? row_exp[row] : 0;
  constexpr int CHUNKS = (G::NC + 7) / 8;
#pragma unroll 1
  for (int ch = warp >> 2; ch < CHUNKS; ch += NW) {
    const int c0 = ch * 8;
    uint32_t v[kLevels - 1][8];
#pragma unroll
    for (int l = 0; l < kLevels - 1; ++l)
      tc_ld8(tq + (uint32_t)(l * G::NPAD + c0), v[l]);
    tc_wait_ld();
    // level sums (exact integers |v_l| < 2^24) -> W = G_hi 2^32 + G_lo with
    // G_hi = v2 2^16 + v3 2^8 + v4, G_lo = v5 2^24 + v6 2^16 + v7 2^8 + v8,
    // written as W = T 2^28 + f (|T| < 2^45, f in [0, 2^28))
    long long wt[8];
    unsigned wf[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      long long x[kLevels - 1];
#pragma unroll
      for (int l = 0; l < kLevels - 1; ++l) {
        // level l + 2 sums l + 1 digit pairs over K: |v| <= (l + 1) K 2^14,
        // below 2^22 (the two-instruction form) while (l + 1) K < 256
        const float fv = __uint_as_float(v[l][j]);
        x[l] = (l + 1) * G::K < 256 ? f32_exact_int(fv) : f32_exact_int24(fv);
      }
      const long long hi = x[0] * 65536 + x[1] * 256 + x[2];
      const long long lo = x[3] * 16777216 + x[4] * 65536 + x[5] * 256 + x[6];
      wt[j] = hi * 16 + (lo >> 28);
      wf[j] = (unsigned)(lo & 0x0fffffffLL);
    }
    if (row < G::M) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int col = c0 + j;
        if (col < G::NC) {
          // C = W 2^(e_m + e_n - 60), e_n = col_emax - 1022; RN(W) 2^(sc - 28)
          const int sc = e_row + col_emax[col] - 1022 - 32;
          double r;
          if (!fixed_to_double(wt[j], wf[j], sc - 28, &r))  // not a normal double
            r = fma((double)wf[j], 0x1p-28, i64_exact_double(wt[j])) * pow2(sc);
          // a NaN or infinity in the column gives NaN, as the FP64 products would
          out[row * G::NC + col] =
              col_emax[col] == 0x7ff ? __longlong_as_double(0x7ff8000000000000LL) : r;
        }
      }
    }
  }
}

}  // namespace tc

template <int N, int EQ, int MODE>
__global__ void __launch_bounds__(tc::kTcBlock, 1) dg_rhs_tc_kernel(const RhsArgs a) {
  using P = tc::Plan<N, EQ>;
  using GV = typename P::GV;
  using GL = typename P::GL;
  constexpr int NP = P::NP, NFPT = P::NFPT, NF = P::NF, E = P::E;
  constexpr bool STAGE = (MODE & MODE_STAGE) != 0;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint64_t mma_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int ops_ok;
  __shared__ uint64_t in_bar[2];  // PREFETCH: input buffer b complete
  __shared__ int in_bulk[2];      // PREFETCH: buffer b's tile came by bulk copies
  constexpr bool PF = P::PREFETCH;

  const int t = threadIdx.x;
  if constexpr (PF) {  // rows past a partial tile's elements stay finite
    for (int idx = t; idx < 2 * P::IN_BYTES / 16; idx += tc::kTcBlock)
      reinterpret_cast<uint4*>(smem + P::SM_IN)[idx] = make_uint4(0u, 0u, 0u, 0u);
  }
  if (t == 0) {
    mbar_init(&bar, 1);
    mbar_init(&mma_bar, 1);
    mbar_init(&in_bar[0], 1);
    mbar_init(&in_bar[1], 1);
    mbar_arrive_expect_tx(&bar, a.ops_bytes);
    bulk_g2s(smem + P::SM_OPS, a.ops, a.ops_bytes, &bar);
    const bool ok = mbar_wait_bounded(&bar, 0);
    if (!ok) {
      raise_status(a.status, DG_ERR_TIMEOUT);
      mbar_wait_bounded(&bar, 0);
    }
    ops_ok = ok ? 1 : 0;
  }
  __syncthreads();
  if (!ops_ok) return;
  // tensor memory for the level accumulators, held until the CTA exits
  if ((t >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(&tmem_base)), "r"(P::TMEM_ALLOC)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_base;
  // barriers 0: products, 1 + b: input buffer b (PREFETCH)
  constexpr int kMma = 0, kIn0 = 1;
  AsyncLedger<3> led;
  led.init();

  const uint32_t ops_s = smem_u32(smem + P::SM_OPS);
  const int* rexp_v = reinterpret_cast<const int*>(smem + P::SM_OPS + P::OPS_GV + GV::DIGITS);
  const int* rexp_l = reinterpret_cast<const int*>(smem + P::SM_OPS + P::OPS_GL + GL::DIGITS);
  double* sQ = reinterpret_cast<double*>(smem + P::SM_Q);
  unsigned char* sR1 = smem + P::SM_R1;
  const uint32_t sR1_s = smem_u32(sR1);
  double* sR2 = reinterpret_cast<double*>(smem + P::SM_R2);
  double* sG = reinterpret_cast<double*>(smem + P::SM_GEO);
  int* sExp = reinterpret_cast<int*>(smem + P::SM_EXP);
  // products of one contraction: issue (thread 0), wait (bounded), fold.
  // false (uniformly) when some thread's wait gave up: the CTA then stops
  // reading tensor memory and leaves its tile loop
  auto contract = [&](auto gtag, uint32_t a_s, const int* rexp, double* out) -> bool {
    using G = decltype(gtag);
    if (t == 0) {
      tc::issue_products<G>(a_s, sR1_s, tmem, &mma_bar);
      led.issue(kMma);
    }
    const bool ok = led.complete(kMma, mbar_wait_bounded(&mma_bar, led.phase[kMma]));
    if (!ok) raise_status(a.status, DG_ERR_TIMEOUT);
    if (__syncthreads_or(!ok)) return false;
    tc::tc_fence_after();
    tc::fold_products<G>(tmem, rexp, sExp, out);
    tc::tc_fence_before();
    __syncthreads();
    return true;
  };

  const int el = t / NP;
  const int i = t - el * NP;
  const bool active = el < E;
  const int64_t nel = a.nel;
  const int64_t nelnp = nel * NP;
  const int64_t ntiles = (nel + E - 1) / E;

  // PREFETCH: (thread 0) the inputs of tile `tl` into buffer b by 1D bulk
  // copies: 1 when issued, 0 when a size or source address is not 16-byte
  // aligned (the tile then loads with plain loads)
  auto issue_in = [&](int64_t tl, int b) -> int {
    const int64_t e0n = tl * E;
    const int ec = (nel - e0n) < (int64_t)E ? (int)(nel - e0n) : E;
    const uint32_t bq = (uint32_t)ec * NP * 8, bf = (uint32_t)ec * NFPT * 8,
                   bg = (uint32_t)ec * 9 * 8;
    bool ok = (bq % 16u) == 0u && (bf % 16u) == 0u && (bg % 16u) == 0u &&
              ((uintptr_t)(a.metric + e0n * 9) & 15u) == 0u;
#pragma unroll
    for (int k = 0; k < NF; ++k)
      ok = ok && ((uintptr_t)(a.q + k * nelnp + e0n * NP) & 15u) == 0u &&
           ((uintptr_t)(a.flux_in + (k * nel + e0n) * NFPT) & 15u) == 0u;
    if (!ok) return 0;
    unsigned char* buf = smem + P::SM_IN + b * P::IN_BYTES;
    led.issue(kIn0 + b);
    mbar_arrive_expect_tx(&in_bar[b], (uint32_t)NF * (bq + bf) + bg);
#pragma unroll
    for (int k = 0; k < NF; ++k) {
      bulk_g2s(buf + k * (E * NP * 8), a.q + k * nelnp + e0n * NP, bq, &in_bar[b]);
      bulk_g2s(buf + P::IN_Q + k * (E * NFPT * 8), a.flux_in + (k * nel + e0n) * NFPT, bf,
               &in_bar[b]);
    }
    bulk_g2s(buf + P::IN_Q + P::IN_F, a.metric + e0n * 9, bg, &in_bar[b]);
    return 1;
  };
  if constexpr (PF) {
    if (t == 0) in_bulk[0] = blockIdx.x < ntiles ? issue_in(blockIdx.x, 0) : 0;
    __syncthreads();
  }

  int it = 0;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int64_t e0 = tile * E;
    const int ecount = (nel - e0) < (int64_t)E ? (int)(nel - e0) : E;
    const int ib = it & 1;
    double* sF = sR2;  // face values (PREFETCH: in the input buffer)
    if constexpr (PF) {
      unsigned char* buf = smem + P::SM_IN + ib * P::IN_BYTES;
      sQ = reinterpret_cast<double*>(buf);
      sF = reinterpret_cast<double*>(buf + P::IN_Q);
      sG = reinterpret_cast<double*>(buf + P::IN_Q + P::IN_F);
      // the other buffer's last reader was the previous tile, before its
      // final barrier
      if (t == 0) {
        const int64_t nx = tile + gridDim.x;
        in_bulk[ib ^ 1] = nx < ntiles ? issue_in(nx, ib ^ 1) : 0;
      }
    }

    // {{{ 1. state and metric (PREFETCH: and face values) -> shared memory
    bool in_ok = true;
    if (PF && in_bulk[ib]) {
      in_ok = led.complete(kIn0 + ib,
                           mbar_wait_bounded(&in_bar[ib], led.phase[kIn0 + ib]));
      if (!in_ok) raise_status(a.status, DG_ERR_TIMEOUT);
    } else {
      const double* qk = a.q + e0 * NP;
#pragma unroll
      for (int k = 0; k < NF; ++k, qk += nelnp)
        for (int rem = t; rem < E * NP; rem += tc::kTcBlock)
          sQ[k * (E * NP) + rem] = rem < ecount * NP ? __ldg(qk + rem) : 0.0;
      const double* mt = a.metric + e0 * 9;
      for (int idx = t; idx < 9 * E; idx += tc::kTcBlock)
        sG[idx] = idx < 9 * ecount ? __ldg(mt + idx) : 0.0;
      if constexpr (PF) {
        const int64_t nfpt_all = nel * NFPT;
        const double* fk = a.flux_in + e0 * NFPT;
#pragma unroll
        for (int k = 0; k < NF; ++k, fk += nfpt_all)
          for (int rem = t; rem < E * NFPT; rem += tc::kTcBlock)
            sF[k * (E * NFPT) + rem] = rem < ecount * NFPT ? __ldg(fk + rem) : 0.0;
      }
    }
    if (__syncthreads_or(!in_ok)) break;  // an input copy never arrived
    // }}}

    // {{{ 2. pointwise pre-pass (FP64): inputs of the weak divergence
    if constexpr (EQ == DG_WAVE) {
      if (active) {
        const double* G = sG + el * 9;
        const double v0 = sQ[(1 * E + el) * NP + i], v1 = sQ[(2 * E + el) * NP + i],
                     v2 = sQ[(3 * E + el) * NP + i];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          sR2[(r * E + el) * NP + i] =
              fma(G[r * 3 + 0], v0, fma(G[r * 3 + 1], v1, G[r * 3 + 2] * v2));
      }
    } else if constexpr (EQ == DG_EULER) {
      if (active) {
        const double* G = sG + el * 9;
        double p = 0.0, rinv = 0.0;
        if (el < ecount) {
          const int64_t gidx = e0 * NP + (el * NP + i);
          p = __ldg(a.aux + gidx);
          rinv = __ldg(a.aux + nelnp + gidx);
        }
        const double en = sQ[(1 * E + el) * NP + i];
        const double m[3] = {sQ[(2 * E + el) * NP + i], sQ[(3 * E + el) * NP + i],
                             sQ[(4 * E + el) * NP + i]};
        // metric-combined fluxes through U_r = (G u)_r (as in dg_rhs_kernel)
        const double u[3] = {m[0] * rinv, m[1] * rinv, m[2] * rinv};
        const double ep = en + p;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const double* Gr = G + r * 3;
          const double ur = fma(Gr[0], u[0], fma(Gr[1], u[1], Gr[2] * u[2]));
          double* out = sR2 + (r * E + el) * NP + i;
          constexpr int KS = 3 * E * NP;  // stride of k in R2
          out[0 * KS] = fma(Gr[0], m[0], fma(Gr[1], m[1], Gr[2] * m[2]));
          out[1 * KS] = ep * ur;
#pragma unroll
          for (int c = 0; c < 3; ++c) out[(2 + c) * KS] = fma(m[c], ur, p * Gr[c]);
        }
      }
    }
    if constexpr (P::NAUX > 0) __syncthreads();
    // }}}

    // {{{ 3. volume data -> digit slices, 4. volume product -> R2 (FP64)
    if constexpr (EQ == DG_WAVE) {
      tc::split_columns<GV>(sR1, sExp, [&](int n, int k) {
        const int f = n / E, e = n - f * E;  // f = 0: u; f = 1..3: (G v)_{f-1}
        return f == 0 ? sQ[e * NP + k] : sR2[((f - 1) * E + e) * NP + k];
      });
    } else if constexpr (EQ == DG_EULER) {
      tc::split_columns<GV>(sR1, sExp, [&](int n, int k) {
        const int f = n / E, e = n - f * E;  // column (field, element)
        const int r = k / NP, j = k - r * NP;
        return sR2[((f * 3 + r) * E + e) * NP + j];
      });
    } else {
      tc::split_columns<GV>(sR1, sExp, [&](int n, int k) { return sQ[n * NP + k]; });
    }
    __syncthreads();
    if (!contract(GV{}, ops_s + P::OPS_GV, rexp_v, sR2)) break;
    // }}}

    // {{{ 5. volume term per node (registers)
    double vol[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) vol[k] = 0.0;
    if (active) {
      const double* G = sG + el * 9;
      const double* o = sR2;  // GV::M x GV::NC
      constexpr int NC = GV::NC;
      if constexpr (EQ == DG_WAVE) {
        // ur_r = W_r u (column 0 block); div = sum_r W_r (G v)_r (diagonal blocks)
        const double c = a.p0;
        const double u0 = o[(0 * NP + i) * NC + el], u1 = o[(1 * NP + i) * NC + el],
                     u2 = o[(2 * NP + i) * NC + el];
        const double dv = o[(0 * NP + i) * NC + 1 * E + el] +
                          o[(1 * NP + i) * NC + 2 * E + el] +
                          o[(2 * NP + i) * NC + 3 * E + el];
        vol[0] = -c * dv;
#pragma unroll
        for (int x = 0; x < 3; ++x)
          vol[1 + x] = -c * fma(G[0 * 3 + x], u0, fma(G[1 * 3 + x], u1, G[2 * 3 + x] * u2));
      } else if constexpr (EQ == DG_EULER) {
#pragma unroll
        for (int k = 0; k < 5; ++k) vol[k] = o[i * NC + k * E + el];
      } else {
        auto dx = [&](int k, int x) {
          const double d0 = o[(0 * NP + i) * NC + k * E + el];
          const double d1 = o[(1 * NP + i) * NC + k * E + el];
          const double d2 = o[(2 * NP + i) * NC + k * E + el];
          return fma(G[0 * 3 + x], d0, fma(G[1 * 3 + x], d1, G[2 * 3 + x] * d2));
        };
        vol[0] = dx(5, 1) - dx(4, 2);
        vol[1] = dx(3, 2) - dx(5, 0);
        vol[2] = dx(4, 0) - dx(3, 1);
        vol[3] = -(dx(2, 1) - dx(1, 2));
        vol[4] = -(dx(0, 2) - dx(2, 0));
        vol[5] = -(dx(1, 0) - dx(0, 1));
      }
    }
    __syncthreads();
    // }}}

    // {{{ 6. face values of the tile (NF, E, 4 Nfp) -> R2 (PREFETCH: already
    //        in the input buffer), digit slices, 7. LIFT product
    if constexpr (!PF) {
      const int64_t nfpt_all = nel * NFPT;
      const double* fk = a.flux_in + e0 * NFPT;
#pragma unroll
      for (int k = 0; k < NF; ++k, fk += nfpt_all)
        for (int rem = t; rem < E * NFPT; rem += tc::kTcBlock)
          sF[k * (E * NFPT) + rem] = rem < ecount * NFPT ? __ldg(fk + rem) : 0.0;
      __syncthreads();
    }
    tc::split_columns<GL>(sR1, sExp, [&](int n, int k) { return sF[n * NFPT + k]; });
    __syncthreads();
    double* sL = sR2 + NF * E * NFPT;            // Np x (NF E)
    if (!contract(GL{}, ops_s + P::OPS_GL, rexp_l, sL)) break;
    // }}}

    // {{{ 8. epilogue: store or fold into the RK stage
    if (active && el < ecount) {
      int64_t gidx = e0 * NP + (el * NP + i);
#pragma unroll
      for (int k = 0; k < NF; ++k, gidx += nelnp) {
        double val = vol[k] + sL[i * (NF * E) + k * E + el];
        if constexpr (EQ == DG_MAXWELL) val = val * (k < 3 ? a.k[4] : a.k[5]);
        if constexpr (STAGE)
          if (a.rhs_unscaled) a.rhs_unscaled[gidx] = val;
        if (a.elem_scale) val *= __ldg(a.elem_scale + e0 + el);
        if constexpr (!STAGE) {
          a.rhs[gidx] = val;
        } else {
          const double r = (a.rk_a != 0.0 ? a.rk_a * a.res[gidx] : 0.0) + a.rk_dt * val;
          a.res[gidx] = r;
          a.q_out[gidx] = sQ[(k * E + el) * NP + i] + a.rk_b * r;
        }
      }
    }
    __syncthreads();
    // }}}
  }
  // after a wait gave up: before shared and tensor memory are released, the
  // issuing thread waits (bounded) for the copies and products it still owes.
  // If one of them never completes, the status already reads DG_ERR_TIMEOUT
  // and the tensor memory is released with that product outstanding.
  if (t == 0 && led.owes_any()) {
    if (led.owes(kMma)) mbar_wait_bounded(&mma_bar, led.phase[kMma]);
    for (int b = 0; b < 2; ++b)
      if (led.owes(kIn0 + b)) mbar_wait_bounded(&in_bar[b], led.phase[kIn0 + b]);
  }
  tc::tc_fence_before();
  __syncthreads();
  if ((t >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"(P::TMEM_ALLOC)
                 : "memory");
}

}  // namespace dg
