// FP64 RHS with the contractions on the tensor cores: exact FP64 emulation
// by FP16 digit slices (error-free splitting in the manner of Ozaki et al.,
// "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applicability", Numer.
// Algorithms 59, 2012).
//
// GB300 issues FP64 at about 1.2 TFLOP/s but FP16 tensor-core products at
// hundreds of TFLOP/s, and the high-order DG contractions (volume
// derivatives, LIFT) keep the FP64 pipe ~97 % busy.  Here every contraction
// C = A X (A: a reference operator, M x K; X: K x NC columns of FP64 data,
// one column per element and field) is evaluated as
//
//   A = 2^(e_m - 54) A_int,  X = 2^(e_n - 54) X_int   (per-row / per-column
//   exponents, 54-bit integers), each integer written as 8 balanced base-128
//   digits d_1..d_8 in [-64, 64] (exact in FP16);
//   v_l = sum_{i + j = l} D^A_i D^X_j    for l = 2..9, one FP16 tensor-core
//   GEMM per digit pair, accumulated in FP32 -- exactly, because
//   |v_l| <= 8 * K * 64^2 < 2^22 for K <= 112;
//   C = 2^(e_m + e_n - 31) (G_hi + 2^-28 G_lo),  G_hi = sum_{l<=5} v_l 2^(7(5-l)),
//   G_lo = sum_{l>=6} v_l 2^(7(9-l)) in 64-bit integers (exact).
//
// Dropped digit pairs (l > 9) and the 54-bit rounding of the inputs bound the
// error by ~2^-53 of sum_k |A_mk| |X_kn| -- the size of FP64's own
// rounding.  Splitting and recombination are integer work (no FP64 pipe);
// per output the FP64 pipe sees 4 instructions instead of K FMAs.
//
// The kernel is the volume/LIFT half of the face-shared path: face values
// come from dg_face_flux_kernel (and, for Euler, pressure and 1/rho from
// dg_euler_aux_kernel), pointwise work (Euler fluxes, metric terms, curl,
// RK epilogue) stays in FP64.  Tensor-core products use the warp-level
// mma.sync m16n8k16 FP16 -> FP32 form: its operands come from registers and
// shared memory the kernel itself fills, so no tensor-memory allocation or
// asynchronous completion is involved.
#pragma once

#include <cuda_fp16.h>

#include <type_traits>

#include "dg_face.cuh"
#include "dg_rhs.cuh"

namespace dg {
namespace tc {

constexpr int kS = 8;        // digits per value
constexpr int kFix = 54;     // fixed-point bits
constexpr int kLevels = 9;   // digit pairs with i + j <= kLevels are kept

constexpr int r16(int x) { return (x + 15) & ~15; }
constexpr int r8(int x) { return (x + 7) & ~7; }
constexpr int p16(int bytes) { return (bytes + 15) & ~15; }

// One emulated product: operator A (M x K) times NC data columns of length K.
//   operator block (global and shared): FP16 digits in blocks of 512 bytes per
//   (digit s, m-tile, k-step), each block the four 8 x 8 matrices of the mma
//   A fragment in ldmatrix.x4 order (rows 0-7 / 8-15 x columns 0-7 / 8-15),
//   then M_P int32 row exponents;
//   data slices (shared): FP16 digits, blocks of 256 bytes per (digit, n-tile,
//   k-step) in ldmatrix.x2 order (two 8 x 8 matrices, row = column n).
// A warp unit covers 1 or 2 m-tiles x 2 n-tiles, so every operator
// fragment loaded from shared memory feeds two tensor-core products.
template <int M_, int K_, int NC_>
struct Gemm {
  static constexpr int M = M_, K = K_, NC = NC_;
  static constexpr int MP = r16(M), KP = r16(K), NCP = r8(NC);
  static constexpr int MT = MP / 16, KT = KP / 16, NT = NCP / 8;
  // warp unit: UM x 2 tiles; UM = 2 only when that still leaves >= 16 units
  static constexpr int UM = ((MT + 1) / 2) * ((NT + 1) / 2) >= 16 ? 2 : 1;
  static constexpr int MB = (MT + UM - 1) / UM, NB = (NT + 1) / 2;
  static constexpr int UNITS = MB * NB;
  static constexpr int DIGITS = kS * MT * KT * 512;
  static constexpr int OPS_BYTES = p16(DIGITS + MP * 4);
  static constexpr int SLICE_STRIDE = NT * KT * 256;   // bytes per digit slice
  static constexpr int SLICE_BYTES = kS * SLICE_STRIDE;
  static_assert(K <= 112, "exact FP32 level sums need K <= 112");
};

// Elements per CTA tile: 256 / Np, fewer at order 4 so the FP16 operator
// digits and the tile's slices fit in shared memory.
constexpr int tile_elems(int N, int EQ, int np) {
  return N < 4 ? 256 / np : (EQ == DG_EULER ? 5 : (EQ == DG_MAXWELL ? 6 : 7));
}

// Products of one equation at order N.  GV, the volume product:
//   wave, maxwell: stacked rows [A_0; A_1; A_2] (3 Np x Np) applied to
//     columns (field f, element e) at n = f E + e -- maxwell the six fields,
//     wave u and the three metric-combined velocity components (of whose
//     products only the diagonal blocks are used);
//   euler: concatenated columns [A_0 A_1 A_2] (Np x 3 Np) applied to the
//     metric-combined fluxes of each (field, element);
// GL: LIFT (Np x 4 Nfp) applied to the face values of each (field, element).
template <int N, int EQ>
struct Plan {
  static constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP, NFPT = Shape<N>::NFPT;
  static constexpr int NF = EqInfo<EQ>::NF;
  static constexpr int E = tile_elems(N, EQ, NP);
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
  static constexpr int NCOLS = cmax(GV::NCP, GL::NCP);
  // shared memory: ops | state (FP64) | R1 (slices) | R2 (FP64 scratch) |
  // metric | column exponents
  static constexpr int SM_OPS = 0;
  static constexpr int SM_Q = p16(OPS_BYTES);
  static constexpr int SM_R1 = SM_Q + p16(NF * E * NP * 8);
  static constexpr int SM_R2 = SM_R1 + R1_BYTES;
  static constexpr int SM_GEO = SM_R2 + R2_BYTES;
  static constexpr int SM_EXP = SM_GEO + p16(9 * E * 8);
  static constexpr int SMEM_BYTES = SM_EXP + p16(NCOLS * 4);
  static_assert(SMEM_BYTES <= 227 * 1024, "tile does not fit in shared memory");
};

// {{{ device helpers

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// The "memory" clobbers keep the compiler from moving these shared-memory
// reads above the barrier and the stores that fill the slices: the address
// is a plain integer, so without it the read is invisible to alias analysis.
__device__ __forceinline__ void ldsm_x2(uint32_t& r0, uint32_t& r1, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(addr)
               : "memory");
}

__device__ __forceinline__ void ldsm_x4(uint32_t* r, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr)
               : "memory");
}

// two digits in [-64, 64] -> half2: the bit pattern 0x6600 + d is the half
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
  return __float_as_int(v + 12582912.0f) - 0x4B400000;
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

// biased exponent field of a double (0 for zero and subnormals)
__device__ __forceinline__ int dexp(double x) {
  return (__double2hiint(x) >> 20) & 0x7ff;
}

// x -> round(x 2^(54 - e_n)) as a 64-bit integer, where e_n = emax - 1022 and
// emax is the largest exponent field in x's column (so |result| <= 2^54)
__device__ __forceinline__ long long to_fixed(double x, int emax) {
  const long long bits = __double_as_longlong(x);
  int ex = (int)((bits >> 52) & 0x7ff);
  long long m = bits & 0xfffffffffffffLL;
  if (ex != 0) m |= 0x10000000000000LL;
  else ex = 1;
  const int sh = emax - ex - 1;  // right shift
  long long r;
  if (sh < 0) r = m << 1;
  else if (sh == 0) r = m;
  else if (sh > 60) r = 0;
  else r = (m + (1LL << (sh - 1))) >> sh;
  return bits < 0 ? -r : r;
}

// 8 balanced base-128 digits of |x| <= 2^54, most significant first, with
// 32-bit arithmetic: the low 28 bits give digits 4..7 (leaving a carry of
// 0 or 1), the high part plus the carry gives digits 0..3
__device__ __forceinline__ void digits8(long long x, int* d) {
  int hi = (int)(x >> 28);
  int lo = (int)(x & 0x0fffffffLL);
#pragma unroll
  for (int s = 7; s >= 4; --s) {
    const int q = ((lo + 64) & 127) - 64;
    d[s] = q;
    lo = (lo - q) >> 7;
  }
  hi += lo;
#pragma unroll
  for (int s = 3; s >= 0; --s) {
    const int q = ((hi + 64) & 127) - 64;
    d[s] = q;
    hi = (hi - q) >> 7;
  }
}

// }}}

// Split data columns into FP16 digit slices (+ column exponent fields).
// src(n, k) returns the FP64 value of column n < NC, row k < K.
template <class G, class Src>
__device__ __forceinline__ void split_columns(unsigned char* slices, int* col_emax,
                                              Src src) {
  const int t = threadIdx.x, lane = t & 31;
  // column exponents: one warp per column, lanes split the rows
  for (int n = t >> 5; n < G::NCP; n += kBlock / 32) {
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
  // digits: each warp fills whole 8 x 8 matrices, one 4-byte word (two rows
  // k, k + 1 of one column) per lane, so the stores are free of bank conflicts
  constexpr int ITEMS = G::NT * G::KT * 64;
  for (int idx = t; idx < ITEMS; idx += kBlock) {
    const int kp4 = idx & 3, nr = (idx >> 2) & 7, kh = (idx >> 5) & 1;
    const int blk = idx >> 6;                 // nt * KT + kt
    const int nt = blk / G::KT, kt = blk - nt * G::KT;
    const int n = nt * 8 + nr;
    const int k = kt * 16 + kh * 8 + 2 * kp4;
    long long x0 = 0, x1 = 0;
    if (n < G::NC) {
      const int em = col_emax[n];
      if (k < G::K) x0 = to_fixed(src(n, k), em);
      if (k + 1 < G::K) x1 = to_fixed(src(n, k + 1), em);
    }
    int d0[kS], d1[kS];
    digits8(x0, d0);
    digits8(x1, d1);
    unsigned char* dst = slices + blk * 256 + kh * 128 + nr * 16 + kp4 * 4;
#pragma unroll
    for (int sl = 0; sl < kS; ++sl)
      *reinterpret_cast<uint32_t*>(dst + sl * G::SLICE_STRIDE) = digits_to_half2(d0[sl], d1[sl]);
  }
}

// One warp's unit of an emulated product: m-tiles 2 mb, 2 mb + 1 and n-tiles
// 2 nb, 2 nb + 1 (where they exist).  Writes C (FP64) into out[row * NC + col].
template <class G>
__device__ __forceinline__ void gemm_unit(int unit, uint32_t ops_s, const int* row_exp,
                                          uint32_t slices_s, const int* col_emax,
                                          double* out) {
  const int lane = threadIdx.x & 31;
  const int mb = unit / G::NB;
  const int mt0 = G::UM * mb, nt0 = 2 * (unit - mb * G::NB);
  const bool m2 = G::UM == 2 && mt0 + 1 < G::MT, n2 = nt0 + 1 < G::NT;
  long long ghi[2][2][4], glo[2][2][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) ghi[a][b][c] = glo[a][b][c] = 0;

#pragma unroll 1
  for (int l = 2; l <= kLevels; ++l) {
    float acc[2][2][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
    const int ilo = l - kS > 1 ? l - kS : 1;
    const int ihi = l - 1 < kS ? l - 1 : kS;
#pragma unroll 2
    for (int i = ilo; i <= ihi; ++i) {
      const int j = l - i;
      const uint32_t ablk = ops_s + ((i - 1) * G::MT + mt0) * G::KT * 512 + lane * 16;
      const uint32_t bblk =
          slices_s + (j - 1) * G::SLICE_STRIDE + nt0 * G::KT * 256 + (lane & 15) * 16;
#pragma unroll
      for (int kt = 0; kt < G::KT; ++kt) {
        uint32_t a0[4], a1[4], b0[2], b1[2];
        ldsm_x4(a0, ablk + kt * 512);
        ldsm_x2(b0[0], b0[1], bblk + kt * 256);
        mma16816(acc[0][0], a0, b0[0], b0[1]);
        if (n2) {
          ldsm_x2(b1[0], b1[1], bblk + (G::KT + kt) * 256);
          mma16816(acc[0][1], a0, b1[0], b1[1]);
        }
        if (m2) {
          ldsm_x4(a1, ablk + (G::KT + kt) * 512);
          mma16816(acc[1][0], a1, b0[0], b0[1]);
          if (n2) mma16816(acc[1][1], a1, b1[0], b1[1]);
        }
      }
    }
    const int sh = l <= 5 ? 7 * (5 - l) : 7 * (9 - l);
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const long long v = (long long)((unsigned long long)(long long)
                                              f32_exact_int(acc[a][b][c]) << sh);
          if (l <= 5) ghi[a][b][c] += v;
          else glo[a][b][c] += v;
        }
  }
  const int g = lane >> 2, tq = lane & 3;
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    if (a == 1 && !m2) break;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      if (b == 1 && !n2) break;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int row = (mt0 + a) * 16 + g + (c >= 2 ? 8 : 0);
        const int col = (nt0 + b) * 8 + 2 * tq + (c & 1);
        if (row < G::M && col < G::NC) {
          const double r = fma(i64_exact_double(glo[a][b][c]), 0x1p-28,
                               i64_exact_double(ghi[a][b][c]));
          out[row * G::NC + col] = r * pow2(row_exp[row] + col_emax[col] - 1022 - 31);
        }
      }
    }
  }
}

// All units of one product, spread over the CTA's warps.
template <class G>
__device__ __forceinline__ void gemm_all(uint32_t ops_s, const int* row_exp,
                                         uint32_t slices_s, const int* col_emax,
                                         double* out) {
  for (int u = threadIdx.x >> 5; u < G::UNITS; u += kBlock / 32)
    gemm_unit<G>(u, ops_s, row_exp, slices_s, col_emax, out);
}

}  // namespace tc

template <int N, int EQ, int MODE>
__global__ void __launch_bounds__(kBlock, 1) dg_rhs_tc_kernel(const RhsArgs a) {
  using P = tc::Plan<N, EQ>;
  using GV = typename P::GV;
  using GL = typename P::GL;
  constexpr int NP = P::NP, NFPT = P::NFPT, NF = P::NF, E = P::E;
  constexpr bool STAGE = (MODE & MODE_STAGE) != 0;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ int ops_ok;

  const int t = threadIdx.x;
  if (t == 0) {
    mbar_init(&bar, 1);
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

  const uint32_t ops_s = smem_u32(smem + P::SM_OPS);
  const int* rexp_v = reinterpret_cast<const int*>(smem + P::SM_OPS + P::OPS_GV + GV::DIGITS);
  const int* rexp_l = reinterpret_cast<const int*>(smem + P::SM_OPS + P::OPS_GL + GL::DIGITS);
  double* sQ = reinterpret_cast<double*>(smem + P::SM_Q);
  unsigned char* sR1 = smem + P::SM_R1;
  const uint32_t sR1_s = smem_u32(sR1);
  double* sR2 = reinterpret_cast<double*>(smem + P::SM_R2);
  double* sG = reinterpret_cast<double*>(smem + P::SM_GEO);
  int* sExp = reinterpret_cast<int*>(smem + P::SM_EXP);

  const int el = t / NP;
  const int i = t - el * NP;
  const bool active = el < E;
  const int64_t nel = a.nel;
  const int64_t nelnp = nel * NP;
  const int64_t ntiles = (nel + E - 1) / E;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t e0 = tile * E;
    const int ecount = (nel - e0) < (int64_t)E ? (int)(nel - e0) : E;

    // {{{ 1. state and metric -> shared memory
    {
      const double* qk = a.q + e0 * NP;
#pragma unroll
      for (int k = 0; k < NF; ++k, qk += nelnp)
        for (int rem = t; rem < E * NP; rem += kBlock)
          sQ[k * (E * NP) + rem] = rem < ecount * NP ? __ldg(qk + rem) : 0.0;
      const double* mt = a.metric + e0 * 9;
      for (int idx = t; idx < 9 * E; idx += kBlock)
        sG[idx] = idx < 9 * ecount ? __ldg(mt + idx) : 0.0;
    }
    __syncthreads();
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
        const double u[3] = {m[0] * rinv, m[1] * rinv, m[2] * rinv};
        double F[5][3];
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          F[0][x] = m[x];
          F[1][x] = u[x] * (en + p);
#pragma unroll
          for (int c = 0; c < 3; ++c) F[2 + c][x] = m[c] * u[x] + (c == x ? p : 0.0);
        }
#pragma unroll
        for (int k = 0; k < 5; ++k)
#pragma unroll
          for (int r = 0; r < 3; ++r)
            sR2[((k * 3 + r) * E + el) * NP + i] =
                fma(G[r * 3 + 0], F[k][0], fma(G[r * 3 + 1], F[k][1], G[r * 3 + 2] * F[k][2]));
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
    tc::gemm_all<GV>(ops_s + P::OPS_GV, rexp_v, sR1_s, sExp, sR2);
    __syncthreads();
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

    // {{{ 6. face values of the tile -> R2, digit slices, 7. LIFT product
    double* sF = sR2;                            // (NF, E, 4 Nfp)
    {
      const int64_t nfpt_all = nel * NFPT;
      const double* fk = a.flux_in + e0 * NFPT;
#pragma unroll
      for (int k = 0; k < NF; ++k, fk += nfpt_all)
        for (int rem = t; rem < E * NFPT; rem += kBlock)
          sF[k * (E * NFPT) + rem] = rem < ecount * NFPT ? __ldg(fk + rem) : 0.0;
    }
    __syncthreads();
    tc::split_columns<GL>(sR1, sExp, [&](int n, int k) { return sF[n * NFPT + k]; });
    __syncthreads();
    double* sL = sR2 + NF * E * NFPT;            // Np x (NF E)
    tc::gemm_all<GL>(ops_s + P::OPS_GL, rexp_l, sR1_s, sExp, sL);
    __syncthreads();
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
}

}  // namespace dg
