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
//   operator block (global and shared): int8 digits + 64, blocks of 256 bytes
//   per (digit s, m-tile, k-step) in lane order (8 bytes per lane: the four
//   half2 registers of the mma A fragment), then M_P int32 row exponents;
//   data slices (shared): FP16 digits, blocks of 256 bytes per (digit, n-tile,
//   k-step) in ldmatrix order (two 8 x 8 matrices, row = column n).
template <int M_, int K_, int NC_>
struct Gemm {
  static constexpr int M = M_, K = K_, NC = NC_;
  static constexpr int MP = r16(M), KP = r16(K), NCP = r8(NC);
  static constexpr int MT = MP / 16, KT = KP / 16, NT = NCP / 8;
  static constexpr int NT2 = (NT + 1) / 2;     // n-tile pairs (one warp unit)
  static constexpr int UNITS = MT * NT2;
  static constexpr int DIGITS = kS * MT * KT * 256;
  static constexpr int OPS_BYTES = p16(DIGITS + MP * 4);
  static constexpr int SLICE_BYTES = kS * NT * KT * 256;
  static_assert(K <= 112, "exact FP32 level sums need K <= 112");
};

// Products of one equation at order N: G1 = stacked rows [A_0; A_1; A_2]
// (3 Np x Np), G2 = concatenated columns [A_0 A_1 A_2] (Np x 3 Np), GL = LIFT.
template <int N, int EQ>
struct Plan {
  static constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP, NFPT = Shape<N>::NFPT;
  static constexpr int NF = EqInfo<EQ>::NF;
  static constexpr int E = kBlock / NP;
  static constexpr bool HAS_G1 = EQ != DG_EULER;
  static constexpr bool HAS_G2 = EQ != DG_MAXWELL;
  // data columns: wave G1/G2 one per element; euler G2, maxwell G1 one per
  // (field, element) at column k * E + el; LIFT one per (field, element)
  using G1 = Gemm<3 * NP, NP, (EQ == DG_WAVE ? E : NF * E)>;
  using G2 = Gemm<NP, 3 * NP, (EQ == DG_WAVE ? E : NF * E)>;
  using GL = Gemm<NP, NFPT, NF * E>;
  // operator block: [G1 | G2 | GL] (absent products take no space)
  static constexpr int OPS_G1 = 0;
  static constexpr int OPS_G2 = OPS_G1 + (HAS_G1 ? G1::OPS_BYTES : 0);
  static constexpr int OPS_GL = OPS_G2 + (HAS_G2 ? G2::OPS_BYTES : 0);
  static constexpr int OPS_BYTES = OPS_GL + GL::OPS_BYTES;

  static constexpr int NAUX = EQ == DG_WAVE ? 3 : (EQ == DG_EULER ? 15 : 0);
  static constexpr int cmax(int x, int y) { return x > y ? x : y; }
  static constexpr int VOL_SLICES = (HAS_G1 ? G1::SLICE_BYTES : 0) +
                                    (HAS_G2 ? G2::SLICE_BYTES : 0);
  static constexpr int R1_BYTES = p16(cmax(VOL_SLICES, GL::SLICE_BYTES));
  static constexpr int OUT_G1 = HAS_G1 ? G1::M * G1::NC : 0;  // doubles
  static constexpr int OUT_G2 = HAS_G2 ? G2::M * G2::NC : 0;
  static constexpr int R2_BYTES = p16(8 * cmax(cmax(NAUX * E * NP, OUT_G1 + OUT_G2),
                                               NF * E * NFPT + GL::M * GL::NC));
  static constexpr int NCOLS = cmax(cmax(HAS_G1 ? G1::NCP : 0, HAS_G2 ? G2::NCP : 0),
                                    GL::NCP);
  // shared memory: ops | state (FP64) | R1 (slices) | R2 (FP64 scratch) |
  // metric | column exponents (two sets)
  static constexpr int SM_OPS = 0;
  static constexpr int SM_Q = p16(OPS_BYTES);
  static constexpr int SM_R1 = SM_Q + p16(NF * E * NP * 8);
  static constexpr int SM_R2 = SM_R1 + R1_BYTES;
  static constexpr int SM_GEO = SM_R2 + R2_BYTES;
  static constexpr int SM_EXP = SM_GEO + p16(9 * E * 8);
  static constexpr int SMEM_BYTES = SM_EXP + p16(2 * NCOLS * 4);
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

// The "memory" clobber keeps the compiler from moving this shared-memory read
// above the barrier and the stores that fill the slices: the address is a
// plain integer, so without it the read is invisible to alias analysis.
__device__ __forceinline__ void ldsm_x2(uint32_t& r0, uint32_t& r1, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r0), "=r"(r1)
               : "r"(addr)
               : "memory");
}

// two biased int8 digits (byte + 64 each) -> half2 of the digits: the bit
// pattern 0x6600 + d is the half 1536 + d for |d| <= 64; one HSUB2 removes
// the 1536 exactly
// (bit moves through the __ushort_as_half / __half_as_ushort intrinsics: no
// pointer type punning, which the optimiser is free to break)
__device__ __forceinline__ uint32_t digits_to_half2(uint32_t packed16) {
  const uint32_t bits = packed16 + 0x65C065C0u;
  const __half2 h = __halves2half2(__ushort_as_half((unsigned short)(bits & 0xffffu)),
                                   __ushort_as_half((unsigned short)(bits >> 16)));
  const __half2 c = __halves2half2(__ushort_as_half((unsigned short)0x6600u),
                                   __ushort_as_half((unsigned short)0x6600u));
  const __half2 d = __hsub2(h, c);
  return (uint32_t)__half_as_ushort(__low2half(d)) |
         ((uint32_t)__half_as_ushort(__high2half(d)) << 16);
}

// 8 biased digit bytes (one lane's share of an A fragment) -> a0..a3
__device__ __forceinline__ void expand_a(const uint2 w, uint32_t* a) {
  a[0] = digits_to_half2(__byte_perm(w.x, 0u, 0x4140));
  a[1] = digits_to_half2(__byte_perm(w.x, 0u, 0x4342));
  a[2] = digits_to_half2(__byte_perm(w.y, 0u, 0x4140));
  a[3] = digits_to_half2(__byte_perm(w.y, 0u, 0x4342));
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

// }}}

// Split data columns into FP16 digit slices (+ column exponent fields).
// src(n, k) returns the FP64 value of column n < NC, row k < K.
template <class G, class Src>
__device__ __forceinline__ void split_columns(unsigned char* slices, int* col_emax,
                                              Src src) {
  const int t = threadIdx.x;
  // column exponents (one thread per column)
  for (int n = t; n < G::NCP; n += kBlock) {
    int em = 0;
    if (n < G::NC)
      for (int k = 0; k < G::K; ++k) {
        const int ex = dexp(src(n, k));
        em = ex > em ? ex : em;
      }
    col_emax[n] = em;
  }
  __syncthreads();
  // digits: one thread per (column, pair of rows)
  constexpr int KH = G::KP / 2;
  for (int idx = t; idx < G::NCP * KH; idx += kBlock) {
    const int n = idx / KH;
    const int k = 2 * (idx - n * KH);
    long long x0 = 0, x1 = 0;
    if (n < G::NC) {
      const int em = col_emax[n];
      if (k < G::K) x0 = to_fixed(src(n, k), em);
      if (k + 1 < G::K) x1 = to_fixed(src(n, k + 1), em);
    }
    const int nt = n >> 3, kt = k >> 4;
    unsigned char* dst = slices + (nt * G::KT + kt) * 256 + ((k & 15) >> 3) * 128 +
                         (n & 7) * 16 + (k & 7) * 2;
#pragma unroll
    for (int s = kS - 1; s >= 0; --s) {  // least significant digit first
      const long long d0 = ((x0 + 64) & 127) - 64;
      const long long d1 = ((x1 + 64) & 127) - 64;
      x0 = (x0 - d0) >> 7;
      x1 = (x1 - d1) >> 7;
      const uint32_t packed =
          ((uint32_t)(d0 + 64) & 0xffffu) | (((uint32_t)(d1 + 64) & 0xffffu) << 16);
      *reinterpret_cast<uint32_t*>(dst + s * (G::NT * G::KT * 256)) =
          digits_to_half2(packed);
    }
  }
}

// One warp's unit of an emulated product: rows of m-tile mt, columns of
// n-tiles 2 p and 2 p + 1.  Writes C (FP64) into out[row * NC + col].
template <class G>
__device__ __forceinline__ void gemm_unit(int unit, const unsigned char* ops,
                                          uint32_t slices_s, const int* col_emax,
                                          double* out) {
  const int lane = threadIdx.x & 31;
  const int mt = unit / G::NT2;
  const int nt0 = 2 * (unit - mt * G::NT2);
  const bool two = nt0 + 1 < G::NT;
  const int* row_exp = reinterpret_cast<const int*>(ops + G::DIGITS);
  long long ghi[2][4], glo[2][4];
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int c = 0; c < 4; ++c) ghi[q][c] = glo[q][c] = 0;

#pragma unroll 1
  for (int l = 2; l <= kLevels; ++l) {
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    const int ilo = l - kS > 1 ? l - kS : 1;
    const int ihi = l - 1 < kS ? l - 1 : kS;
#pragma unroll 1
    for (int i = ilo; i <= ihi; ++i) {
      const int j = l - i;
      const unsigned char* ablk = ops + ((i - 1) * G::MT + mt) * G::KT * 256 + lane * 8;
      const uint32_t bblk = slices_s + (((j - 1) * G::NT + nt0) * G::KT) * 256 +
                            (lane & 15) * 16;
#pragma unroll
      for (int kt = 0; kt < G::KT; ++kt) {
        uint32_t afr[4];
        expand_a(*reinterpret_cast<const uint2*>(ablk + kt * 256), afr);
        uint32_t b0, b1;
        ldsm_x2(b0, b1, bblk + kt * 256);
        mma16816(acc[0], afr, b0, b1);
        if (two) {
          ldsm_x2(b0, b1, bblk + (G::KT + kt) * 256);
          mma16816(acc[1], afr, b0, b1);
        }
      }
    }
    const int sh = l <= 5 ? 7 * (5 - l) : 7 * (9 - l);
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const long long v =
            (long long)((unsigned long long)(long long)f32_exact_int(acc[q][c]) << sh);
        if (l <= 5) ghi[q][c] += v;
        else glo[q][c] += v;
      }
  }
  const int g = lane >> 2, tq = lane & 3;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    if (q == 1 && !two) break;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int row = mt * 16 + g + (c >= 2 ? 8 : 0);
      const int col = (nt0 + q) * 8 + 2 * tq + (c & 1);
      if (row < G::M && col < G::NC) {
        const double r = fma(i64_exact_double(glo[q][c]), 0x1p-28,
                             i64_exact_double(ghi[q][c]));
        out[row * G::NC + col] = r * pow2(row_exp[row] + col_emax[col] - 1022 - 31);
      }
    }
  }
}

}  // namespace tc

template <int N, int EQ, int MODE>
__global__ void __launch_bounds__(kBlock, 1) dg_rhs_tc_kernel(const RhsArgs a) {
  using P = tc::Plan<N, EQ>;
  constexpr int NP = P::NP, NFPT = P::NFPT, NF = P::NF, E = P::E;
  constexpr bool STAGE = (MODE & MODE_STAGE) != 0;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ int ops_ok;

  const int t = threadIdx.x;
  const int warp = t >> 5;
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

  const unsigned char* ops = smem + P::SM_OPS;
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

    // {{{ 3. volume data -> digit slices
    using G1 = typename P::G1;
    using G2 = typename P::G2;
    using GL = typename P::GL;
    constexpr int SL2 = P::HAS_G1 ? G1::SLICE_BYTES : 0;  // G2 slices after G1's
    if constexpr (EQ == DG_WAVE) {
      tc::split_columns<G1>(sR1, sExp, [&](int n, int k) {  // u of element n
        return sQ[(0 * E + n) * NP + k];
      });
      tc::split_columns<G2>(sR1 + SL2, sExp + P::NCOLS, [&](int n, int k) {
        const int r = k / NP, j = k - r * NP;  // (G v)_r of element n
        return sR2[(r * E + n) * NP + j];
      });
    } else if constexpr (EQ == DG_EULER) {
      tc::split_columns<G2>(sR1 + SL2, sExp + P::NCOLS, [&](int n, int k) {
        const int f = n / E, e = n - f * E;  // column (field, element)
        const int r = k / NP, j = k - r * NP;
        return sR2[((f * 3 + r) * E + e) * NP + j];
      });
    } else {
      tc::split_columns<G1>(sR1, sExp, [&](int n, int k) {  // q_f of element e
        return sQ[n * NP + k];
      });
    }
    __syncthreads();
    // }}}

    // {{{ 4. volume products (tensor cores) -> R2 (FP64)
    {
      constexpr int U1 = P::HAS_G1 ? G1::UNITS : 0;
      constexpr int U2 = P::HAS_G2 ? G2::UNITS : 0;
      double* out1 = sR2;
      double* out2 = sR2 + P::OUT_G1;
      // One call site per loop: G1 units from warp 0 up, G2 units from the
      // last warp down, so the two products run side by side.  (With both
      // inlined calls in one loop body, selected per unit, the G1 outputs of
      // the order-3 wave kernel were lost in code generation.)
      constexpr int NW = kBlock / 32;
      if constexpr (P::HAS_G1)
        for (int u = warp; u < U1; u += NW)
          tc::gemm_unit<G1>(u, ops + P::OPS_G1, sR1_s, sExp, out1);
      if constexpr (P::HAS_G2)
        for (int u = NW - 1 - warp; u < U2; u += NW)
          tc::gemm_unit<G2>(u, ops + P::OPS_G2, sR1_s + SL2, sExp + P::NCOLS, out2);
    }
    __syncthreads();
    // }}}

    // {{{ 5. volume term per node (registers)
    double vol[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) vol[k] = 0.0;
    if (active) {
      const double* G = sG + el * 9;
      if constexpr (EQ == DG_WAVE) {
        const double c = a.p0;
        const double* ur = sR2;                  // (3 Np) x E: row r Np + i
        const double* dv = sR2 + P::OUT_G1;      // Np x E
        const double u0 = ur[(0 * NP + i) * E + el], u1 = ur[(1 * NP + i) * E + el],
                     u2 = ur[(2 * NP + i) * E + el];
        vol[0] = -c * dv[i * E + el];
#pragma unroll
        for (int x = 0; x < 3; ++x)
          vol[1 + x] = -c * fma(G[0 * 3 + x], u0, fma(G[1 * 3 + x], u1, G[2 * 3 + x] * u2));
      } else if constexpr (EQ == DG_EULER) {
        const double* o = sR2 + P::OUT_G1;       // Np x (5 E)
#pragma unroll
        for (int k = 0; k < 5; ++k) vol[k] = o[i * (5 * E) + k * E + el];
      } else {
        const double* o = sR2;                   // (3 Np) x (6 E)
        auto dx = [&](int k, int x) {
          const double d0 = o[(0 * NP + i) * (6 * E) + k * E + el];
          const double d1 = o[(1 * NP + i) * (6 * E) + k * E + el];
          const double d2 = o[(2 * NP + i) * (6 * E) + k * E + el];
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

    // {{{ 6. face values of the tile -> R2, then digit slices
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
    // }}}

    // {{{ 7. LIFT product -> R2 after the face values
    double* sL = sR2 + NF * E * NFPT;            // Np x (NF E)
    for (int u = warp; u < GL::UNITS; u += kBlock / 32)
      tc::gemm_unit<GL>(u, ops + P::OPS_GL, sR1_s, sExp, sL);
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
