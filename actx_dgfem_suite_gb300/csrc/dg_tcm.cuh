// Mixed-precision RHS with the contractions on the tcgen05 tensor cores.
//
// The volume derivatives and LIFT of the mixed-precision path (FP32
// arithmetic, FP64 state) as tensor-core products per tile, with the roles
// of data and operator chosen for the tensor core's 128-row shape:
//
//   D (128 x Np) = X_V (128 x 3 Np) B_V^T + X_L (128 x 4 Nfp) B_L^T
//
// Each of the 128 rows of X is one (field c, element e) column of the tile's
// data.  X_V holds the metric-combined inputs w_{c,r}(j) of the three
// reference derivatives (r = 0, 1, 2; nodes j), X_L the field's lifted face
// values:
//   wave    w_{0,r} = -c (G v)_r,  w_{1+x,r} = -c G_{r x} u;
//   euler   w_{k,r} = sum_x G_{r x} F_{k x}(q);
//   maxwell w_{c,r} from E_t = curl H, H_t = -curl E, e.g.
//           w_{0,r} = G_{r 1} H_z - G_{r 2} H_y;
// B_V = [A_0 A_1 A_2] (A_r the reference derivative the equation uses) and
// B_L = LIFT, Np rows each.  D holds vol + lift of every output node
// directly: no per-node combination after the products.
//
// Exact accumulation.  Every row of X and of B is scaled by a power of two
// to 31-bit integers and written as four balanced base-256 digits
// (|d| <= 128, exact in FP16): x = 2^(E - 31) sum_i d_i 2^(24 - 8 i).  The ten
// digit-pair products with i + j <= 3 run as tcgen05.mma kind::f16 (M = 128,
// N = Np padded to 16, K = 16) into one FP32 tensor-memory accumulator per
// level l = i + j and phase; each level sum is an integer of magnitude at
// most 2^23 (FP32 holds integers exactly up to 2^24), so the tensor core adds
// it exactly whatever its internal rounding.  The fold
// recombines L_0 + 2^-8 L_1 + 2^-16 L_2 + 2^-24 L_3 with three
// round-to-nearest FP32 operations.  Row scaling with 31 bits keeps the
// entries of a row that are up to 2^7 below its maximum at FP32's 24-bit
// resolution (P4 operator rows span a factor 4-7 in rms), and the dropped
// pairs weigh 2^-32: the result carries the error of FP32 arithmetic,
// unbiased, where TF32 products accumulated by the tensor core lose accuracy
// with every accumulation step.
//
// 3xTF32 form (TF = true, variant 5).  Every value of X and B is split into
// x = hi + lo, both TF32 (cvt.rna; hi carries 11 significant bits, lo the
// next 11), and tcgen05.mma kind::tf32 (M = 128, N = NB, K = 8) forms
// hi hi in one accumulator and hi lo + lo hi in a second one (2^-11 smaller,
// so its own roundings do not matter); the epilogue adds the two.  No row
// scaling and no digit fold: the split is three instructions per value
// against ~30 for the four digits, the volume inputs are computed once and
// written straight into X, and there are 3 products per k-step instead of
// 10.  Its error is that of FP32 arithmetic with the tensor core's own
// accumulation order (FP32 partial sums, no exactness argument), so the
// bounded autotuner decides per plan whether it is admissible.
//
// Per tile of E = 128 / NF elements (8 elements x 4 pairs of nodes or face
// points per warp; a pair's digits are one 4-byte word per digit slice, and
// the 32 words a warp stores fall in 32 distinct banks):
//   0. (during the previous tile's LIFT products) the tile's metric and face
//      geometry converted once to FP32 in shared memory;
//   1. per node pair: the FP64 state (one 16-byte load where Np is even) ->
//      FP32 copy, (Euler: the pressure from the per-node table, which
//      dg_euler_pressure_f32_kernel fills by the FP64 recovery from total
//      energy), the inputs w -> row maxima (digits: shuffles + shared
//      atomics) or straight into X_V as TF32 pairs;
//   2. (digits) per node again: w -> digits of X_V;
//   3. L2 prefetch of the next tile's state rows and gather indices; one
//      thread issues the volume products (asynchronous, completion on an
//      mbarrier); meanwhile every thread evaluates the numerical flux of its
//      face points into registers (and their row maxima); after the volume
//      products have read X, X_L replaces it and the LIFT products run;
//   4. tcgen05.ld of the accumulators -> FP32 staging, then coalesced FP64
//      stores (RHS) or the fused low-storage RK stage.
// Waits on the mbarriers are bounded (DG_ERR_TIMEOUT instead of spinning).
//
// Flux formulas as in dg_rhs.cuh (wave.py:80-114, grudge's Euler LF flux
// with InviscidWallBC, MaxwellOperator alpha-flux with PEC).
#pragma once

#include <cuda_fp16.h>

#include "dg_tc.cuh"

namespace dg {
namespace tcm {

constexpr int r16(int x) { return (x + 15) & ~15; }
constexpr int p16(int b) { return (b + 15) & ~15; }
// row pitch (words) >= n with pitch % 8 == 4: a warp's 8 elements x 4 node
// pairs reach 16 distinct banks with one node of each pair (two lanes per bank)
constexpr int pitch_q(int n) { return ((n + 3) / 8) * 8 + 4; }
constexpr int pow2_cols(int c) {
  return c <= 32 ? 32 : c <= 64 ? 64 : c <= 128 ? 128 : c <= 256 ? 256 : 512;
}

constexpr int rup(int x, int m) { return (x + m - 1) / m * m; }

// Tile plan of the kernel.  TF = false: exact FP16 digit pairs (variant 4);
// TF = true: 3xTF32 products (variant 5; see dg_rhs_tcm_kernel).  ALT: the
// other CTA size for the same 128-row tile (variant 6), a tile shape the
// autotuner chooses: 128 threads where the default is 256 (orders 2-3: the
// same warps per SM spread over twice the tiles in flight, where shared
// memory allows), 256 where it is 128 or 512 (orders 1 and 4).
template <int N, int EQ, bool TF = false, bool ALT = false>
struct MPlan {
  static constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP, NFPT = Shape<N>::NFPT;
  static constexpr int NF = EqInfo<EQ>::NF;
  static constexpr int BASE_THREADS = N == 1 ? 128 : (N == 4 ? 512 : 256);
  static constexpr int THREADS = !ALT ? BASE_THREADS : (BASE_THREADS == 256 ? 128 : 256);
  static constexpr int MIN_BLOCKS = N == 4 ? 1 : (THREADS == 128 ? 4 : 2);
  static constexpr int E = 128 / NF;      // elements per tile
  static constexpr int NCOL = NF * E;     // rows of X in use (m = c E + e)
  static constexpr int NB = r16(NP);      // operator rows (MMA N)
  // X_V column of derivative r and node j: k = r NPP + j, NPP = Np rounded up
  // to even, so the two nodes a lane writes share one 4-byte word
  static constexpr int NPP = NP + (NP & 1);
  // operand elements: FP16 digits (2 bytes) or TF32 parts (4 bytes); a
  // core-matrix row holds 16 bytes (KG elements), one MMA consumes two core
  // matrices along K (KSTEP = 16 FP16 or 8 TF32 values)
  static constexpr int ESZ = TF ? 4 : 2, KG = 16 / ESZ, KSTEP = 2 * KG;
  static constexpr int KV = rup(3 * NPP, KSTEP), KL = rup(NFPT, KSTEP);
  // K-major, no swizzle: element (m, k) of a slice at
  //   (m / 8) SBO + (k / KG) 128 + (m % 8) 16 + (k % KG) ESZ bytes
  static constexpr int SBO_V = (KV / KG) * 128, SBO_L = (KL / KG) * 128;
  static constexpr int A_SLICE_V = 16 * SBO_V, A_SLICE_L = 16 * SBO_L;
  static constexpr int NDIG = TF ? 2 : 4;  // slices per value: digits, or TF32 hi / lo
  static constexpr int A_BYTES = NDIG * (A_SLICE_V > A_SLICE_L ? A_SLICE_V : A_SLICE_L);
  // operator block (global and shared): B_V slices | B_L slices | (digits
  // only) FP32 row scales 2^e of B_V | of B_L (|B_ik| < 2^e) | int32 face nodes
  static constexpr int B_SLICE_V = (NB / 8) * SBO_V, B_SLICE_L = (NB / 8) * SBO_L;
  static constexpr int OPS_V = 0, OPS_L = NDIG * B_SLICE_V;
  static constexpr int OPS_EV = OPS_L + NDIG * B_SLICE_L;
  static constexpr int OPS_EL = OPS_EV + (TF ? 0 : NB * 4);
  static constexpr int OPS_FN = OPS_EL + (TF ? 0 : NB * 4);
  static constexpr int OPS_BYTES = OPS_FN + p16(NFPT * 4);
  static constexpr int QP = pitch_q(NP);  // FP32 state rows
  static constexpr int OP = NP | 1;       // FP32 result rows (odd pitch)
  static constexpr int SM_A = 0;
  static constexpr int SM_OPS = SM_A + A_BYTES;
  static constexpr int SM_Q = SM_OPS + OPS_BYTES;
  // FP32 metric (9 values at a pitch of 12 per element) and face geometry
  // (n_x, n_y, n_z, sJ/J per face), converted once per tile
  static constexpr int SM_G = SM_Q + p16(NF * E * QP * 4);
  static constexpr int SM_FG = SM_G + p16(12 * E * 4);
  // FP32 results.  TF32: staged over X once the LIFT products have read it
  // (X's padding then holds finite FP32 values, harmless against the zero
  // operator columns); digits: a region of their own, since FP32 bit
  // patterns read as FP16 digits may be infinite or NaN in X's padding
  static constexpr int SM_OUT = TF ? SM_A : SM_FG + p16(16 * E * 4);
  // digits only: row maxima [2 tiles][2 phases][128]
  static constexpr int SM_RMAX = TF ? SM_FG + p16(16 * E * 4) : SM_OUT + p16(NCOL * OP * 4);
  static constexpr int SM_P = SM_RMAX + (TF ? 0 : 4 * 128 * 4);  // euler: node pressures
  static constexpr int SMEM_BYTES = SM_P + (EQ == DG_EULER ? p16(E * NP * 4) : 0);
  // accumulators of the volume phase, then of the LIFT phase: levels 0..3
  // (digits), or hi x hi and the two cross terms (TF32)
  static constexpr int NACC = TF ? 2 : 4;
  static constexpr int ACC_L = NACC * NB;
  static constexpr int TMEM_COLS = pow2_cols(2 * NACC * NB);
  // instruction descriptor: D FP32, A and B FP16 (0) or TF32 (2), both
  // K-major, N, M = 128
  static constexpr uint32_t IDESC = (1u << 4) | (TF ? (2u << 7) | (2u << 10) : 0u) |
                                    ((uint32_t)(NB >> 3) << 17) | (8u << 24);
  static_assert(NCOL <= 128, "one 128-row product per tile");
  static_assert(NB >= 16 && NB <= 256, "MMA N range");
  static_assert(TF || (KV <= 128 && KL <= 128),
                "level sums (4 pairs) of at most 2^23 need K <= 128");
  static_assert(TMEM_COLS <= 512, "accumulators fit in tensor memory");
  static_assert(NCOL * OP * 4 <= A_BYTES, "result staging fits over X");
  static_assert(SMEM_BYTES <= 227 * 1024, "tile does not fit in shared memory");
};

// FP32 copies of the equation constants, converted once per CTA (on the
// integer ALU: conversions that touch FP64 issue at GB300's FP64 rate)
struct FluxConsts {
  float p0;      // wave speed c / gamma / maxwell alpha
  float z, y;    // maxwell impedance and admittance
  float ce, ch;  // maxwell flux factors -1/(2z), 1/(2y)
  float ie, im;  // maxwell 1/eps, 1/mu
};

__device__ __forceinline__ FluxConsts flux_consts(const RhsArgs& a) {
  FluxConsts f;
  f.p0 = d2f_alu(a.p0);
  f.z = d2f_alu(a.k[0]);
  f.y = d2f_alu(a.k[1]);
  f.ce = d2f_alu(a.k[2]);
  f.ch = d2f_alu(a.k[3]);
  f.ie = d2f_alu(a.k[4]);
  f.im = d2f_alu(a.k[5]);
  return f;
}

// byte offset of element (m, k) in a K-major slice of KG elements per
// 16-byte core-matrix row
template <int KG = 8>
__device__ __forceinline__ int kmajor_off(int m, int k, int sbo) {
  return (m >> 3) * sbo + (k / KG) * 128 + (m & 7) * 16 + (k % KG) * (16 / KG);
}

// x -> TF32 (round to nearest, ties away from zero), as a bit pattern
__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// two values of one row at columns k, k + 1 (k even: one 8-byte word per
// slice) -> x = hi + lo, both TF32, hi in the first slice, lo in the second
__device__ __forceinline__ void put_tf32x2(unsigned char* base, int slice, int off, float x0,
                                           float x1) {
  const uint32_t h0 = tf32_bits(x0), h1 = tf32_bits(x1);
  const uint32_t l0 = tf32_bits(x0 - __uint_as_float(h0));
  const uint32_t l1 = tf32_bits(x1 - __uint_as_float(h1));
  *reinterpret_cast<uint2*>(base + off) = make_uint2(h0, h1);
  *reinterpret_cast<uint2*>(base + slice + off) = make_uint2(l0, l1);
}

// zeros at columns k, k + 1 (k even) of one row in every slice of X
template <bool TF>
__device__ __forceinline__ void zero_pair(unsigned char* base, int slice, int off) {
  if constexpr (TF) {
    *reinterpret_cast<uint2*>(base + off) = make_uint2(0u, 0u);
    *reinterpret_cast<uint2*>(base + slice + off) = make_uint2(0u, 0u);
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) *reinterpret_cast<uint32_t*>(base + i * slice + off) = 0u;
  }
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
      ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// One phase of 3xTF32 products: per k-step of 8, hi x hi into acc and
// hi x lo + lo x hi into acc + NB (the cross terms, 2^-11 smaller, in an
// accumulator of their own so that they do not lengthen the main sum's
// chain of roundings).
template <int K, int SBO, int A_SLICE, int B_SLICE, int NB>
__device__ __forceinline__ void issue_phase_tf32(uint32_t a_s, uint32_t b_s, uint32_t acc,
                                                 uint32_t idesc) {
  tc::tc_fence_after();
#pragma unroll 1
  for (int kt = 0; kt < K / 8; ++kt) {
    const uint32_t ka = a_s + kt * 256, kb = b_s + kt * 256;
    const uint64_t ah = tc::smem_desc(ka, 128, SBO), al = tc::smem_desc(ka + A_SLICE, 128, SBO);
    const uint64_t bh = tc::smem_desc(kb, 128, SBO), bl = tc::smem_desc(kb + B_SLICE, 128, SBO);
    const uint32_t more = kt > 0 ? 1u : 0u;
    mma_tf32(acc, ah, bh, idesc, more);
    mma_tf32(acc + (uint32_t)NB, ah, bl, idesc, more);
    mma_tf32(acc + (uint32_t)NB, al, bh, idesc, 1u);
  }
}

// 2^s as a float for s in [-126, 127]
__device__ __forceinline__ float pow2f(int s) {
  s = s < -126 ? -126 : (s > 127 ? 127 : s);
  return __uint_as_float((uint32_t)(s + 127) << 23);
}

// biased exponent of a row maximum (float bits of |x|), clamped so that the
// scale 2^(157 - e) stays a normal float: |x| < 2^(e - 126)
__device__ __forceinline__ int row_exp_bits(uint32_t maxbits) {
  const int e = (int)(maxbits >> 23);
  return e < 30 ? 30 : e;
}

// x (|x| < 2^(e - 126)) -> four digits of v = round(x 2^(157 - e)),
// |v| <= 2^31, most significant first.  FP32 arithmetic is exact here: v has
// at most 24 significant bits, and every remainder is a multiple of ulp(v)
// below 2^24 ulp(v).
__device__ __forceinline__ void digits4(float x, float scale, float* d) {
  const float v = rintf(x * scale);
  d[0] = rintf(v * 0x1p-24f);
  const float r1 = fmaf(-d[0], 0x1p24f, v);
  d[1] = rintf(r1 * 0x1p-16f);
  const float r2 = fmaf(-d[1], 65536.f, r1);
  d[2] = rintf(r2 * 0x1p-8f);
  d[3] = fmaf(-d[2], 256.f, r2);
}

// two values of one row at columns k, k + 1 (k even: one 4-byte word per
// slice) -> their FP16 digits in the four slices at byte offset `off`
__device__ __forceinline__ void put_digits2(unsigned char* base, int slice, int off,
                                            float x0, float x1, int e) {
  const float scale = __uint_as_float((uint32_t)(284 - e) << 23);
  float a[4], b[4];
  digits4(x0, scale, a);
  digits4(x1, scale, b);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __half2 h = __floats2half2_rn(a[i], b[i]);  // low half: column k
    *reinterpret_cast<__half2*>(base + i * slice + off) = h;
  }
}

// max over the four lanes of a warp that share lane & 7 (elements; the
// lanes differ in their pair of nodes or face points), then one shared
// atomic per element row
__device__ __forceinline__ void row_max(unsigned* rmax, int m, float a, bool lead) {
  a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, 8));
  a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, 16));
  if (lead) atomicMax(rmax + m, __float_as_uint(a));
}

// One phase: per k-step of 16 the ten digit pairs (i, j), i + j <= 3, into the
// level accumulators acc + (i + j) NB.
template <int K, int SBO, int A_SLICE, int B_SLICE, int NB>
__device__ __forceinline__ void issue_phase(uint32_t a_s, uint32_t b_s, uint32_t acc,
                                            uint32_t idesc) {
  tc::tc_fence_after();
#pragma unroll 1
  for (int kt = 0; kt < K / 16; ++kt) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4 - i; ++j) {
        const uint64_t da = tc::smem_desc(a_s + i * A_SLICE + kt * 256, 128, SBO);
        const uint64_t db = tc::smem_desc(b_s + j * B_SLICE + kt * 256, 128, SBO);
        // the first product of each level (kt = 0, i = 0) starts it
        tc::tc_mma(acc + (uint32_t)((i + j) * NB), da, db, idesc,
                   (kt == 0 && i == 0) ? 0u : 1u);
      }
  }
}

// L_0 + 2^-8 L_1 + 2^-16 L_2 + 2^-24 L_3 (exact integer level sums), three
// roundings, smallest terms first
__device__ __forceinline__ float levels4(const uint32_t* l, int jj) {
  const float t2 = fmaf(__uint_as_float(l[24 + jj]), 0x1p-8f, __uint_as_float(l[16 + jj]));
  const float t1 = fmaf(t2, 0x1p-8f, __uint_as_float(l[8 + jj]));
  return fmaf(t1, 0x1p-8f, __uint_as_float(l[jj]));
}

// Numerical flux of one face point in FP32 (FP64 exterior state; Euler:
// interior and exterior pressures from the per-node table); out[c] = the
// lifted face value of field c.
template <int EQ, int NF>
__device__ __forceinline__ void face_point_flux(const FluxConsts& fc, const float* qi,
                                                const double* qed, bool bdry, float nx,
                                                float ny, float nz, float scale,
                                                float pi, float pe, float* out) {
  float qe[NF];
  if (!bdry) {
#pragma unroll
    for (int k = 0; k < NF; ++k) qe[k] = d2f_alu(qed[k]);
  }
  if constexpr (EQ == DG_WAVE) {
    if (bdry) {  // Dirichlet mirror: exterior (-u, v)
      qe[0] = -qi[0];
      qe[1] = qi[1];
      qe[2] = qi[2];
      qe[3] = qi[3];
    }
    const float c = fc.p0;
    const float vavg_n = 0.5f * (qi[1] + qe[1]) * nx + 0.5f * (qi[2] + qe[2]) * ny +
                         0.5f * (qi[3] + qe[3]) * nz;
    const float uavg = 0.5f * (qi[0] + qe[0]);
    const float vjump = (qe[1] - qi[1]) * nx + (qe[2] - qi[2]) * ny + (qe[3] - qi[3]) * nz;
    const float fu = c * (vavg_n + 0.5f * (qe[0] - qi[0]));
    const float fv = c * (uavg + 0.5f * vjump);
    out[0] = scale * fu;
    out[1] = scale * (fv * nx);
    out[2] = scale * (fv * ny);
    out[3] = scale * (fv * nz);
  } else if constexpr (EQ == DG_EULER) {
    const float gamma = fc.p0;
    if (bdry) {  // the wall mirror keeps rho, |m| and E (so the pressure)
      const float mn = qi[2] * nx + qi[3] * ny + qi[4] * nz;
      qe[0] = qi[0];
      qe[1] = qi[1];
      qe[2] = qi[2] - 2.f * nx * mn;
      qe[3] = qi[3] - 2.f * ny * mn;
      qe[4] = qi[4] - 2.f * nz * mn;
    }
    float fn_i[5], fn_e[5], lam_i, lam_e;
    auto side = [&](const float* q, float p, float* fn, float& lam) {
      const float rinv = 1.f / q[0];
      const float ux = q[2] * rinv, uy = q[3] * rinv, uz = q[4] * rinv;
      const float un = ux * nx + uy * ny + uz * nz;
      fn[0] = q[2] * nx + q[3] * ny + q[4] * nz;
      fn[1] = un * (q[1] + p);
      fn[2] = q[2] * un + p * nx;
      fn[3] = q[3] * un + p * ny;
      fn[4] = q[4] * un + p * nz;
      lam = sqrtf(ux * ux + uy * uy + uz * uz) + sqrtf(gamma * (p * rinv));
    };
    side(qi, pi, fn_i, lam_i);
    side(qe, bdry ? pi : pe, fn_e, lam_e);
    const float lam = fmaxf(lam_i, lam_e);
    const float nn = nx * nx + ny * ny + nz * nz;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const float fk = 0.5f * (fn_i[k] + fn_e[k]) - 0.5f * lam * (qe[k] - qi[k]) * nn;
      out[k] = -scale * fk;
    }
  } else {  // DG_MAXWELL
    if (bdry) {  // PEC: exterior (-E, H)
      qe[0] = -qi[0];
      qe[1] = -qi[1];
      qe[2] = -qi[2];
      qe[3] = qi[3];
      qe[4] = qi[4];
      qe[5] = qi[5];
    }
    const float alpha = fc.p0;
    const float z = fc.z, y = fc.y;
    const float je[3] = {qe[0] - qi[0], qe[1] - qi[1], qe[2] - qi[2]};
    const float jh[3] = {qe[3] - qi[3], qe[4] - qi[4], qe[5] - qi[5]};
    const float n[3] = {nx, ny, nz};
    auto cross = [](const float* a_, const float* b_, float* c_) {
      c_[0] = a_[1] * b_[2] - a_[2] * b_[1];
      c_[1] = a_[2] * b_[0] - a_[0] * b_[2];
      c_[2] = a_[0] * b_[1] - a_[1] * b_[0];
    };
    float nxe[3], nxh[3], te[3], th[3], fe[3], fh[3];
    cross(n, je, nxe);
    cross(n, jh, nxh);
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      te[x] = z * jh[x] - alpha * nxe[x];
      th[x] = y * je[x] + alpha * nxh[x];
    }
    cross(n, te, fe);
    cross(n, th, fh);
    const float ce = fc.ce, ch = fc.ch;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      out[x] = -scale * (ce * fe[x]);
      out[3 + x] = -scale * (ch * fh[x]);
    }
  }
}

}  // namespace tcm

template <int N, int EQ, int MODE, bool TF = false, bool ALT = false>
__global__ void __launch_bounds__(tcm::MPlan<N, EQ, TF, ALT>::THREADS,
                                  tcm::MPlan<N, EQ, TF, ALT>::MIN_BLOCKS)
    dg_rhs_tcm_kernel(const RhsArgs a) {
  using P = tcm::MPlan<N, EQ, TF, ALT>;
  constexpr int NP = P::NP, NFP = P::NFP, NFPT = P::NFPT, NF = P::NF, E = P::E;
  constexpr int QP = P::QP, OP = P::OP, NB = P::NB, THREADS = P::THREADS, KG = P::KG;
  constexpr bool STAGE = (MODE & MODE_STAGE) != 0;
  constexpr int NWARP = THREADS / 32;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint64_t mma_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int ops_ok;

  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  unsigned char* sA = smem + P::SM_A;
  const int* sFN = reinterpret_cast<const int*>(smem + P::SM_OPS + P::OPS_FN);
  const float* sEV = reinterpret_cast<const float*>(smem + P::SM_OPS + P::OPS_EV);
  const float* sEL = reinterpret_cast<const float*>(smem + P::SM_OPS + P::OPS_EL);
  float* sq = reinterpret_cast<float*>(smem + P::SM_Q);
  float* sG = reinterpret_cast<float*>(smem + P::SM_G);
  float* sFG = reinterpret_cast<float*>(smem + P::SM_FG);
  float* sOut = reinterpret_cast<float*>(smem + P::SM_OUT);
  unsigned* sRmax = reinterpret_cast<unsigned*>(smem + P::SM_RMAX);
  float* sP = reinterpret_cast<float*>(smem + P::SM_P);  // euler: node pressures
  const tcm::FluxConsts fc = tcm::flux_consts(a);
  if (t == 0) {
    mbar_init(&bar, 1);
    mbar_init(&mma_bar, 1);
    mbar_arrive_expect_tx(&bar, a.ops_bytes);
    bulk_g2s(smem + P::SM_OPS, a.ops, a.ops_bytes, &bar);
    const bool ok = mbar_wait_bounded(&bar, 0);
    if (!ok) {
      raise_status(a.status, DG_ERR_TIMEOUT);
      mbar_wait_bounded(&bar, 0);
    }
    ops_ok = ok ? 1 : 0;
  }
  // digit padding (k past 3 Np or 4 Nfp, rows past NF E) meets zero operator
  // columns or unused rows; it must hold finite values, so clear X once
  for (int idx = t; idx < P::A_BYTES / 16; idx += THREADS)
    reinterpret_cast<uint4*>(sA)[idx] = make_uint4(0u, 0u, 0u, 0u);
  if constexpr (!TF)
    for (int idx = t; idx < 4 * 128; idx += THREADS) sRmax[idx] = 0u;
  __syncthreads();
  if (!ops_ok) return;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(&tmem_base)), "r"(P::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_base;
  AsyncLedger<1> led;  // barrier 0: the tensor-core products
  led.init();
  const uint32_t a_s = smem_u32(sA);
  const uint32_t b_s = smem_u32(smem + P::SM_OPS);

  const int64_t nel = a.nel;
  const int64_t nelnp = nel * NP;
  const int64_t ntiles = (nel + E - 1) / E;
  // warp items: 8 elements x 4 pairs of nodes (face points); a lane takes
  // nodes (face points) 2 p and 2 p + 1
  constexpr int NPP = P::NPP;
  constexpr int EG = (E + 7) / 8, JG = (NPP / 2 + 3) / 4, FG = (NFPT / 2 + 3) / 4;
  constexpr int FROUNDS = (EG * FG + NWARP - 1) / NWARP;  // face items per thread
  static_assert(NFPT % 2 == 0, "face points come in pairs");

  // bounded wait for the products; false if it gave up
  auto wait_mma = [&]() -> bool {
    const bool ok = led.complete(0, mbar_wait_bounded(&mma_bar, led.phase[0]));
    if (!ok) raise_status(a.status, DG_ERR_TIMEOUT);
    tc::tc_fence_after();
    return ok;
  };

  // metric-combined volume inputs of node j of element e from FP32 values
  auto vol_inputs = [&](const float* qf, const float* G, float p, float rinv, float (*w)[3]) {
    if constexpr (EQ == DG_WAVE) {
      const float c = fc.p0;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        w[0][r] = -c * fmaf(G[r * 3 + 0], qf[1], fmaf(G[r * 3 + 1], qf[2], G[r * 3 + 2] * qf[3]));
#pragma unroll
        for (int x = 0; x < 3; ++x) w[1 + x][r] = -c * (G[r * 3 + x] * qf[0]);
      }
    } else if constexpr (EQ == DG_EULER) {
      const float u3[3] = {qf[2] * rinv, qf[3] * rinv, qf[4] * rinv};
      float F[5][3];
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        F[0][x] = qf[2 + x];
        F[1][x] = u3[x] * (qf[1] + p);
#pragma unroll
        for (int c = 0; c < 3; ++c) F[2 + c][x] = qf[2 + c] * u3[x] + (c == x ? p : 0.f);
      }
#pragma unroll
      for (int k = 0; k < 5; ++k)
#pragma unroll
        for (int r = 0; r < 3; ++r)
          w[k][r] = fmaf(G[r * 3 + 0], F[k][0], fmaf(G[r * 3 + 1], F[k][1], G[r * 3 + 2] * F[k][2]));
    } else {  // maxwell: E_t = curl H, H_t = -curl E (strong derivatives)
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const float g0 = G[r * 3 + 0], g1 = G[r * 3 + 1], g2 = G[r * 3 + 2];
        w[0][r] = g1 * qf[5] - g2 * qf[4];
        w[1][r] = g2 * qf[3] - g0 * qf[5];
        w[2][r] = g0 * qf[4] - g1 * qf[3];
        w[3][r] = g2 * qf[1] - g1 * qf[2];
        w[4][r] = g0 * qf[2] - g2 * qf[0];
        w[5][r] = g1 * qf[0] - g0 * qf[1];
      }
    }
  };

  // a tile's metric and face geometry in FP32 (coalesced loads); the first
  // tile's here, every further tile's while the previous tile's LIFT
  // products run
  auto stage_geometry = [&](int64_t tile) {
    const int64_t g0 = tile * E;
    const int cnt = (nel - g0) < (int64_t)E ? (int)(nel - g0) : E;
    for (int idx = t; idx < 9 * E; idx += THREADS) {
      const int e = idx / 9;
      sG[e * 12 + (idx - e * 9)] = e < cnt ? d2f_alu(__ldg(a.metric + g0 * 9 + idx)) : 0.f;
    }
    for (int idx = t; idx < 16 * E; idx += THREADS)
      sFG[idx] = idx < 16 * cnt ? d2f_alu(__ldg(a.face_geom + g0 * 16 + idx)) : 0.f;
  };
  if (blockIdx.x < ntiles) stage_geometry(blockIdx.x);
  __syncthreads();
  // the next tile's state rows and gather indices into L2 (prefetch hints on
  // addresses inside the arrays), so that its phase-1 and face loads wait for
  // L2 rather than HBM
  auto prefetch_next = [&](int64_t nt) {
    const int64_t g0 = nt * E;
    const int cnt = (nel - g0) < (int64_t)E ? (int)(nel - g0) : E;
    const int qlines = (cnt * NP * 8 + 127) / 128;
    const int glines = (cnt * NFPT * 4 + 127) / 128;
    for (int idx = t; idx < NF * qlines + glines; idx += THREADS) {
      const char* ptr;
      if (idx < NF * qlines) {
        const int k = idx / qlines, l = idx - k * qlines;
        ptr = reinterpret_cast<const char*>(a.q + k * nelnp + g0 * NP) + l * 128;
      } else {
        ptr = reinterpret_cast<const char*>(a.gather + g0 * NFPT) + (idx - NF * qlines) * 128;
      }
      asm volatile("prefetch.global.L2 [%0];" ::"l"(ptr));
    }
  };

  // X's padding columns (k past 3 NPP, or past 4 Nfp) meet zero operator
  // columns; they are rewritten with zeros every tile, because X shares its
  // bytes with the other phase's layout (and, for 3xTF32, with the previous
  // tile's staged results): a NaN left there would reach other elements
  auto zero_pad_v = [&]() {
    constexpr int PADV = (P::KV - 3 * NPP) / 2;
    for (int idx = t; idx < 128 * PADV; idx += THREADS) {
      const int m = idx / PADV, c = idx - m * PADV;
      tcm::zero_pair<TF>(sA, P::A_SLICE_V, tcm::kmajor_off<KG>(m, 3 * NPP + 2 * c, P::SBO_V));
    }
  };
  auto zero_pad_l = [&]() {
    constexpr int PADL = (P::KL - NFPT) / 2;
    for (int idx = t; idx < 128 * PADL; idx += THREADS) {
      const int m = idx / PADL, c = idx - m * PADL;
      tcm::zero_pair<TF>(sA, P::A_SLICE_L, tcm::kmajor_off<KG>(m, NFPT + 2 * c, P::SBO_L));
    }
  };

  int it = 0;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int64_t e0 = tile * E;
    const int ecount = (nel - e0) < (int64_t)E ? (int)(nel - e0) : E;
    unsigned* rmaxV = sRmax + (it & 1) * 256;  // this tile's row maxima
    unsigned* rmaxL = rmaxV + 128;
    if constexpr (!TF) {  // the other buffer was last read before the previous tile's final barrier
      unsigned* other = sRmax + ((it + 1) & 1) * 256;
      for (int idx = t; idx < 256; idx += THREADS) other[idx] = 0u;
    }
    const bool pair_loads = (NP % 2 == 0) && ((reinterpret_cast<uintptr_t>(a.q) & 15u) == 0u);

    // {{{ 1. state -> FP32 copies, volume inputs -> row maxima (digits) or
    //        straight into X_V as TF32 pairs
    for (int u = warp; u < EG * JG; u += NWARP) {
      const int e = (u % EG) * 8 + (lane & 7);
      const int j0 = 2 * ((u / EG) * 4 + (lane >> 3));
      const bool ein = e < E;
      float G[12];
      {
        const float4* g4 = reinterpret_cast<const float4*>(sG + (ein ? e : 0) * 12);
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          const float4 v = g4[x];
          G[4 * x] = v.x;
          G[4 * x + 1] = v.y;
          G[4 * x + 2] = v.z;
          G[4 * x + 3] = v.w;
        }
      }
      // both nodes' FP64 state as 16-byte loads (a node past Np or an element
      // past the mesh reads the neutral state rho = 1, else 0)
      [[maybe_unused]] double2 qpair[NF];
      if constexpr (NP % 2 == 0) {
        if (pair_loads) {
          const bool vp = ein && j0 < NP && e < ecount;
          const int64_t g0 = (e0 + e) * NP + j0;
#pragma unroll
          for (int k = 0; k < NF; ++k)
            qpair[k] = vp ? __ldg(reinterpret_cast<const double2*>(a.q + k * nelnp + g0))
                          : make_double2(k == 0 ? 1.0 : 0.0, k == 0 ? 1.0 : 0.0);
        }
      }
      float m[NF];
#pragma unroll
      for (int c = 0; c < NF; ++c) m[c] = 0.f;
      [[maybe_unused]] float wt[2][NF][3];  // TF32: both nodes' inputs
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int j = j0 + h;
        const bool item = ein && j < NP;
        const bool valid = item && e < ecount;
        const int64_t gnode = (e0 + e) * NP + j;
        float qf[NF];
        float p = 0.f, rinv = 1.f;
#pragma unroll
        for (int k = 0; k < NF; ++k) {
          double qd;
          if constexpr (NP % 2 == 0)
            qd = pair_loads ? (h == 0 ? qpair[k].x : qpair[k].y)
                            : (valid ? __ldg(a.q + k * nelnp + gnode) : (k == 0 ? 1.0 : 0.0));
          else
            qd = valid ? __ldg(a.q + k * nelnp + gnode) : (k == 0 ? 1.0 : 0.0);
          qf[k] = d2f_alu(qd);
          if (item) sq[(k * E + e) * QP + j] = qf[k];
        }
        if constexpr (EQ == DG_EULER) {  // pressure table: FP64 recovery once per node
          p = valid ? __ldg(a.pres + gnode) : 0.f;
          rinv = __frcp_rn(qf[0]);
          if (item) sP[e * NP + j] = p;
        }
        float w[NF][3];
        vol_inputs(qf, G, p, rinv, w);
        if constexpr (TF) {  // a node past Np is the zero padding column
#pragma unroll
          for (int c = 0; c < NF; ++c)
#pragma unroll
            for (int r = 0; r < 3; ++r) wt[h][c][r] = item ? w[c][r] : 0.f;
        } else if (item) {
#pragma unroll
          for (int c = 0; c < NF; ++c)
            m[c] = fmaxf(m[c], fmaxf(fabsf(w[c][0]), fmaxf(fabsf(w[c][1]), fabsf(w[c][2]))));
        }
      }
      if constexpr (TF) {
        if (ein && j0 < NP) {
#pragma unroll
          for (int c = 0; c < NF; ++c)
#pragma unroll
            for (int r = 0; r < 3; ++r)
              tcm::put_tf32x2(sA, P::A_SLICE_V,
                              tcm::kmajor_off<KG>(c * E + e, r * NPP + j0, P::SBO_V),
                              wt[0][c][r], wt[1][c][r]);
        }
      } else {
#pragma unroll
        for (int c = 0; c < NF; ++c)
          tcm::row_max(rmaxV, c * E + (ein ? e : 0), m[c], (lane >> 3) == 0 && ein);
      }
    }
    if constexpr (TF) {
      zero_pad_v();
      tc::fence_async_smem();
    }
    __syncthreads();
    // }}}

    // {{{ 2. (digits) volume inputs -> digits of X_V (node pairs; a node past
    //        Np is the zero padding column)
    for (int u = warp; u < (TF ? 0 : EG * JG); u += NWARP) {
      const int e = (u % EG) * 8 + (lane & 7);
      const int j0 = 2 * ((u / EG) * 4 + (lane >> 3));
      if (e >= E || j0 >= NP) continue;
      const bool two = j0 + 1 < NP;
      float w0[NF][3], w1[NF][3];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int j = two ? j0 + h : j0;
        float qf[NF];
#pragma unroll
        for (int k = 0; k < NF; ++k) qf[k] = sq[(k * E + e) * QP + j];
        float p = 0.f, rinv = 1.f;
        if constexpr (EQ == DG_EULER) {
          p = sP[e * NP + j];
          rinv = __frcp_rn(qf[0]);
        }
        vol_inputs(qf, sG + e * 12, p, rinv, h == 0 ? w0 : w1);
      }
#pragma unroll
      for (int c = 0; c < NF; ++c) {
        const int m = c * E + e;
        const int ex = tcm::row_exp_bits(rmaxV[m]);
#pragma unroll
        for (int r = 0; r < 3; ++r)
          tcm::put_digits2(sA, P::A_SLICE_V, tcm::kmajor_off(m, r * NPP + j0, P::SBO_V),
                           w0[c][r], two ? w1[c][r] : 0.f, ex);
      }
    }
    if constexpr (!TF) {
      zero_pad_v();
      tc::fence_async_smem();
      __syncthreads();
    }
    // }}}

    // {{{ 3. volume products (one thread); face fluxes (registers) and their
    //        row maxima; then X_L and the LIFT products
    if (tile + gridDim.x < ntiles) prefetch_next(tile + gridDim.x);
    if (t == 0) {
      if constexpr (TF)
        tcm::issue_phase_tf32<P::KV, P::SBO_V, P::A_SLICE_V, P::B_SLICE_V, NB>(
            a_s, b_s + P::OPS_V, tmem, P::IDESC);
      else
        tcm::issue_phase<P::KV, P::SBO_V, P::A_SLICE_V, P::B_SLICE_V, NB>(
            a_s, b_s + P::OPS_V, tmem, P::IDESC);
      tc::tc_commit(&mma_bar);
      led.issue(0);
    }
    float fv[FROUNDS][2][NF];
    int fm[FROUNDS];  // e | fj0 << 8 (fj0 even), or -1
#pragma unroll
    for (int rd = 0; rd < FROUNDS; ++rd) {
      fm[rd] = -1;
      const int u = warp + rd * NWARP;
      const int e = (u % EG) * 8 + (lane & 7);
      const int fj0 = 2 * ((u / EG) * 4 + (lane >> 3));
      const bool item = u < EG * FG && e < E && fj0 < NFPT;
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int c = 0; c < NF; ++c) fv[rd][h][c] = 0.f;
      if (item && e < ecount) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int fj = fj0 + h;
          const int f = fj / NFP;
          const int node = sFN[fj];
          const uint32_t g = __ldg(a.gather + (e0 + e) * NFPT + fj);
          const bool bdry = (g >> 31) != 0u;
          uint32_t gi = g & 0x7fffffffu;
          if (gi >= (uint32_t)nelnp) {  // never read out of bounds
            raise_status(a.status, DG_ERR_INDEX);
            gi = (uint32_t)((e0 + e) * NP + node);
          }
          const float4 fg = *reinterpret_cast<const float4*>(sFG + (e * 4 + f) * 4);
          const float nx = fg.x, ny = fg.y, nz = fg.z, scale = fg.w;
          float qi[NF];
          double qed[NF];
#pragma unroll
          for (int k = 0; k < NF; ++k) {
            qi[k] = sq[(k * E + e) * QP + node];
            qed[k] = bdry ? 0.0 : __ldg(a.q + k * nelnp + gi);
          }
          float pi = 0.f, pe = 0.f;
          if constexpr (EQ == DG_EULER) {
            pi = sP[e * NP + node];
            pe = bdry ? pi : __ldg(a.pres + gi);
          }
          tcm::face_point_flux<EQ, NF>(fc, qi, qed, bdry, nx, ny, nz, scale, pi, pe,
                                       fv[rd][h]);
        }
        fm[rd] = e | (fj0 << 8);
      }
      if (!TF && u < EG * FG) {  // warp-uniform: every lane joins the shuffles
#pragma unroll
        for (int c = 0; c < NF; ++c)
          tcm::row_max(rmaxL, c * E + (e < E ? e : 0),
                       fmaxf(fabsf(fv[rd][0][c]), fabsf(fv[rd][1][c])),
                       (lane >> 3) == 0 && e < E);
      }
    }
    const bool vol_ok = wait_mma();        // the volume products have read X
    if (__syncthreads_or(!vol_ok)) break;  // (and the row maxima of X_L are complete)
#pragma unroll
    for (int rd = 0; rd < FROUNDS; ++rd) {
      if (fm[rd] < 0) continue;
      const int e = fm[rd] & 0xff, fj0 = fm[rd] >> 8;
#pragma unroll
      for (int c = 0; c < NF; ++c) {
        const int m = c * E + e;
        if constexpr (TF)
          tcm::put_tf32x2(sA, P::A_SLICE_L, tcm::kmajor_off<KG>(m, fj0, P::SBO_L),
                          fv[rd][0][c], fv[rd][1][c]);
        else
          tcm::put_digits2(sA, P::A_SLICE_L, tcm::kmajor_off(m, fj0, P::SBO_L), fv[rd][0][c],
                           fv[rd][1][c], tcm::row_exp_bits(rmaxL[m]));
      }
    }
    zero_pad_l();
    tc::fence_async_smem();
    __syncthreads();
    if (t == 0) {
      if constexpr (TF)
        tcm::issue_phase_tf32<P::KL, P::SBO_L, P::A_SLICE_L, P::B_SLICE_L, NB>(
            a_s, b_s + P::OPS_L, tmem + P::ACC_L, P::IDESC);
      else
        tcm::issue_phase<P::KL, P::SBO_L, P::A_SLICE_L, P::B_SLICE_L, NB>(
            a_s, b_s + P::OPS_L, tmem + P::ACC_L, P::IDESC);
      tc::tc_commit(&mma_bar);
      led.issue(0);
    }
    // the face phase and the volume inputs of this tile are complete (they
    // read the geometry before the barrier above): stage the next tile's
    if (tile + gridDim.x < ntiles) stage_geometry(tile + gridDim.x);
    if (__syncthreads_or(!wait_mma())) break;  // a wait gave up: leave the tile loop
    // }}}

    // {{{ 4. level sums -> staging (warp w reads lanes 32 (w % 4)..), epilogue
    if constexpr (TF) {
      const int qd = warp & 3;
      const int row = 32 * qd + lane;
      const uint32_t tq = tmem + ((uint32_t)(32 * qd) << 16);
      float sc = 1.f;
      if constexpr (EQ == DG_MAXWELL) sc = (row / E) < 3 ? fc.ie : fc.im;
#pragma unroll 1
      for (int ch = warp >> 2; ch < NB / 8; ch += NWARP / 4) {
        uint32_t v[16], l[16];  // hi x hi, cross terms x 8 columns
        tc::tc_ld8(tq + (uint32_t)(ch * 8), v);
        tc::tc_ld8(tq + (uint32_t)(NB + ch * 8), v + 8);
        tc::tc_ld8(tq + (uint32_t)(P::ACC_L + ch * 8), l);
        tc::tc_ld8(tq + (uint32_t)(P::ACC_L + NB + ch * 8), l + 8);
        tc::tc_wait_ld();
        if (row < P::NCOL) {
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) {
            const int col = ch * 8 + jj;
            if (col < NP) {
              const float vol = __uint_as_float(v[jj]) + __uint_as_float(v[8 + jj]);
              const float lift = __uint_as_float(l[jj]) + __uint_as_float(l[8 + jj]);
              sOut[row * OP + col] = sc * (vol + lift);
            }
          }
        }
      }
    } else {
      const int qd = warp & 3;
      const int row = 32 * qd + lane;
      const uint32_t tq = tmem + ((uint32_t)(32 * qd) << 16);
      float sc = 1.f;
      if constexpr (EQ == DG_MAXWELL) sc = (row / E) < 3 ? fc.ie : fc.im;
      // row factors 2^(E_m - 14), E_m = e - 126 (the column factors 2^e_B
      // come with the operator); products of powers of two are exact
      const float rsv = tcm::pow2f(tcm::row_exp_bits(rmaxV[row]) - 140);
      const float rsl = tcm::pow2f(tcm::row_exp_bits(rmaxL[row]) - 140);
#pragma unroll 1
      for (int ch = warp >> 2; ch < NB / 8; ch += NWARP / 4) {
        uint32_t v[32], l[32];  // levels 0..3 x 8 columns
#pragma unroll
        for (int lv = 0; lv < 4; ++lv) {
          tc::tc_ld8(tq + (uint32_t)(lv * NB + ch * 8), v + 8 * lv);
          tc::tc_ld8(tq + (uint32_t)(P::ACC_L + lv * NB + ch * 8), l + 8 * lv);
        }
        tc::tc_wait_ld();
        if (row < P::NCOL) {
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) {
            const int col = ch * 8 + jj;
            if (col < NP) {
              const float vol = tcm::levels4(v, jj) * (rsv * sEV[col]);
              const float lift = tcm::levels4(l, jj) * (rsl * sEL[col]);
              sOut[row * OP + col] = sc * (vol + lift);
            }
          }
        }
      }
    }
    tc::tc_fence_before();
    __syncthreads();
    for (int idx = t; idx < ecount * NP; idx += THREADS) {
      const int e = idx / NP, i = idx - e * NP;
      int64_t gidx = e0 * NP + idx;
      const double es = a.elem_scale ? __ldg(a.elem_scale + e0 + e) : 1.0;
#pragma unroll
      for (int k = 0; k < NF; ++k, gidx += nelnp) {
        double val = f2d_alu(sOut[(k * E + e) * OP + i]);
        if constexpr (STAGE)
          if (a.rhs_unscaled) a.rhs_unscaled[gidx] = val;
        if (a.elem_scale) val *= es;
        if constexpr (!STAGE) {
          a.rhs[gidx] = val;
        } else {
          const double r = (a.rk_a != 0.0 ? a.rk_a * a.res[gidx] : 0.0) + a.rk_dt * val;
          a.res[gidx] = r;
          a.q_out[gidx] = __ldg(a.q + gidx) + a.rk_b * r;
        }
      }
    }
    // digits: no barrier, the next tile's phase 1 writes the state copies and
    // the other row-maxima buffer, which no thread still reads.  TF32: its
    // phase 1 writes X, where the results above were staged.  The first
    // tensor-memory use follows two barriers.
    if constexpr (TF) __syncthreads();
    // }}}
  }
  // after a wait gave up: the issuing thread waits (bounded) for products it
  // still owes before the tensor memory is released; if they never complete
  // the status already reads DG_ERR_TIMEOUT and the memory is released with
  // them outstanding
  if (t == 0 && led.owes(0)) mbar_wait_bounded(&mma_bar, led.phase[0]);
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"(P::TMEM_COLS)
                 : "memory");
}

}  // namespace dg
