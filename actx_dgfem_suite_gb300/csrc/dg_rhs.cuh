// Fused DG-FEM RHS kernel for affine tetrahedra on sm_103a.
//
// One persistent launch evaluates the whole RHS of one equation.  Each CTA
// stages the reference operators (weak or strong D_r and LIFT, with the face
// node table) into shared memory once, by a single TMA bulk copy, then loops
// over tiles of E = 256 / Np elements:
//
//   1. load the tile's state (all fields, FP64) and geometry into shared memory;
//   2. pointwise pre-pass per node: metric-combined inputs of the weak
//      divergence (wave: v, euler: the flux F(q)); maxwell needs none;
//   3. volume term per output node, in registers:
//        wave    -c * sum_r W_r (G v)_r        and  -c * G^T (W_r u)
//        euler    sum_r W_r (G F(q))_r
//        maxwell  curl via sum_r G[r][x] D_r q
//      (the fused einsums ``xre,rij,xej->ei`` and ``re,rij,ej->ei`` of
//      actx_dgfem_suite/arraycontext/mass_inverse_fuser.py:39-74, with the
//      three reference derivatives of a field shared by its gradient
//      components);
//   4. face gather + numerical flux per face node, scaled by sJ/J, into
//      shared memory (exterior values through the flat gather index of
//      actx_dgfem_suite/arraycontext/constants_folder.py:69-100);
//   5. LIFT ``jfi,fe,fej->ei`` (mass_inverse_fuser.py:21-38 after the
//      transpose of transpose_consts_in_einsums.py:5-35) added to the volume
//      term, optionally multiplied by a per-element factor (variable wave
//      speed), then either stored (MODE_RHS) or folded into a low-storage
//      Runge-Kutta stage (MODE_STAGE): res = a res + dt L(q), q_out = q + b res.
//
// With MODE_SPLIT (FP64 only) step 4 is replaced by a coalesced load of face
// values that dg_face_flux_kernel (dg_face.cuh) evaluated once per glued pair
// of face points, and the Euler pre-pass reads pressure and 1/rho from the
// per-node table of dg_euler_aux_kernel instead of dividing.
//
// ``Real`` is the arithmetic type of steps 2-5.  double: the plain FP64 path.
// float: the mixed-precision path -- derivative, flux and LIFT arithmetic in
// FP32 while the state, the RK accumulation and the Euler pressure recovery
// from total energy stay FP64.
//
// The flux formulas follow actx_dgfem_suite/equations/wave.py:80-114 (wave),
// grudge's euler_numerical_flux with LF stabilisation and InviscidWallBC
// (configured at equations/euler.py:168-174) and grudge's MaxwellOperator
// alpha-flux with PEC (configured at equations/maxwell.py:55-59).
#pragma once

#include <type_traits>

#include "dg_common.cuh"

namespace dg {

// bit 0: RK stage epilogue; bit 1: face values from the face-shared kernels;
// bit 2: mixed precision with the volume and LIFT contractions on the tensor
// cores (3xTF32 split, FP32 accumulation); bits 3 and 4 (MODE_TC only): the
// tile shape, 128 or 512 threads per CTA and E = 128 / Np or 512 / Np
// elements per tile instead of kBlock = 256 threads and 256 / Np elements
enum { MODE_RHS = 0, MODE_STAGE = 1, MODE_SPLIT = 2, MODE_TC = 4, MODE_B128 = 8,
       MODE_B512 = 16 };

// threads per CTA (one per (element, node) of the tile) of a mode
constexpr int block_of(int mode) {
  return (mode & MODE_B128) ? 128 : ((mode & MODE_B512) ? 512 : kBlock);
}

struct RhsArgs {
  const double* q;
  double* rhs;             // MODE_RHS output
  double* q_out;           // MODE_STAGE outputs
  double* res;
  double rk_a, rk_b, rk_dt;
  const double* elem_scale;  // (Nel) per-element factor on the RHS, or NULL
  double* rhs_unscaled;      // MODE_STAGE: L(q) before elem_scale, or NULL
  const double* metric;
  const double* face_geom;
  const uint32_t* gather;
  const void* ops;         // [Wt | Lt | face_nodes], see OpsLayout
  uint32_t ops_bytes;
  int64_t nel;
  int* status;
  double p0, p1, p2;       // equation parameters
  double k[6];             // maxwell: z, 1/z, -1/(2z), 1/(2/z), 1/eps, 1/mu
  const double* flux_in;   // MODE_SPLIT: (NF, Nel, 4 Nfp) face values
  const double* aux;       // MODE_SPLIT euler: (3, Nel, Np) p, 1/rho, |u| + c
  const float* pres;       // mixed-precision euler: (Nel, Np) pressure, recovered
                           // from total energy in FP64 once per node, as FP32
};

template <int N>
struct Shape {
  static constexpr int NP = (N + 1) * (N + 2) * (N + 3) / 6;
  static constexpr int NFP = (N + 1) * (N + 2) / 2;
  static constexpr int NFPT = 4 * NFP;  // face points per element
};

template <int EQ>
struct EqInfo;
template <>
struct EqInfo<DG_WAVE> {
  static constexpr int NF = 4, NAUX = 3;
};
template <>
struct EqInfo<DG_EULER> {
  static constexpr int NF = 5, NAUX = 15;
};
template <>
struct EqInfo<DG_MAXWELL> {
  static constexpr int NF = 6, NAUX = 0;
};

constexpr int pad16(int bytes) { return (bytes + 15) & ~15; }

// Row pitch (in floats) for rows read with 16-byte shared-memory loads: a
// multiple of 4 whose quotient by 4 is odd, so 8 consecutive rows map to 8
// distinct 16-byte bank groups (conflict-free LDS.128 across a quarter warp).
constexpr int odd4(int n) {
  return (((n + 3) & ~3) / 4) % 2 == 0 ? ((n + 3) & ~3) + 4 : ((n + 3) & ~3);
}

// Shared-memory row pitches.  FP64: the unpadded scalar layout.  Mixed:
// padded rows read four entries at a time (float4).
template <int N, typename Real>
struct Pitch {
  static constexpr bool MIXED = !std::is_same<Real, double>::value;
  static constexpr int ROW = MIXED ? odd4(Shape<N>::NP) : Shape<N>::NP;
  static constexpr int FROW = MIXED ? odd4(Shape<N>::NFPT) : Shape<N>::NFPT;
};

// Layout of the operator block in bytes, identical in global and shared memory.
//   FP64:  W^T as Wt[r][j][i] (i fastest) | LIFT^T as Lt[fj][i]   (scalar reads)
//   mixed: W as W[r][i][j] (j fastest, pitch ROW) | LIFT as L[i][fj] (pitch FROW)
template <int N, typename Real>
struct OpsLayout {
  static constexpr int NP = Shape<N>::NP, NFPT = Shape<N>::NFPT;
  static constexpr int RS = (int)sizeof(Real);
  static constexpr bool MIXED = Pitch<N, Real>::MIXED;
  static constexpr int W = 0;
  static constexpr int L =
      W + pad16((MIXED ? 3 * NP * Pitch<N, Real>::ROW : 3 * NP * NP) * RS);
  static constexpr int FN =
      L + pad16((MIXED ? NP * Pitch<N, Real>::FROW : NFPT * NP) * RS);
  static constexpr int SIZE = FN + pad16(NFPT * 4);
};

// Shared-memory layout of one CTA, in bytes.  SPLIT (the face-shared FP64
// path, face values computed by the face kernel): no face geometry is
// staged, and for Euler the face values reuse the flux-input buffer of the
// volume term (they are loaded after the volume contractions), which keeps
// more CTAs resident at the low orders.
template <int N, int EQ, typename Real, bool SPLIT = false, int BLOCK = kBlock>
struct Tile {
  static constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP,
                       NFPT = Shape<N>::NFPT;
  static constexpr int NF = EqInfo<EQ>::NF, NAUX = EqInfo<EQ>::NAUX;
  static constexpr int E = BLOCK / NP;
  static constexpr bool MIXED = !std::is_same<Real, double>::value;
  static constexpr int RS = (int)sizeof(Real);
  static constexpr int ROW = Pitch<N, Real>::ROW, FROW = Pitch<N, Real>::FROW;
  static constexpr int Q = OpsLayout<N, Real>::SIZE;              // double
  static constexpr int QR = Q + pad16(NF * E * NP * 8);           // Real copy
  static constexpr int AUX = QR + (MIXED ? pad16(NF * E * ROW * RS) : 0);
  static constexpr int AUX_BYTES = pad16(NAUX * E * ROW * RS);
  static constexpr int FLUX_BYTES = pad16(NF * E * FROW * RS);
  // face values loaded late over the volume inputs (split Euler only)
  static constexpr bool LATE_FLUX = SPLIT && EQ == DG_EULER;
  static constexpr int FLUX = LATE_FLUX ? AUX : AUX + AUX_BYTES;
  static constexpr int GEO =
      LATE_FLUX ? AUX + (AUX_BYTES > FLUX_BYTES ? AUX_BYTES : FLUX_BYTES) : FLUX + FLUX_BYTES;
  static constexpr int FGEO = GEO + pad16(9 * E * RS);
  // mixed-precision Euler: FP64 pressure of every node of the tile
  static constexpr int PRES = FGEO + (SPLIT ? 0 : pad16(16 * E * RS));
  static constexpr int SMEM_BASE =
      PRES + ((MIXED && EQ == DG_EULER) ? pad16(E * NP * 8) : 0);
  // MODE_TC: FP32 outputs of the tensor-core products (volume, then LIFT)
  static constexpr int VOL_M = EQ == DG_EULER ? NP : 3 * NP;
  static constexpr int VOL_NC = EQ == DG_MAXWELL ? NF * E : (EQ == DG_WAVE ? E : NF * E);
  static constexpr int TC_FLOATS_VOL = VOL_M * VOL_NC + (EQ == DG_WAVE ? NP * E : 0);
  static constexpr int TC_FLOATS = TC_FLOATS_VOL > NP * NF * E ? TC_FLOATS_VOL : NP * NF * E;
  static constexpr int TC = SMEM_BASE;
  static constexpr int SMEM_BYTES_TC = TC + pad16(TC_FLOATS * 4);
};

// {{{ 3xTF32 tensor-core products (mixed precision, MODE_TC)

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// x = hi + lo with both parts TF32: hi carries 11 significant bits, lo the next 11
__device__ __forceinline__ void tf32_split(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32_rna(x);
  lo = tf32_rna(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float* c, const uint32_t* a, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// C (M x NC, FP32, row-major with leading dimension NC) = A (M x K) B (K x NC)
// with A(m, k), B(k, n) read through accessors (zero outside the ranges),
// a b = a_hi b_hi + a_hi b_lo + a_lo b_hi in FP32 (relative error ~2^-21,
// the accuracy of FP32 arithmetic).  Warp units: one m-tile x two n-tiles,
// spread over the CTA's NWARPS warps.
template <int M, int K, int NC, int NWARPS, class FA, class FB>
__device__ __forceinline__ void tf32x3_gemm(FA fa, FB fb, float* out) {
  constexpr int MT = (M + 15) / 16, KT = (K + 7) / 8, NT = (NC + 7) / 8;
  constexpr int NB = (NT + 1) / 2, UNITS = MT * NB;
  const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  for (int u = threadIdx.x >> 5; u < UNITS; u += NWARPS) {
    const int mt = u / NB, nt0 = 2 * (u - mt * NB);
    const bool two = nt0 + 1 < NT;
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    const int r0 = mt * 16 + g, r1 = r0 + 8;
#pragma unroll 2
    for (int kt = 0; kt < KT; ++kt) {
      const int k0 = kt * 8 + tq, k1 = k0 + 4;
      uint32_t ah[4], al[4];
      tf32_split(r0 < M && k0 < K ? fa(r0, k0) : 0.f, ah[0], al[0]);
      tf32_split(r1 < M && k0 < K ? fa(r1, k0) : 0.f, ah[1], al[1]);
      tf32_split(r0 < M && k1 < K ? fa(r0, k1) : 0.f, ah[2], al[2]);
      tf32_split(r1 < M && k1 < K ? fa(r1, k1) : 0.f, ah[3], al[3]);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        if (q == 1 && !two) break;
        const int n = (nt0 + q) * 8 + g;
        uint32_t bh0, bl0, bh1, bl1;
        tf32_split(n < NC && k0 < K ? fb(k0, n) : 0.f, bh0, bl0);
        tf32_split(n < NC && k1 < K ? fb(k1, n) : 0.f, bh1, bl1);
        mma_tf32(acc[q], al, bh0, bh1);
        mma_tf32(acc[q], ah, bl0, bl1);
        mma_tf32(acc[q], ah, bh0, bh1);
      }
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q == 1 && !two) break;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int row = c >= 2 ? r1 : r0;
        const int col = (nt0 + q) * 8 + 2 * tq + (c & 1);
        if (row < M && col < NC) out[row * NC + col] = acc[q][c];
      }
    }
  }
}

// }}}

// FP64 reciprocal from the FP32 estimate refined by one Newton step
// (relative error below 2^-45).  The mixed-precision path uses it for the
// FP64 pressure recovery, where a correctly rounded FP64 division would
// dominate the cost on GB300's narrow FP64 pipe.
__device__ __forceinline__ double rcp64_fast(double x) {
  const double r0 = (double)__frcp_rn((float)x);
  const double e = fma(-x, r0, 1.0);
  return fma(r0, e, r0);
}

__device__ __forceinline__ float dot4(const float4 w, const float4 x, float acc) {
  return fmaf(w.x, x.x, fmaf(w.y, x.y, fmaf(w.z, x.z, fmaf(w.w, x.w, acc))));
}

// double -> arithmetic type; the mixed path converts on the integer ALU
template <typename Real>
__device__ __forceinline__ Real to_real(double v) {
  if constexpr (std::is_same<Real, double>::value) return v;
  else return d2f_alu(v);
}

template <int N, int EQ, typename Real, int MODE>
__global__ void __launch_bounds__(block_of(MODE)) dg_rhs_kernel(const RhsArgs a) {
  constexpr int BLOCK = block_of(MODE);
  using T = Tile<N, EQ, Real, (MODE & MODE_SPLIT) != 0, BLOCK>;
  using Ops = OpsLayout<N, Real>;
  constexpr bool STAGE = (MODE & MODE_STAGE) != 0;
  constexpr bool SPLIT = (MODE & MODE_SPLIT) != 0;
  constexpr bool TCM = (MODE & MODE_TC) != 0;
  static_assert(!(SPLIT && T::MIXED), "the face-shared path is FP64 only");
  static_assert(!TCM || T::MIXED, "tensor-core products are a mixed-precision mode");
  static_assert(BLOCK == kBlock || TCM, "other tile shapes are MODE_TC variants");
  static_assert(T::E >= 1, "at least one element per tile");
  constexpr int NP = T::NP, NFPT = T::NFPT, NF = T::NF, E = T::E;
  constexpr int ROW = T::ROW, FROW = T::FROW;  // shared-memory row pitches
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ int ops_ok;

  const Real* sW = reinterpret_cast<const Real*>(smem + Ops::W);
  const Real* sL = reinterpret_cast<const Real*>(smem + Ops::L);
  const int* sFN = reinterpret_cast<const int*>(smem + Ops::FN);
  double* sQ = reinterpret_cast<double*>(smem + T::Q);
  Real* sQr = T::MIXED ? reinterpret_cast<Real*>(smem + T::QR)
                       : reinterpret_cast<Real*>(smem + T::Q);
  Real* sAux = reinterpret_cast<Real*>(smem + T::AUX);
  Real* sFlux = reinterpret_cast<Real*>(smem + T::FLUX);
  Real* sG = reinterpret_cast<Real*>(smem + T::GEO);
  Real* sFG = reinterpret_cast<Real*>(smem + T::FGEO);
  float* sPf = reinterpret_cast<float*>(smem + T::PRES);  // mixed euler: node pressures
  float* sTC = reinterpret_cast<float*>(smem + T::TC);  // MODE_TC outputs

  const int t = threadIdx.x;
  if (t == 0) {
    mbar_init(&bar, 1);
    mbar_arrive_expect_tx(&bar, a.ops_bytes);
    bulk_g2s(smem, a.ops, a.ops_bytes, &bar);
    const bool ok = mbar_wait_bounded(&bar, 0);
    if (!ok) {
      raise_status(a.status, DG_ERR_TIMEOUT);
      mbar_wait_bounded(&bar, 0);  // give the copy one more bounded chance
    }
    ops_ok = ok ? 1 : 0;
  }
  if constexpr (T::MIXED) {
    // padded rows are read by the vector loads: give the pads a value once
    float* z = reinterpret_cast<float*>(smem + T::QR);
    const int nz = (T::GEO - T::QR) / 4;
    for (int idx = t; idx < nz; idx += BLOCK) z[idx] = 0.0f;
  }
  __syncthreads();
  if (!ops_ok) return;

  const int el = t / NP;
  const int i = t - el * NP;
  const bool active = el < E;
  const int64_t nel = a.nel;
  const int64_t nelnp = nel * NP;
  const int64_t ntiles = (nel + E - 1) / E;
  const Real p0 = (Real)a.p0;
  const Real half = (Real)0.5, two = (Real)2, zero = (Real)0;
  const Real inv_eps = (Real)a.k[4], inv_mu = (Real)a.k[5];

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t e0 = tile * E;
    const int ecount = (nel - e0) < (int64_t)E ? (int)(nel - e0) : E;

    // {{{ 1. state and geometry -> shared memory (coalesced; 64-bit address
    //         arithmetic once per tile and field, 32-bit offsets inside)
    {
      const double* qk = a.q + e0 * NP;
#pragma unroll
      for (int k = 0; k < NF; ++k, qk += nelnp) {
        for (int rem = t; rem < E * NP; rem += BLOCK) {
          const double v = rem < ecount * NP ? __ldg(qk + rem) : 0.0;
          sQ[k * (E * NP) + rem] = v;
          if constexpr (T::MIXED) {
            const int le = rem / NP;
            sQr[(k * E + le) * ROW + (rem - le * NP)] = to_real<Real>(v);
          }
        }
      }
    }
    {
      const double* mt = a.metric + e0 * 9;
      for (int idx = t; idx < 9 * E; idx += BLOCK)
        sG[idx] = idx < 9 * ecount ? to_real<Real>(__ldg(mt + idx)) : zero;
      if constexpr (!SPLIT) {  // face geometry: the fused path's fluxes only
        const double* ft = a.face_geom + e0 * 16;
        for (int idx = t; idx < 16 * E; idx += BLOCK)
          sFG[idx] = idx < 16 * ecount ? to_real<Real>(__ldg(ft + idx)) : zero;
      }
    }
    // face values of the tile, contiguous per field (split Euler: after the
    // volume term, over its inputs)
    auto load_face_values = [&]() {
      const int64_t nfpt_all = nel * NFPT;
      const double* fk = a.flux_in + e0 * NFPT;
#pragma unroll
      for (int k = 0; k < NF; ++k, fk += nfpt_all)
        for (int rem = t; rem < E * NFPT; rem += BLOCK)
          sFlux[k * (E * FROW) + rem] = rem < ecount * NFPT ? __ldg(fk + rem) : zero;
    };
    if constexpr (SPLIT && !T::LATE_FLUX) load_face_values();
    __syncthreads();
    // }}}

    // {{{ 2. pointwise pre-pass
    if constexpr (EQ == DG_WAVE) {
      if (active && el < ecount) {
        const Real* G = sG + el * 9;
        const Real v0 = sQr[(1 * E + el) * ROW + i];
        const Real v1 = sQr[(2 * E + el) * ROW + i];
        const Real v2 = sQr[(3 * E + el) * ROW + i];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          sAux[(r * E + el) * ROW + i] =
              fma(G[r * 3 + 0], v0, fma(G[r * 3 + 1], v1, G[r * 3 + 2] * v2));
      }
    } else if constexpr (EQ == DG_EULER) {
      if (active && el < ecount) {
        const Real* G = sG + el * 9;
        Real p, en, m[3], rinv;
        if constexpr (T::MIXED) {
          // the pressure from the per-node table (recovered from total
          // energy in FP64 by dg_euler_pressure_f32_kernel)
          p = __ldg(a.pres + e0 * NP + (el * NP + i));
          sPf[el * NP + i] = p;
          en = sQr[(1 * E + el) * ROW + i];
#pragma unroll
          for (int c = 0; c < 3; ++c) m[c] = sQr[((2 + c) * E + el) * ROW + i];
          rinv = __frcp_rn(sQr[(0 * E + el) * ROW + i]);
        } else {
          const double rho_d = sQ[(0 * E + el) * NP + i];
          const double en_d = sQ[(1 * E + el) * NP + i];
          const double md[3] = {sQ[(2 * E + el) * NP + i], sQ[(3 * E + el) * NP + i],
                                sQ[(4 * E + el) * NP + i]};
          double rinv_d, p_d;
          if constexpr (SPLIT) {
            const int64_t gidx = e0 * NP + (el * NP + i);
            p_d = __ldg(a.aux + gidx);
            rinv_d = __ldg(a.aux + nelnp + gidx);
          } else {
            rinv_d = 1.0 / rho_d;
            p_d = (a.p0 - 1.0) *
                  (en_d - 0.5 * (md[0] * md[0] + md[1] * md[1] + md[2] * md[2]) * rinv_d);
          }
          p = p_d;
          en = en_d;
#pragma unroll
          for (int c = 0; c < 3; ++c) m[c] = md[c];
          rinv = rinv_d;
        }
        // metric-combined fluxes A_k^r = sum_x G[r][x] F_k,x with
        // F_0 = m, F_1 = u (E + p), F_{2+c} = m_c u + p e_c; through
        // U_r = (G u)_r: A_0^r = (G m)_r, A_1^r = (E + p) U_r,
        // A_{2+c}^r = m_c U_r + p G[r][c] (43 operations per node, not 64)
        const Real u[3] = {m[0] * rinv, m[1] * rinv, m[2] * rinv};
        const Real ep = en + p;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const Real* Gr = G + r * 3;
          const Real ur = fma(Gr[0], u[0], fma(Gr[1], u[1], Gr[2] * u[2]));
          Real* out = sAux + (r * E + el) * ROW + i;
          constexpr int KS = 3 * E * ROW;  // stride of k in sAux
          out[0 * KS] = fma(Gr[0], m[0], fma(Gr[1], m[1], Gr[2] * m[2]));
          out[1 * KS] = ep * ur;
#pragma unroll
          for (int c = 0; c < 3; ++c) out[(2 + c) * KS] = fma(m[c], ur, p * Gr[c]);
        }
      }
    }
    if constexpr (T::NAUX > 0) __syncthreads();
    // }}}

    // {{{ 3. volume term (registers)
    Real vol[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) vol[k] = zero;
    if constexpr (TCM) {
      // tensor-core products into sTC, then the per-node combinations
      constexpr int VNC = T::VOL_NC;
      if constexpr (EQ == DG_WAVE) {
        tf32x3_gemm<3 * NP, NP, E, BLOCK / 32>(
            [&](int m, int k) { return sW[m * ROW + k]; },
            [&](int k, int n) { return sQr[n * ROW + k]; }, sTC);
        tf32x3_gemm<NP, 3 * NP, E, BLOCK / 32>(
            [&](int m, int k) { const int r = k / NP; return sW[(r * NP + m) * ROW + k - r * NP]; },
            [&](int k, int n) { const int r = k / NP; return sAux[(r * E + n) * ROW + k - r * NP]; },
            sTC + 3 * NP * E);
      } else if constexpr (EQ == DG_EULER) {
        tf32x3_gemm<NP, 3 * NP, VNC, BLOCK / 32>(
            [&](int m, int k) { const int r = k / NP; return sW[(r * NP + m) * ROW + k - r * NP]; },
            [&](int k, int n) {
              const int r = k / NP, f = n / E, e = n - f * E;
              return sAux[((f * 3 + r) * E + e) * ROW + k - r * NP];
            },
            sTC);
      } else {
        tf32x3_gemm<3 * NP, NP, VNC, BLOCK / 32>(
            [&](int m, int k) { return sW[m * ROW + k]; },
            [&](int k, int n) { return sQr[n * ROW + k]; }, sTC);
      }
      __syncthreads();
      if (active && el < ecount) {
        const Real* G = sG + el * 9;
        if constexpr (EQ == DG_WAVE) {
          const float ur0 = sTC[(0 * NP + i) * E + el], ur1 = sTC[(1 * NP + i) * E + el],
                      ur2 = sTC[(2 * NP + i) * E + el];
          const Real c = p0;
          vol[0] = -c * sTC[3 * NP * E + i * E + el];
#pragma unroll
          for (int x = 0; x < 3; ++x)
            vol[1 + x] = -c * fma(G[0 * 3 + x], ur0, fma(G[1 * 3 + x], ur1, G[2 * 3 + x] * ur2));
        } else if constexpr (EQ == DG_EULER) {
#pragma unroll
          for (int k = 0; k < 5; ++k) vol[k] = sTC[i * VNC + k * E + el];
        } else {
          auto dx = [&](int k, int x) {
            const float d0 = sTC[(0 * NP + i) * VNC + k * E + el];
            const float d1 = sTC[(1 * NP + i) * VNC + k * E + el];
            const float d2 = sTC[(2 * NP + i) * VNC + k * E + el];
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
    } else if (active && el < ecount) {
      const Real* G = sG + el * 9;
      if constexpr (T::MIXED) {
        // float4 operands: four matrix entries per 16-byte shared load
        const float4* w0v = reinterpret_cast<const float4*>(sW + (0 * NP + i) * ROW);
        const float4* w1v = reinterpret_cast<const float4*>(sW + (1 * NP + i) * ROW);
        const float4* w2v = reinterpret_cast<const float4*>(sW + (2 * NP + i) * ROW);
        auto row = [&](const Real* base, int r) {
          return reinterpret_cast<const float4*>(base + (r * E + el) * ROW);
        };
        if constexpr (EQ == DG_WAVE) {
          const float4* uv = row(sQr, 0);
          const float4 *a0 = row(sAux, 0), *a1 = row(sAux, 1), *a2 = row(sAux, 2);
          float ur0 = 0.f, ur1 = 0.f, ur2 = 0.f, dv = 0.f;
#pragma unroll
          for (int jj = 0; jj < ROW / 4; ++jj) {
            const float4 w0 = w0v[jj], w1 = w1v[jj], w2 = w2v[jj], u = uv[jj];
            ur0 = dot4(w0, u, ur0);
            ur1 = dot4(w1, u, ur1);
            ur2 = dot4(w2, u, ur2);
            dv = dot4(w0, a0[jj], dot4(w1, a1[jj], dot4(w2, a2[jj], dv)));
          }
          const Real c = p0;
          vol[0] = -c * dv;
#pragma unroll
          for (int x = 0; x < 3; ++x)
            vol[1 + x] = -c * fma(G[0 * 3 + x], ur0,
                                  fma(G[1 * 3 + x], ur1, G[2 * 3 + x] * ur2));
        } else if constexpr (EQ == DG_EULER) {
#pragma unroll
          for (int jj = 0; jj < ROW / 4; ++jj) {
            const float4 w0 = w0v[jj], w1 = w1v[jj], w2 = w2v[jj];
#pragma unroll
            for (int k = 0; k < 5; ++k)
              vol[k] = dot4(w0, row(sAux, k * 3 + 0)[jj],
                            dot4(w1, row(sAux, k * 3 + 1)[jj],
                                 dot4(w2, row(sAux, k * 3 + 2)[jj], vol[k])));
          }
        } else {  // DG_MAXWELL
          float d[6][3];
#pragma unroll
          for (int k = 0; k < 6; ++k) d[k][0] = d[k][1] = d[k][2] = 0.f;
#pragma unroll
          for (int jj = 0; jj < ROW / 4; ++jj) {
            const float4 w0 = w0v[jj], w1 = w1v[jj], w2 = w2v[jj];
#pragma unroll
            for (int k = 0; k < 6; ++k) {
              const float4 qv = row(sQr, k)[jj];
              d[k][0] = dot4(w0, qv, d[k][0]);
              d[k][1] = dot4(w1, qv, d[k][1]);
              d[k][2] = dot4(w2, qv, d[k][2]);
            }
          }
          auto dx = [&](int k, int x) {
            return fma(G[0 * 3 + x], d[k][0],
                       fma(G[1 * 3 + x], d[k][1], G[2 * 3 + x] * d[k][2]));
          };
          vol[0] = dx(5, 1) - dx(4, 2);
          vol[1] = dx(3, 2) - dx(5, 0);
          vol[2] = dx(4, 0) - dx(3, 1);
          vol[3] = -(dx(2, 1) - dx(1, 2));
          vol[4] = -(dx(0, 2) - dx(2, 0));
          vol[5] = -(dx(1, 0) - dx(0, 1));
        }
      } else if constexpr (EQ == DG_WAVE) {
        const Real c = p0;
        const Real* u = sQr + el * NP;
        Real ur0 = zero, ur1 = zero, ur2 = zero, dv = zero;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const Real w0 = sW[(0 * NP + j) * NP + i];
          const Real w1 = sW[(1 * NP + j) * NP + i];
          const Real w2 = sW[(2 * NP + j) * NP + i];
          const Real uj = u[j];
          ur0 = fma(w0, uj, ur0);
          ur1 = fma(w1, uj, ur1);
          ur2 = fma(w2, uj, ur2);
          dv = fma(w0, sAux[(0 * E + el) * NP + j],
                   fma(w1, sAux[(1 * E + el) * NP + j],
                       fma(w2, sAux[(2 * E + el) * NP + j], dv)));
        }
        vol[0] = -c * dv;
#pragma unroll
        for (int x = 0; x < 3; ++x)
          vol[1 + x] = -c * fma(G[0 * 3 + x], ur0,
                                fma(G[1 * 3 + x], ur1, G[2 * 3 + x] * ur2));
      } else if constexpr (EQ == DG_EULER) {
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const Real w0 = sW[(0 * NP + j) * NP + i];
          const Real w1 = sW[(1 * NP + j) * NP + i];
          const Real w2 = sW[(2 * NP + j) * NP + i];
#pragma unroll
          for (int k = 0; k < 5; ++k)
            vol[k] = fma(w0, sAux[((k * 3 + 0) * E + el) * NP + j],
                         fma(w1, sAux[((k * 3 + 1) * E + el) * NP + j],
                             fma(w2, sAux[((k * 3 + 2) * E + el) * NP + j],
                                 vol[k])));
        }
      } else {  // DG_MAXWELL: strong derivatives, curl
        Real d[6][3];
#pragma unroll
        for (int k = 0; k < 6; ++k) d[k][0] = d[k][1] = d[k][2] = zero;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const Real w0 = sW[(0 * NP + j) * NP + i];
          const Real w1 = sW[(1 * NP + j) * NP + i];
          const Real w2 = sW[(2 * NP + j) * NP + i];
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            const Real qj = sQr[(k * E + el) * NP + j];
            d[k][0] = fma(w0, qj, d[k][0]);
            d[k][1] = fma(w1, qj, d[k][1]);
            d[k][2] = fma(w2, qj, d[k][2]);
          }
        }
        // dq_k/dx_x = sum_r G[r][x] d[k][r]
        auto dx = [&](int k, int x) {
          return fma(G[0 * 3 + x], d[k][0],
                     fma(G[1 * 3 + x], d[k][1], G[2 * 3 + x] * d[k][2]));
        };
        // E_t = curl H, H_t = -curl E
        vol[0] = dx(5, 1) - dx(4, 2);
        vol[1] = dx(3, 2) - dx(5, 0);
        vol[2] = dx(4, 0) - dx(3, 1);
        vol[3] = -(dx(2, 1) - dx(1, 2));
        vol[4] = -(dx(0, 2) - dx(2, 0));
        vol[5] = -(dx(1, 0) - dx(0, 1));
      }
    }
    // }}}

    // {{{ 4. face gather + numerical flux (fused path only)
    const uint32_t* gt = a.gather + e0 * NFPT;
    const uint32_t tile_node0 = (uint32_t)(e0 * NP);
    for (int pidx = t; pidx < (SPLIT ? 0 : ecount * NFPT); pidx += BLOCK) {
      const int elp = pidx / NFPT;
      const int fj = pidx - elp * NFPT;
      const int f = fj / Shape<N>::NFP;
      const int node = sFN[fj];
      const uint32_t g = __ldg(gt + pidx);
      const bool bdry = (g >> 31) != 0u;
      uint32_t gi = g & 0x7fffffffu;
      if (gi >= (uint32_t)nelnp) {  // never read out of bounds
        raise_status(a.status, DG_ERR_INDEX);
        gi = tile_node0 + (uint32_t)(elp * NP + node);
      }
      const Real* fg = sFG + (elp * 4 + f) * 4;
      const Real nx = fg[0], ny = fg[1], nz = fg[2], scale = fg[3];
      // interior trace from shared memory (already in the arithmetic type),
      // exterior trace from HBM through the gather index (FP64 state)
      Real qi[NF], qe[NF];
      double qed[NF];
#pragma unroll
      for (int k = 0; k < NF; ++k) qi[k] = sQr[(k * E + elp) * ROW + node];
      if (!bdry) {
        const double* qk = a.q + gi;
#pragma unroll
        for (int k = 0; k < NF; ++k, qk += nelnp) {
          qed[k] = __ldg(qk);
          qe[k] = to_real<Real>(qed[k]);
        }
      }
      Real* out = sFlux + elp * FROW + fj;
      constexpr int FS = E * FROW;  // field stride in sFlux

      if constexpr (EQ == DG_WAVE) {
        if (bdry) {  // Dirichlet mirror: exterior (-u, v)
          qe[0] = -qi[0];
          qe[1] = qi[1];
          qe[2] = qi[2];
          qe[3] = qi[3];
        }
        const Real c = p0;
        const Real vavg_n = half * (qi[1] + qe[1]) * nx + half * (qi[2] + qe[2]) * ny +
                            half * (qi[3] + qe[3]) * nz;
        const Real uavg = half * (qi[0] + qe[0]);
        const Real vjump = (qe[1] - qi[1]) * nx + (qe[2] - qi[2]) * ny +
                           (qe[3] - qi[3]) * nz;
        const Real fu = c * (vavg_n + half * (qe[0] - qi[0]));
        const Real fv = c * (uavg + half * vjump);
        out[0 * FS] = scale * fu;
        out[1 * FS] = scale * (fv * nx);
        out[2 * FS] = scale * (fv * ny);
        out[3 * FS] = scale * (fv * nz);
      } else if constexpr (EQ == DG_EULER) {
        const Real gamma = p0;
        Real pi_m = zero, pe_m = zero;
        if constexpr (T::MIXED) {
          // pressures from the per-node table: interior through the pre-pass
          // copy, exterior at the gathered node (the wall mirror keeps rho,
          // |m| and E, so its pressure)
          pi_m = sPf[elp * NP + node];
          pe_m = bdry ? pi_m : __ldg(a.pres + gi);
        }
        if (bdry) {  // InviscidWallBC: mirror the normal momentum
          if constexpr (T::MIXED) {
            const Real mn = qi[2] * nx + qi[3] * ny + qi[4] * nz;
            qe[0] = qi[0];
            qe[1] = qi[1];
            qe[2] = qi[2] - two * nx * mn;
            qe[3] = qi[3] - two * ny * mn;
            qe[4] = qi[4] - two * nz * mn;
          } else {  // FP64: the normal in FP64 from HBM
            const double* fgd = a.face_geom + e0 * 16 + (elp * 4 + f) * 4;
            const double ndx = fgd[0], ndy = fgd[1], ndz = fgd[2];
            const double mn = qi[2] * ndx + qi[3] * ndy + qi[4] * ndz;
            qe[0] = qi[0];
            qe[1] = qi[1];
            qe[2] = qi[2] - 2.0 * ndx * mn;
            qe[3] = qi[3] - 2.0 * ndy * mn;
            qe[4] = qi[4] - 2.0 * ndz * mn;
          }
        }
        Real fn_i[5], fn_e[5], lam_i, lam_e;
        auto side = [&](const Real* q, Real p_mixed, Real* fn, Real& lam) {
          Real p, rinv;
          if constexpr (T::MIXED) {
            p = p_mixed;
            rinv = (Real)1 / q[0];
          } else {
            const double rinv_d = 1.0 / q[0];
            p = (a.p0 - 1.0) *
                (q[1] - 0.5 * (q[2] * q[2] + q[3] * q[3] + q[4] * q[4]) * rinv_d);
            rinv = rinv_d;
          }
          const Real ux = q[2] * rinv, uy = q[3] * rinv, uz = q[4] * rinv;
          const Real un = ux * nx + uy * ny + uz * nz;
          fn[0] = q[2] * nx + q[3] * ny + q[4] * nz;
          fn[1] = un * (q[1] + p);
          fn[2] = q[2] * un + p * nx;
          fn[3] = q[3] * un + p * ny;
          fn[4] = q[4] * un + p * nz;
          lam = sqrt(ux * ux + uy * uy + uz * uz) + sqrt(gamma * (p * rinv));
        };
        side(qi, pi_m, fn_i, lam_i);
        side(qe, pe_m, fn_e, lam_e);
        const Real lam = fmax(lam_i, lam_e);
        const Real nn = nx * nx + ny * ny + nz * nz;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const Real dq = qe[k] - qi[k];
          const Real fk = half * (fn_i[k] + fn_e[k]) - half * lam * dq * nn;
          out[k * FS] = -scale * fk;
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
        const Real alpha = p0;
        const Real z = (Real)a.k[0], y = (Real)a.k[1];
        const Real je[3] = {qe[0] - qi[0], qe[1] - qi[1], qe[2] - qi[2]};
        const Real jh[3] = {qe[3] - qi[3], qe[4] - qi[4], qe[5] - qi[5]};
        const Real n[3] = {nx, ny, nz};
        auto cross = [](const Real* a_, const Real* b_, Real* c_) {
          c_[0] = a_[1] * b_[2] - a_[2] * b_[1];
          c_[1] = a_[2] * b_[0] - a_[0] * b_[2];
          c_[2] = a_[0] * b_[1] - a_[1] * b_[0];
        };
        Real nxe[3], nxh[3], te[3], th[3], fe[3], fh[3];
        cross(n, je, nxe);
        cross(n, jh, nxh);
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          te[x] = z * jh[x] - alpha * nxe[x];
          th[x] = y * je[x] + alpha * nxh[x];
        }
        cross(n, te, fe);
        cross(n, th, fh);
        const Real ce = (Real)a.k[2], ch = (Real)a.k[3];
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          out[x * FS] = -scale * (ce * fe[x]);
          out[(3 + x) * FS] = -scale * (ch * fh[x]);
        }
      }
    }
    __syncthreads();
    if constexpr (T::LATE_FLUX) {  // the volume term no longer reads its inputs
      load_face_values();
      __syncthreads();
    }
    // }}}

    // {{{ 5. LIFT, then store or fold into the RK stage
    if constexpr (TCM) {
      tf32x3_gemm<NP, NFPT, NF * E, BLOCK / 32>(
          [&](int m, int k) { return sL[m * FROW + k]; },
          [&](int k, int n) { return sFlux[n * FROW + k]; }, sTC);
      __syncthreads();
    }
    if (active && el < ecount) {
      const Real* fl = sFlux + el * FROW;
      int64_t gidx = e0 * NP + (el * NP + i);  // advanced by nelnp per field
#pragma unroll
      for (int k = 0; k < NF; ++k, gidx += nelnp) {
        Real acc = vol[k];
        if constexpr (TCM) {
          acc += sTC[i * (NF * E) + k * E + el];
        } else if constexpr (T::MIXED) {
          const float4* lv = reinterpret_cast<const float4*>(sL + i * FROW);
          const float4* fv = reinterpret_cast<const float4*>(fl + k * E * FROW);
#pragma unroll
          for (int jj = 0; jj < FROW / 4; ++jj) acc = dot4(lv[jj], fv[jj], acc);
        } else {
#pragma unroll 4
          for (int fj = 0; fj < NFPT; ++fj)
            acc = fma(sL[fj * NP + i], fl[k * E * NFPT + fj], acc);
        }
        if constexpr (EQ == DG_MAXWELL) acc = acc * (k < 3 ? inv_eps : inv_mu);
        double val;
        if constexpr (T::MIXED) val = f2d_alu(acc);
        else val = acc;
        if constexpr (STAGE)
          if (a.rhs_unscaled) a.rhs_unscaled[gidx] = val;
        if (a.elem_scale) val *= __ldg(a.elem_scale + e0 + el);
        if constexpr (!STAGE) {
          a.rhs[gidx] = val;
        } else {
          const double r =
              (a.rk_a != 0.0 ? a.rk_a * a.res[gidx] : 0.0) + a.rk_dt * val;
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
