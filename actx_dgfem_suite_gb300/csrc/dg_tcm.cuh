// Mixed-precision RHS with the contractions on the tcgen05 tensor cores.
//
// The volume derivatives and LIFT of the mixed-precision path (FP32
// arithmetic, FP64 state) as one product per tile, with the roles of data and
// operator chosen for the tensor core's 128-row shape:
//
//   D (128 x Np) = X (128 x K) B^T,   K = 3 Np + 4 Nfp (two phases)
//
// Each of the 128 rows of X is one (field c, element e) column of the tile's
// data: the metric-combined inputs w_{c,r}(j) of the three reference
// derivatives (r = 0, 1, 2; nodes j), then the field's lifted face values:
//   wave    w_{0,r} = -c (G v)_r,  w_{1+x,r} = -c G_{r x} u;
//   euler   w_{k,r} = sum_x G_{r x} F_{k x}(q);
//   maxwell w_{c,r} from E_t = curl H, H_t = -curl E, e.g.
//           w_{0,r} = G_{r 1} H_z - G_{r 2} H_y;
// B is the operator [A_0 A_1 A_2 | LIFT] (Np rows; A_r the reference
// derivative the equation uses).  So D holds vol + lift of every output node
// directly: no per-node combination after the product.  X and B are split
// into TF32 pairs x = x_hi + x_lo (cvt.rna) and multiplied as
// x_hi b_hi + x_hi b_lo + x_lo b_hi with FP32 accumulation in tensor memory
// (tcgen05.mma kind::tf32, M = 128, N = Np padded to 16, K = 8 per
// instruction): FP32 accuracy, the error of the CUDA-core FP32 path.
//
// Per tile of E = 128 / NF elements:
//   1. per node (8 elements x 4 nodes per warp, so the 4-byte stores into the
//      K-major operand layout are free of bank conflicts): the FP64 state ->
//      FP32 copy in shared memory, the metric-combined inputs (Euler: the
//      pressure from total energy in FP64) -> X (volume phase);
//   2. one thread issues the volume products (asynchronous, completion on an
//      mbarrier); meanwhile every thread evaluates the numerical flux of its
//      face points into registers;
//   3. after the volume products have read X, the face values are written
//      into X (LIFT phase) and the LIFT products accumulate into the same D;
//   4. tcgen05.ld of D -> shared staging, then coalesced FP64 stores (RHS) or
//      the fused low-storage RK stage.
// Waits on the mbarriers are bounded (DG_ERR_TIMEOUT instead of spinning).
//
// Flux formulas as in dg_rhs.cuh (wave.py:80-114, grudge's Euler LF flux
// with InviscidWallBC, MaxwellOperator alpha-flux with PEC).
#pragma once

#include "dg_tc.cuh"

namespace dg {
namespace tcm {

constexpr int kThreads = 512;  // one CTA per SM

constexpr int r8(int x) { return (x + 7) & ~7; }
constexpr int r16(int x) { return (x + 15) & ~15; }
constexpr int p16(int b) { return (b + 15) & ~15; }
// row pitch (words) >= n with pitch % 32 == 4: 8 elements x 4 nodes of a warp
// hit 32 distinct banks
constexpr int pitch_q(int n) { return n <= 4 ? 4 : ((n - 4 + 31) / 32) * 32 + 4; }

template <int N, int EQ>
struct MPlan {
  static constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP, NFPT = Shape<N>::NFPT;
  static constexpr int NF = EqInfo<EQ>::NF;
  static constexpr int E = 128 / NF;      // elements per tile
  static constexpr int NCOL = NF * E;     // rows of X in use (m = c E + e)
  static constexpr int NB = r16(NP);      // operator rows (MMA N)
  static constexpr int KV = r8(3 * NP), KL = r8(NFPT);
  // K-major, no swizzle: element (m, k) of a slice at
  //   (m / 8) SBO + (k / 4) 128 + (m % 8) 16 + (k % 4) 4 bytes
  static constexpr int SBO_V = (KV / 4) * 128, SBO_L = (KL / 4) * 128;
  static constexpr int A_SLICE_V = 16 * SBO_V, A_SLICE_L = 16 * SBO_L;
  static constexpr int A_BYTES = 2 * (A_SLICE_V > A_SLICE_L ? A_SLICE_V : A_SLICE_L);
  // operator block (global and shared): vol hi | vol lo | lift hi | lift lo |
  // int32 face nodes
  static constexpr int B_SLICE_V = (NB / 8) * SBO_V, B_SLICE_L = (NB / 8) * SBO_L;
  static constexpr int OPS_V = 0, OPS_L = 2 * B_SLICE_V, OPS_FN = OPS_L + 2 * B_SLICE_L;
  static constexpr int OPS_BYTES = OPS_FN + p16(NFPT * 4);
  static constexpr int QP = pitch_q(NP);  // FP32 state rows
  static constexpr int OP = NP | 1;       // FP32 result rows (odd pitch)
  static constexpr int SM_A = 0;
  static constexpr int SM_OPS = SM_A + A_BYTES;
  static constexpr int SM_Q = SM_OPS + OPS_BYTES;
  static constexpr int SM_OUT = SM_Q + p16(NF * E * QP * 4);
  static constexpr int SM_P = SM_OUT + p16(NCOL * OP * 4);
  static constexpr int SMEM_BYTES = SM_P + (EQ == DG_EULER ? p16(E * NP * 8) : 0);
  static constexpr int TMEM_COLS = NB <= 32 ? 32 : (NB <= 64 ? 64 : 128);
  // instruction descriptor: D FP32, A and B TF32, both K-major, N, M = 128
  static constexpr uint32_t IDESC =
      (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NB >> 3) << 17) | (8u << 24);
  static_assert(NCOL <= 128, "one 128-row product per tile");
  static_assert(NB >= 16 && NB <= 256, "MMA N range");
  static_assert(SMEM_BYTES <= 227 * 1024, "tile does not fit in shared memory");
};

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
      ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// x -> (hi, lo) TF32 pair stored at byte offset `off` of both slices
__device__ __forceinline__ void put_split(unsigned char* base, int slice_bytes, int off,
                                          float x) {
  uint32_t hi, lo;
  tf32_split(x, hi, lo);
  *reinterpret_cast<uint32_t*>(base + off) = hi;
  *reinterpret_cast<uint32_t*>(base + slice_bytes + off) = lo;
}

__device__ __forceinline__ int kmajor_off(int m, int k, int sbo) {
  return (m >> 3) * sbo + (k >> 2) * 128 + (m & 7) * 16 + (k & 3) * 4;
}

// One K phase: per k-step of 8, x_hi b_hi, x_hi b_lo, x_lo b_hi into D.
template <int K, int SBO, int A_SLICE, int B_SLICE>
__device__ __forceinline__ void issue_phase(uint32_t a_s, uint32_t b_s, uint32_t tmem,
                                            uint32_t idesc, bool first) {
  tc::tc_fence_after();
#pragma unroll 1
  for (int kt = 0; kt < K / 8; ++kt) {
    const uint32_t ka = a_s + kt * 256, kb = b_s + kt * 256;
    const uint64_t ah = tc::smem_desc(ka, 128, SBO), al = tc::smem_desc(ka + A_SLICE, 128, SBO);
    const uint64_t bh = tc::smem_desc(kb, 128, SBO), bl = tc::smem_desc(kb + B_SLICE, 128, SBO);
    mma_tf32(tmem, al, bh, idesc, (first && kt == 0) ? 0u : 1u);
    mma_tf32(tmem, ah, bl, idesc, 1u);
    mma_tf32(tmem, ah, bh, idesc, 1u);
  }
}

// Numerical flux of one face point in FP32 (FP64 exterior state, FP64
// Euler pressures); out[c] = the lifted face value of field c.
template <int EQ, int NF>
__device__ __forceinline__ void face_point_flux(const RhsArgs& a, const float* qi,
                                                const double* qed, bool bdry, float nx,
                                                float ny, float nz, float scale,
                                                double pi_d, float* out) {
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
    const float c = (float)a.p0;
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
    const float gamma = (float)a.p0;
    double pe_d;
    if (bdry) {
      pe_d = pi_d;  // the wall mirror keeps rho, |m| and E
      const float mn = qi[2] * nx + qi[3] * ny + qi[4] * nz;
      qe[0] = qi[0];
      qe[1] = qi[1];
      qe[2] = qi[2] - 2.f * nx * mn;
      qe[3] = qi[3] - 2.f * ny * mn;
      qe[4] = qi[4] - 2.f * nz * mn;
    } else {
      const double rinv_e = rcp64_fast(qed[0]);
      pe_d = (a.p0 - 1.0) *
             (qed[1] - 0.5 * (qed[2] * qed[2] + qed[3] * qed[3] + qed[4] * qed[4]) * rinv_e);
    }
    float fn_i[5], fn_e[5], lam_i, lam_e;
    auto side = [&](const float* q, double p_d, float* fn, float& lam) {
      const float p = d2f_alu(p_d);
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
    side(qi, pi_d, fn_i, lam_i);
    side(qe, pe_d, fn_e, lam_e);
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
    const float alpha = (float)a.p0;
    const float z = (float)a.k[0], y = (float)a.k[1];
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
    const float ce = (float)a.k[2], ch = (float)a.k[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      out[x] = -scale * (ce * fe[x]);
      out[3 + x] = -scale * (ch * fh[x]);
    }
  }
}

}  // namespace tcm

template <int N, int EQ, int MODE>
__global__ void __launch_bounds__(tcm::kThreads, 1) dg_rhs_tcm_kernel(const RhsArgs a) {
  using P = tcm::MPlan<N, EQ>;
  constexpr int NP = P::NP, NFP = P::NFP, NFPT = P::NFPT, NF = P::NF, E = P::E;
  constexpr int QP = P::QP, OP = P::OP;
  constexpr bool STAGE = (MODE & MODE_STAGE) != 0;
  constexpr int NWARP = tcm::kThreads / 32;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint64_t mma_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int ops_ok;

  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  unsigned char* sA = smem + P::SM_A;
  const int* sFN = reinterpret_cast<const int*>(smem + P::SM_OPS + P::OPS_FN);
  float* sq = reinterpret_cast<float*>(smem + P::SM_Q);
  float* sOut = reinterpret_cast<float*>(smem + P::SM_OUT);
  double* sP = reinterpret_cast<double*>(smem + P::SM_P);
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
  // the data operand's padding (k past 3 Np or 4 Nfp) meets zero operator
  // columns; it must hold finite values, so clear the region once
  for (int idx = t; idx < P::A_BYTES / 16; idx += tcm::kThreads)
    reinterpret_cast<uint4*>(sA)[idx] = make_uint4(0u, 0u, 0u, 0u);
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
  uint32_t mma_phase = 0;
  const uint32_t a_s = smem_u32(sA);
  const uint32_t b_s = smem_u32(smem + P::SM_OPS);

  const int64_t nel = a.nel;
  const int64_t nelnp = nel * NP;
  const int64_t ntiles = (nel + E - 1) / E;
  constexpr int EG = (E + 7) / 8, JG = (NP + 3) / 4, FG = (NFPT + 3) / 4;
  constexpr int FROUNDS = (EG * FG + NWARP - 1) / NWARP;  // face items per thread

  auto wait_mma = [&]() {
    if (!mbar_wait_bounded(&mma_bar, mma_phase)) raise_status(a.status, DG_ERR_TIMEOUT);
    mma_phase ^= 1u;
    tc::tc_fence_after();
  };

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t e0 = tile * E;
    const int ecount = (nel - e0) < (int64_t)E ? (int)(nel - e0) : E;

    // {{{ 1. state -> FP32 copy, metric-combined volume inputs -> X
    for (int u = warp; u < EG * JG; u += NWARP) {
      const int e = (u % EG) * 8 + (lane & 7);
      const int j = (u / EG) * 4 + (lane >> 3);
      if (e >= E || j >= NP) continue;
      const bool valid = e < ecount;
      const int64_t gnode = (e0 + e) * NP + j;
      double qd[NF];
      float qf[NF];
#pragma unroll
      for (int k = 0; k < NF; ++k) {
        qd[k] = valid ? __ldg(a.q + k * nelnp + gnode) : (k == 0 ? 1.0 : 0.0);
        qf[k] = d2f_alu(qd[k]);
        sq[(k * E + e) * QP + j] = qf[k];
      }
      float G[9];
#pragma unroll
      for (int x = 0; x < 9; ++x) G[x] = valid ? d2f_alu(__ldg(a.metric + (e0 + e) * 9 + x)) : 0.f;
      float w[NF][3];
      if constexpr (EQ == DG_WAVE) {
        const float c = (float)a.p0;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          w[0][r] = -c * fmaf(G[r * 3 + 0], qf[1], fmaf(G[r * 3 + 1], qf[2], G[r * 3 + 2] * qf[3]));
#pragma unroll
          for (int x = 0; x < 3; ++x) w[1 + x][r] = -c * (G[r * 3 + x] * qf[0]);
        }
      } else if constexpr (EQ == DG_EULER) {
        const double rinv_d = rcp64_fast(qd[0]);
        const double p_d =
            (a.p0 - 1.0) *
            (qd[1] - 0.5 * (qd[2] * qd[2] + qd[3] * qd[3] + qd[4] * qd[4]) * rinv_d);
        sP[e * NP + j] = p_d;
        const float p = d2f_alu(p_d), rinv = d2f_alu(rinv_d);
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
#pragma unroll
      for (int c = 0; c < NF; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r)
          tcm::put_split(sA, P::A_SLICE_V, tcm::kmajor_off(c * E + e, r * NP + j, P::SBO_V),
                         w[c][r]);
    }
    tc::fence_async_smem();
    __syncthreads();
    // }}}

    // {{{ 2. volume products (one thread), face fluxes (registers)
    if (t == 0) {
      tcm::issue_phase<P::KV, P::SBO_V, P::A_SLICE_V, P::B_SLICE_V>(
          a_s, b_s + P::OPS_V, tmem, P::IDESC, true);
      tc::tc_commit(&mma_bar);
    }
    float fv[FROUNDS][NF];
    int fm[FROUNDS];  // kmajor offset of (row c = 0, k = fj), -1: none
#pragma unroll
    for (int rd = 0; rd < FROUNDS; ++rd) {
      fm[rd] = -1;
      const int u = warp + rd * NWARP;
      if (u >= EG * FG) continue;
      const int e = (u % EG) * 8 + (lane & 7);
      const int fj = (u / EG) * 4 + (lane >> 3);
      if (e >= ecount || fj >= NFPT) continue;
      const int f = fj / NFP;
      const int node = sFN[fj];
      const uint32_t g = __ldg(a.gather + (e0 + e) * NFPT + fj);
      const bool bdry = (g >> 31) != 0u;
      uint32_t gi = g & 0x7fffffffu;
      if (gi >= (uint32_t)nelnp) {  // never read out of bounds
        raise_status(a.status, DG_ERR_INDEX);
        gi = (uint32_t)((e0 + e) * NP + node);
      }
      const double* fg = a.face_geom + (e0 + e) * 16 + f * 4;
      const float nx = d2f_alu(__ldg(fg + 0)), ny = d2f_alu(__ldg(fg + 1)),
                  nz = d2f_alu(__ldg(fg + 2)), scale = d2f_alu(__ldg(fg + 3));
      float qi[NF];
      double qed[NF];
#pragma unroll
      for (int k = 0; k < NF; ++k) {
        qi[k] = sq[(k * E + e) * QP + node];
        qed[k] = bdry ? 0.0 : __ldg(a.q + k * nelnp + gi);
      }
      const double pi_d = EQ == DG_EULER ? sP[e * NP + node] : 0.0;
      tcm::face_point_flux<EQ, NF>(a, qi, qed, bdry, nx, ny, nz, scale, pi_d, fv[rd]);
      fm[rd] = e | (fj << 8);
    }
    wait_mma();  // the volume products have read X
    // }}}

    // {{{ 3. face values -> X, LIFT products into the same accumulator
#pragma unroll
    for (int rd = 0; rd < FROUNDS; ++rd) {
      if (fm[rd] < 0) continue;
      const int e = fm[rd] & 0xff, fj = fm[rd] >> 8;
#pragma unroll
      for (int c = 0; c < NF; ++c)
        tcm::put_split(sA, P::A_SLICE_L, tcm::kmajor_off(c * E + e, fj, P::SBO_L), fv[rd][c]);
    }
    tc::fence_async_smem();
    __syncthreads();
    if (t == 0) {
      tcm::issue_phase<P::KL, P::SBO_L, P::A_SLICE_L, P::B_SLICE_L>(
          a_s, b_s + P::OPS_L, tmem, P::IDESC, false);
      tc::tc_commit(&mma_bar);
    }
    wait_mma();
    // }}}

    // {{{ 4. D -> staging (warp w reads lanes 32 (w % 4)..), then the epilogue
    {
      const int qd = warp & 3;
      const int row = 32 * qd + lane;
      const uint32_t tq = tmem + ((uint32_t)(32 * qd) << 16);
      float sc = 1.f;
      if constexpr (EQ == DG_MAXWELL) sc = (row / E) < 3 ? (float)a.k[4] : (float)a.k[5];
#pragma unroll 1
      for (int ch = warp >> 2; ch < P::NB / 8; ch += NWARP / 4) {
        uint32_t v[8];
        tc::tc_ld8(tq + (uint32_t)(ch * 8), v);
        tc::tc_wait_ld();
        if (row < P::NCOL) {
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) {
            const int col = ch * 8 + jj;
            if (col < NP) sOut[row * OP + col] = sc * __uint_as_float(v[jj]);
          }
        }
      }
    }
    tc::tc_fence_before();
    __syncthreads();
    for (int idx = t; idx < ecount * NP; idx += tcm::kThreads) {
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
    // no barrier: the next tile writes X and the state copy, which no thread
    // reads any more, and its first tensor-memory use follows a barrier
    // }}}
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"(P::TMEM_COLS)
                 : "memory");
}

}  // namespace dg
