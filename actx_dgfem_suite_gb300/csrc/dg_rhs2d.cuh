// DG-FEM RHS kernel for affine triangles (2D meshes) on sm_103a, FP64.
//
// The 2D counterpart of dg_rhs_kernel (dg_rhs.cuh) for the suite's runs with
// dim = 2: one persistent launch evaluates the whole RHS.  Each CTA stages
// the reference operators (weak or strong D_r for r = 0, 1, LIFT for three
// edges, the edge node table) into shared memory once by one bulk copy
// completed on an mbarrier (bounded wait), then loops over tiles of
// E = 256 / Np elements with one thread per (element, node):
//
//   1. the tile's state (all fields), metric and edge geometry -> shared memory;
//   2. pointwise pre-pass: metric-combined inputs of the weak divergence
//      (wave: (G v)_r; euler: (G F_k(q))_r);
//   3. volume term per node in registers:
//        wave     -c sum_r W_r (G v)_r  and  -c G^T (W_r u)
//        euler    sum_r W_r (G F_k)_r
//        maxwell  TM curls from the strong derivatives:
//                 E_z: dH_y/dx - dH_x/dy,  H_x: -dE_z/dy,  H_y: dE_z/dx
//   4. edge gather (flat 4-byte index, bit 31 = boundary, bounds checked)
//      and the numerical flux per edge point, scaled by sJ/J;
//   5. LIFT added to the volume term (Maxwell: times 1/eps, 1/mu), then the
//      store or the fused low-storage RK stage, with the optional
//      per-element factor.
//
// Fields: wave (u, v_x, v_y); euler (rho, E, m_x, m_y); maxwell TM (E_z,
// H_x, H_y), grudge's field subset for dimensions = 2.  The fluxes are those
// of the 3D kernel with two-component vectors (wave.py:80-114, grudge's LF
// flux with InviscidWallBC, the Maxwell alpha flux on E = (0, 0, E_z),
// H = (H_x, H_y, 0), n = (n_x, n_y, 0), PEC).
#pragma once

#include "dg_common.cuh"
#include "dg_rhs.cuh"  // RhsArgs, MODE_RHS / MODE_STAGE, pad16

namespace dg {

template <int N>
struct Shape2 {
  static constexpr int NP = (N + 1) * (N + 2) / 2;
  static constexpr int NFP = N + 1;
  static constexpr int NFPT = 3 * NFP;  // edge points per element
};

template <int EQ>
struct Eq2;
template <>
struct Eq2<DG_WAVE> {
  static constexpr int NF = 3, NAUX = 2, NNODE = 0;
};
template <>
struct Eq2<DG_EULER> {
  static constexpr int NF = 4, NAUX = 8, NNODE = 3;  // per node: p, 1/rho, |u| + c
};
template <>
struct Eq2<DG_MAXWELL> {
  static constexpr int NF = 3, NAUX = 0, NNODE = 0;
};

// Operator block in bytes (global and shared): Wt[r][j][i] (2 Np Np
// doubles) | Lt[fj][i] (3 Nfp Np doubles) | int32 edge node table (3 Nfp).
template <int N>
struct Ops2 {
  static constexpr int NP = Shape2<N>::NP, NFPT = Shape2<N>::NFPT;
  static constexpr int W = 0;
  static constexpr int L = W + pad16(2 * NP * NP * 8);
  static constexpr int FN = L + pad16(NFPT * NP * 8);
  static constexpr int SIZE = FN + pad16(NFPT * 4);
};

template <int N, int EQ>
struct Tile2 {
  static constexpr int NP = Shape2<N>::NP, NFP = Shape2<N>::NFP, NFPT = Shape2<N>::NFPT;
  static constexpr int NF = Eq2<EQ>::NF, NAUX = Eq2<EQ>::NAUX;
  static constexpr int E = kBlock / NP;
  static constexpr int Q = Ops2<N>::SIZE;
  static constexpr int AUX = Q + pad16(NF * E * NP * 8);
  static constexpr int FLUX = AUX + pad16(NAUX * E * NP * 8);
  static constexpr int GEO = FLUX + pad16(NF * E * NFPT * 8);
  static constexpr int FGEO = GEO + pad16(4 * E * 8);
  // Euler: pressure, 1/rho and wave speed of every node of the tile, for the
  // interior side of its edge points
  static constexpr int NODE = FGEO + pad16(12 * E * 8);
  static constexpr int SMEM_BYTES = NODE + pad16(Eq2<EQ>::NNODE * E * NP * 8);
};

template <int N, int EQ, int MODE>
__global__ void __launch_bounds__(kBlock) dg_rhs2d_kernel(const RhsArgs a) {
  using T = Tile2<N, EQ>;
  using O = Ops2<N>;
  constexpr bool STAGE = (MODE & MODE_STAGE) != 0;
  constexpr int NP = T::NP, NFP = T::NFP, NFPT = T::NFPT, NF = T::NF, E = T::E;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ int ops_ok;

  const double* sW = reinterpret_cast<const double*>(smem + O::W);
  const double* sL = reinterpret_cast<const double*>(smem + O::L);
  const int* sFN = reinterpret_cast<const int*>(smem + O::FN);
  double* sQ = reinterpret_cast<double*>(smem + T::Q);
  double* sAux = reinterpret_cast<double*>(smem + T::AUX);
  double* sFlux = reinterpret_cast<double*>(smem + T::FLUX);
  double* sG = reinterpret_cast<double*>(smem + T::GEO);
  double* sFG = reinterpret_cast<double*>(smem + T::FGEO);
  [[maybe_unused]] double* sNode = reinterpret_cast<double*>(smem + T::NODE);

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
  __syncthreads();
  if (!ops_ok) return;

  const int el = t / NP;
  const int i = t - el * NP;
  const bool active = el < E;
  const int64_t nel = a.nel;
  const int64_t nelnp = nel * NP;
  const int64_t ntiles = (nel + E - 1) / E;
  const double p0 = a.p0;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t e0 = tile * E;
    const int ecount = (nel - e0) < (int64_t)E ? (int)(nel - e0) : E;

    // {{{ 1. state and geometry -> shared memory (coalesced)
    {
      const double* qk = a.q + e0 * NP;
#pragma unroll
      for (int k = 0; k < NF; ++k, qk += nelnp)
        for (int rem = t; rem < E * NP; rem += kBlock)
          sQ[k * (E * NP) + rem] = rem < ecount * NP ? __ldg(qk + rem) : 0.0;
      const double* mt = a.metric + e0 * 4;
      for (int idx = t; idx < 4 * E; idx += kBlock)
        sG[idx] = idx < 4 * ecount ? __ldg(mt + idx) : 0.0;
      const double* ft = a.face_geom + e0 * 12;
      for (int idx = t; idx < 12 * E; idx += kBlock)
        sFG[idx] = idx < 12 * ecount ? __ldg(ft + idx) : 0.0;
    }
    __syncthreads();
    // }}}

    // {{{ 2. pointwise pre-pass
    if (active && el < ecount) {
      const double* G = sG + el * 4;   // G[r * 2 + x] = dr_r / dx_x
      if constexpr (EQ == DG_WAVE) {
        const double v0 = sQ[(1 * E + el) * NP + i], v1 = sQ[(2 * E + el) * NP + i];
#pragma unroll
        for (int r = 0; r < 2; ++r)
          sAux[(r * E + el) * NP + i] = fma(G[r * 2 + 0], v0, G[r * 2 + 1] * v1);
      } else if constexpr (EQ == DG_EULER) {
        const double rho = sQ[(0 * E + el) * NP + i], en = sQ[(1 * E + el) * NP + i];
        const double m[2] = {sQ[(2 * E + el) * NP + i], sQ[(3 * E + el) * NP + i]};
        const double rinv = 1.0 / rho;
        const double p = (p0 - 1.0) * (en - 0.5 * (m[0] * m[0] + m[1] * m[1]) * rinv);
        const double u[2] = {m[0] * rinv, m[1] * rinv};
        const double ep = en + p;
        sNode[(0 * E + el) * NP + i] = p;
        sNode[(1 * E + el) * NP + i] = rinv;
        sNode[(2 * E + el) * NP + i] = sqrt(u[0] * u[0] + u[1] * u[1]) + sqrt(p0 * (p * rinv));
        // A_k^r = sum_x G[r][x] F_k,x with F_0 = m, F_1 = u (E + p),
        // F_{2+c} = m_c u + p e_c, through U_r = (G u)_r
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const double* Gr = G + r * 2;
          const double ur = fma(Gr[0], u[0], Gr[1] * u[1]);
          constexpr int KS = 2 * E * NP;  // stride of k in sAux
          double* out = sAux + (r * E + el) * NP + i;
          out[0 * KS] = fma(Gr[0], m[0], Gr[1] * m[1]);
          out[1 * KS] = ep * ur;
#pragma unroll
          for (int c = 0; c < 2; ++c) out[(2 + c) * KS] = fma(m[c], ur, p * Gr[c]);
        }
      }
    }
    if constexpr (T::NAUX > 0) __syncthreads();
    // }}}

    // {{{ 3. volume term (registers)
    double vol[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) vol[k] = 0.0;
    if (active && el < ecount) {
      const double* G = sG + el * 4;
      if constexpr (EQ == DG_WAVE) {
        const double* u = sQ + el * NP;
        double ur0 = 0.0, ur1 = 0.0, dv = 0.0;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const double w0 = sW[(0 * NP + j) * NP + i], w1 = sW[(1 * NP + j) * NP + i];
          ur0 = fma(w0, u[j], ur0);
          ur1 = fma(w1, u[j], ur1);
          dv = fma(w0, sAux[(0 * E + el) * NP + j], fma(w1, sAux[(1 * E + el) * NP + j], dv));
        }
        vol[0] = -p0 * dv;
#pragma unroll
        for (int x = 0; x < 2; ++x) vol[1 + x] = -p0 * fma(G[0 * 2 + x], ur0, G[1 * 2 + x] * ur1);
      } else if constexpr (EQ == DG_EULER) {
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const double w0 = sW[(0 * NP + j) * NP + i], w1 = sW[(1 * NP + j) * NP + i];
#pragma unroll
          for (int k = 0; k < 4; ++k)
            vol[k] = fma(w0, sAux[((k * 2 + 0) * E + el) * NP + j],
                         fma(w1, sAux[((k * 2 + 1) * E + el) * NP + j], vol[k]));
        }
      } else {  // DG_MAXWELL (TM): strong derivatives of E_z, H_x, H_y
        double d[3][2];
#pragma unroll
        for (int k = 0; k < 3; ++k) d[k][0] = d[k][1] = 0.0;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const double w0 = sW[(0 * NP + j) * NP + i], w1 = sW[(1 * NP + j) * NP + i];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const double qj = sQ[(k * E + el) * NP + j];
            d[k][0] = fma(w0, qj, d[k][0]);
            d[k][1] = fma(w1, qj, d[k][1]);
          }
        }
        auto dx = [&](int k, int x) { return fma(G[0 * 2 + x], d[k][0], G[1 * 2 + x] * d[k][1]); };
        vol[0] = dx(2, 0) - dx(1, 1);  // (curl H)_z
        vol[1] = -dx(0, 1);            // -(curl E)_x
        vol[2] = dx(0, 0);             // -(curl E)_y
      }
    }
    // }}}

    // {{{ 4. edge gather + numerical flux
    const uint32_t* gt = a.gather + e0 * NFPT;
    const uint32_t tile_node0 = (uint32_t)(e0 * NP);
    for (int pidx = t; pidx < ecount * NFPT; pidx += kBlock) {
      const int elp = pidx / NFPT;
      const int fj = pidx - elp * NFPT;
      const int f = fj / NFP;
      const int node = sFN[fj];
      const uint32_t g = __ldg(gt + pidx);
      const bool bdry = (g >> 31) != 0u;
      uint32_t gi = g & 0x7fffffffu;
      if (gi >= (uint32_t)nelnp) {  // never read out of bounds
        raise_status(a.status, DG_ERR_INDEX);
        gi = tile_node0 + (uint32_t)(elp * NP + node);
      }
      const double* fg = sFG + (elp * 3 + f) * 4;
      const double nx = fg[0], ny = fg[1], scale = fg[2];
      double qi[NF], qe[NF];
#pragma unroll
      for (int k = 0; k < NF; ++k) qi[k] = sQ[(k * E + elp) * NP + node];
      if (!bdry) {
        const double* qk = a.q + gi;
#pragma unroll
        for (int k = 0; k < NF; ++k, qk += nelnp) qe[k] = __ldg(qk);
      }
      double* out = sFlux + elp * NFPT + fj;
      constexpr int FS = E * NFPT;  // field stride in sFlux

      if constexpr (EQ == DG_WAVE) {
        if (bdry) {  // Dirichlet mirror: exterior (-u, v)
          qe[0] = -qi[0];
          qe[1] = qi[1];
          qe[2] = qi[2];
        }
        const double vavg_n = 0.5 * (qi[1] + qe[1]) * nx + 0.5 * (qi[2] + qe[2]) * ny;
        const double uavg = 0.5 * (qi[0] + qe[0]);
        const double vjump = (qe[1] - qi[1]) * nx + (qe[2] - qi[2]) * ny;
        const double fu = p0 * (vavg_n + 0.5 * (qe[0] - qi[0]));
        const double fv = p0 * (uavg + 0.5 * vjump);
        out[0 * FS] = scale * fu;
        out[1 * FS] = scale * (fv * nx);
        out[2 * FS] = scale * (fv * ny);
      } else if constexpr (EQ == DG_EULER) {
        if (bdry) {  // InviscidWallBC: mirror the normal momentum
          const double mn = qi[2] * nx + qi[3] * ny;
          qe[0] = qi[0];
          qe[1] = qi[1];
          qe[2] = qi[2] - 2.0 * nx * mn;
          qe[3] = qi[3] - 2.0 * ny * mn;
        }
        double fn_i[4], fn_e[4], lam_i, lam_e;
        // normal fluxes of one side from its pressure and 1/rho
        auto side = [&](const double* q, double p, double rinv, double* fn) {
          const double un = (q[2] * nx + q[3] * ny) * rinv;
          fn[0] = q[2] * nx + q[3] * ny;
          fn[1] = un * (q[1] + p);
          fn[2] = q[2] * un + p * nx;
          fn[3] = q[3] * un + p * ny;
        };
        // interior: the node's values from the pre-pass; the wall mirror
        // keeps rho, |m| and E, so the boundary exterior shares them too
        const double pi = sNode[(0 * E + elp) * NP + node];
        const double ri = sNode[(1 * E + elp) * NP + node];
        lam_i = sNode[(2 * E + elp) * NP + node];
        side(qi, pi, ri, fn_i);
        if (bdry) {
          side(qe, pi, ri, fn_e);
          lam_e = lam_i;
        } else {
          const double re = 1.0 / qe[0];
          const double pe = (p0 - 1.0) * (qe[1] - 0.5 * (qe[2] * qe[2] + qe[3] * qe[3]) * re);
          const double ux = qe[2] * re, uy = qe[3] * re;
          side(qe, pe, re, fn_e);
          lam_e = sqrt(ux * ux + uy * uy) + sqrt(p0 * (pe * re));
        }
        const double lam = fmax(lam_i, lam_e);
        const double nn = nx * nx + ny * ny;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const double fk = 0.5 * (fn_i[k] + fn_e[k]) - 0.5 * lam * (qe[k] - qi[k]) * nn;
          out[k * FS] = -scale * fk;
        }
      } else {  // DG_MAXWELL, TM
        if (bdry) {  // PEC: exterior (-E, H)
          qe[0] = -qi[0];
          qe[1] = qi[1];
          qe[2] = qi[2];
        }
        const double alpha = p0, z = a.k[0], y = a.k[1];
        const double jez = qe[0] - qi[0], jhx = qe[1] - qi[1], jhy = qe[2] - qi[2];
        // t_e = z j_H - alpha n x j_E,  t_h = y j_E + alpha n x j_H (3-vectors
        // with n_z = 0; only the components the TM fields need)
        const double tex = z * jhx - alpha * (ny * jez);
        const double tey = z * jhy + alpha * (nx * jez);
        const double thz = y * jez + alpha * (nx * jhy - ny * jhx);
        const double fez = nx * tey - ny * tex;  // (n x t_e)_z
        const double fhx = ny * thz;             // (n x t_h)_x
        const double fhy = -nx * thz;            // (n x t_h)_y
        out[0 * FS] = -scale * (a.k[2] * fez);
        out[1 * FS] = -scale * (a.k[3] * fhx);
        out[2 * FS] = -scale * (a.k[3] * fhy);
      }
    }
    __syncthreads();
    // }}}

    // {{{ 5. LIFT, then store or fold into the RK stage
    if (active && el < ecount) {
      const double* fl = sFlux + el * NFPT;
      int64_t gidx = e0 * NP + (el * NP + i);  // advanced by nelnp per field
#pragma unroll
      for (int k = 0; k < NF; ++k, gidx += nelnp) {
        double acc = vol[k];
#pragma unroll 4
        for (int fj = 0; fj < NFPT; ++fj) acc = fma(sL[fj * NP + i], fl[k * E * NFPT + fj], acc);
        if constexpr (EQ == DG_MAXWELL) acc *= (k == 0 ? a.k[4] : a.k[5]);
        double val = acc;
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
