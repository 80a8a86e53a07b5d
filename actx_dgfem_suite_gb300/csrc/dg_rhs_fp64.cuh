// Fused FP64 DG-FEM RHS kernel for affine tetrahedra on sm_103a.
//
// One persistent launch evaluates the whole RHS of one equation.  Each CTA
// stages the reference operators (weak or strong D_r and LIFT, with the face
// node table) into shared memory once, by a single TMA bulk copy, then loops
// over tiles of E = 256 / Np elements:
//
//   1. load the tile's state (all fields) and geometry into shared memory;
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
//      term and stored.
//
// The flux formulas follow actx_dgfem_suite/equations/wave.py:80-114 (wave),
// grudge's euler_numerical_flux with LF stabilisation and InviscidWallBC
// (configured at equations/euler.py:168-174) and grudge's MaxwellOperator
// alpha-flux with PEC (configured at equations/maxwell.py:55-59).
#pragma once

#include "dg_common.cuh"

namespace dg {

struct RhsArgs {
  const double* q;
  double* rhs;
  const double* metric;
  const double* face_geom;
  const uint32_t* gather;
  const double* ops;       // [Wt | Lt | face_nodes], see OpsLayout
  uint32_t ops_bytes;
  int64_t nel;
  int* status;
  double p0, p1, p2;       // equation parameters
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

constexpr int pad2(int n) { return (n + 1) & ~1; }  // doubles -> 16 B multiple

// Layout of the operator block, identical in global and shared memory.
template <int N>
struct OpsLayout {
  static constexpr int NP = Shape<N>::NP, NFPT = Shape<N>::NFPT;
  static constexpr int W = 0;                       // Wt[r][j][i]
  static constexpr int L = W + pad2(3 * NP * NP);   // Lt[fj][i]
  static constexpr int FN = L + pad2(NFPT * NP);    // int32 face_nodes[fj]
  static constexpr int SIZE = FN + pad2((NFPT + 1) / 2);  // in doubles
};

template <int N, int EQ>
struct Tile {
  static constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP,
                       NFPT = Shape<N>::NFPT;
  static constexpr int NF = EqInfo<EQ>::NF, NAUX = EqInfo<EQ>::NAUX;
  static constexpr int E = kBlock / NP;
  static constexpr int Q = OpsLayout<N>::SIZE;
  static constexpr int AUX = Q + pad2(NF * E * NP);
  static constexpr int FLUX = AUX + pad2(NAUX * E * NP);
  static constexpr int GEO = FLUX + pad2(NF * E * NFPT);
  static constexpr int FGEO = GEO + pad2(9 * E);
  static constexpr int SIZE = FGEO + pad2(16 * E);
  static constexpr int SMEM_BYTES = SIZE * 8;
};

template <int N, int EQ>
__global__ void __launch_bounds__(kBlock)
    dg_rhs_fp64_kernel(const RhsArgs a) {
  using T = Tile<N, EQ>;
  constexpr int NP = T::NP, NFPT = T::NFPT, NF = T::NF, E = T::E;
  extern __shared__ __align__(128) double smem[];
  __shared__ uint64_t bar;
  __shared__ int ops_ok;

  const double* sW = smem + OpsLayout<N>::W;
  const double* sL = smem + OpsLayout<N>::L;
  const int* sFN = reinterpret_cast<const int*>(smem + OpsLayout<N>::FN);
  double* sQ = smem + T::Q;
  double* sAux = smem + T::AUX;
  double* sFlux = smem + T::FLUX;
  double* sG = smem + T::GEO;
  double* sFG = smem + T::FGEO;

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
  const double p0 = a.p0, p1 = a.p1, p2 = a.p2;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t e0 = tile * E;
    const int ecount = (nel - e0) < (int64_t)E ? (int)(nel - e0) : E;

    // {{{ 1. state and geometry -> shared memory (coalesced)
    for (int idx = t; idx < NF * E * NP; idx += kBlock) {
      const int k = idx / (E * NP);
      const int rem = idx - k * (E * NP);
      sQ[idx] = rem < ecount * NP ? __ldg(a.q + k * nelnp + e0 * NP + rem) : 0.0;
    }
    for (int idx = t; idx < 9 * E; idx += kBlock)
      sG[idx] = idx < 9 * ecount ? __ldg(a.metric + e0 * 9 + idx) : 0.0;
    for (int idx = t; idx < 16 * E; idx += kBlock)
      sFG[idx] = idx < 16 * ecount ? __ldg(a.face_geom + e0 * 16 + idx) : 0.0;
    __syncthreads();
    // }}}

    // {{{ 2. pointwise pre-pass
    if constexpr (EQ == DG_WAVE) {
      if (active && el < ecount) {
        const double* G = sG + el * 9;
        const double v0 = sQ[(1 * E + el) * NP + i];
        const double v1 = sQ[(2 * E + el) * NP + i];
        const double v2 = sQ[(3 * E + el) * NP + i];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          sAux[(r * E + el) * NP + i] =
              fma(G[r * 3 + 0], v0, fma(G[r * 3 + 1], v1, G[r * 3 + 2] * v2));
      }
    } else if constexpr (EQ == DG_EULER) {
      if (active && el < ecount) {
        const double gamma = p0;
        const double* G = sG + el * 9;
        const double rho = sQ[(0 * E + el) * NP + i];
        const double en = sQ[(1 * E + el) * NP + i];
        const double m[3] = {sQ[(2 * E + el) * NP + i], sQ[(3 * E + el) * NP + i],
                             sQ[(4 * E + el) * NP + i]};
        const double rinv = 1.0 / rho;
        const double u[3] = {m[0] * rinv, m[1] * rinv, m[2] * rinv};
        const double p =
            (gamma - 1.0) * (en - 0.5 * (m[0] * m[0] + m[1] * m[1] + m[2] * m[2]) * rinv);
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
            sAux[((k * 3 + r) * E + el) * NP + i] =
                fma(G[r * 3 + 0], F[k][0],
                    fma(G[r * 3 + 1], F[k][1], G[r * 3 + 2] * F[k][2]));
      }
    }
    if constexpr (T::NAUX > 0) __syncthreads();
    // }}}

    // {{{ 3. volume term (registers)
    double vol[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) vol[k] = 0.0;
    if (active && el < ecount) {
      const double* G = sG + el * 9;
      if constexpr (EQ == DG_WAVE) {
        const double c = p0;
        const double* u = sQ + el * NP;
        double ur0 = 0.0, ur1 = 0.0, ur2 = 0.0, dv = 0.0;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const double w0 = sW[(0 * NP + j) * NP + i];
          const double w1 = sW[(1 * NP + j) * NP + i];
          const double w2 = sW[(2 * NP + j) * NP + i];
          const double uj = u[j];
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
          const double w0 = sW[(0 * NP + j) * NP + i];
          const double w1 = sW[(1 * NP + j) * NP + i];
          const double w2 = sW[(2 * NP + j) * NP + i];
#pragma unroll
          for (int k = 0; k < 5; ++k)
            vol[k] = fma(w0, sAux[((k * 3 + 0) * E + el) * NP + j],
                         fma(w1, sAux[((k * 3 + 1) * E + el) * NP + j],
                             fma(w2, sAux[((k * 3 + 2) * E + el) * NP + j],
                                 vol[k])));
        }
      } else {  // DG_MAXWELL: strong derivatives, curl
        double d[6][3];
#pragma unroll
        for (int k = 0; k < 6; ++k) d[k][0] = d[k][1] = d[k][2] = 0.0;
#pragma unroll
        for (int j = 0; j < NP; ++j) {
          const double w0 = sW[(0 * NP + j) * NP + i];
          const double w1 = sW[(1 * NP + j) * NP + i];
          const double w2 = sW[(2 * NP + j) * NP + i];
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            const double qj = sQ[(k * E + el) * NP + j];
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

    // {{{ 4. face gather + numerical flux
    for (int pidx = t; pidx < ecount * NFPT; pidx += kBlock) {
      const int elp = pidx / NFPT;
      const int fj = pidx - elp * NFPT;
      const int f = fj / Shape<N>::NFP;
      const int node = sFN[fj];
      uint32_t g = __ldg(a.gather + (e0 + elp) * NFPT + fj);
      bool bdry = (g >> 31) != 0u;
      int64_t gi = (int64_t)(g & 0x7fffffffu);
      if (gi >= nelnp) {  // never read out of bounds
        raise_status(a.status, DG_ERR_INDEX);
        gi = (e0 + elp) * NP + node;
      }
      const double* fg = sFG + (elp * 4 + f) * 4;
      const double nx = fg[0], ny = fg[1], nz = fg[2], scale = fg[3];
      double qi[NF], qe[NF];
#pragma unroll
      for (int k = 0; k < NF; ++k) qi[k] = sQ[(k * E + elp) * NP + node];
      if (!bdry) {
#pragma unroll
        for (int k = 0; k < NF; ++k) qe[k] = __ldg(a.q + k * nelnp + gi);
      }
      double* out = sFlux + elp * NFPT + fj;
      constexpr int FS = E * NFPT;  // field stride in sFlux

      if constexpr (EQ == DG_WAVE) {
        const double c = p0;
        if (bdry) {  // Dirichlet mirror: exterior (-u, v)
          qe[0] = -qi[0];
          qe[1] = qi[1];
          qe[2] = qi[2];
          qe[3] = qi[3];
        }
        const double vavg_n = 0.5 * (qi[1] + qe[1]) * nx + 0.5 * (qi[2] + qe[2]) * ny +
                              0.5 * (qi[3] + qe[3]) * nz;
        const double uavg = 0.5 * (qi[0] + qe[0]);
        const double vjump = (qe[1] - qi[1]) * nx + (qe[2] - qi[2]) * ny +
                             (qe[3] - qi[3]) * nz;
        const double fu = c * (vavg_n + 0.5 * (qe[0] - qi[0]));
        const double fv = c * (uavg + 0.5 * vjump);
        out[0 * FS] = scale * fu;
        out[1 * FS] = scale * (fv * nx);
        out[2 * FS] = scale * (fv * ny);
        out[3 * FS] = scale * (fv * nz);
      } else if constexpr (EQ == DG_EULER) {
        const double gamma = p0;
        if (bdry) {  // InviscidWallBC: mirror the normal momentum
          const double mn = qi[2] * nx + qi[3] * ny + qi[4] * nz;
          qe[0] = qi[0];
          qe[1] = qi[1];
          qe[2] = qi[2] - 2.0 * nx * mn;
          qe[3] = qi[3] - 2.0 * ny * mn;
          qe[4] = qi[4] - 2.0 * nz * mn;
        }
        double fn_i[5], fn_e[5], lam_i, lam_e;
        auto side = [&](const double* q, double* fn, double& lam) {
          const double rinv = 1.0 / q[0];
          const double ux = q[2] * rinv, uy = q[3] * rinv, uz = q[4] * rinv;
          const double p = (gamma - 1.0) *
                           (q[1] - 0.5 * (q[2] * q[2] + q[3] * q[3] + q[4] * q[4]) * rinv);
          const double un = ux * nx + uy * ny + uz * nz;
          fn[0] = q[2] * nx + q[3] * ny + q[4] * nz;
          fn[1] = un * (q[1] + p);
          fn[2] = q[2] * un + p * nx;
          fn[3] = q[3] * un + p * ny;
          fn[4] = q[4] * un + p * nz;
          lam = sqrt(ux * ux + uy * uy + uz * uz) + sqrt(gamma * (p * rinv));
        };
        side(qi, fn_i, lam_i);
        side(qe, fn_e, lam_e);
        const double lam = fmax(lam_i, lam_e);
        const double nn = nx * nx + ny * ny + nz * nz;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const double fk = 0.5 * (fn_i[k] + fn_e[k]) - 0.5 * lam * (qe[k] - qi[k]) * nn;
          out[k * FS] = -scale * fk;
        }
      } else {  // DG_MAXWELL
        const double alpha = p0, eps = p1, mu = p2;
        if (bdry) {  // PEC: exterior (-E, H)
          qe[0] = -qi[0];
          qe[1] = -qi[1];
          qe[2] = -qi[2];
          qe[3] = qi[3];
          qe[4] = qi[4];
          qe[5] = qi[5];
        }
        const double z = sqrt(mu / eps), y = 1.0 / z;
        const double je[3] = {qe[0] - qi[0], qe[1] - qi[1], qe[2] - qi[2]};
        const double jh[3] = {qe[3] - qi[3], qe[4] - qi[4], qe[5] - qi[5]};
        const double n[3] = {nx, ny, nz};
        auto cross = [](const double* a_, const double* b_, double* c_) {
          c_[0] = a_[1] * b_[2] - a_[2] * b_[1];
          c_[1] = a_[2] * b_[0] - a_[0] * b_[2];
          c_[2] = a_[0] * b_[1] - a_[1] * b_[0];
        };
        double nxe[3], nxh[3], te[3], th[3], fe[3], fh[3];
        cross(n, je, nxe);
        cross(n, jh, nxh);
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          te[x] = z * jh[x] - alpha * nxe[x];
          th[x] = y * je[x] + alpha * nxh[x];
        }
        cross(n, te, fe);
        cross(n, th, fh);
        const double ce = -1.0 / (z + z), ch = 1.0 / (y + y);
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          out[x * FS] = -scale * (ce * fe[x]);
          out[(3 + x) * FS] = -scale * (ch * fh[x]);
        }
      }
    }
    __syncthreads();
    // }}}

    // {{{ 5. LIFT + store
    if (active && el < ecount) {
      const double* fl = sFlux + el * NFPT;
#pragma unroll
      for (int k = 0; k < NF; ++k) {
        double acc = vol[k];
#pragma unroll 4
        for (int fj = 0; fj < NFPT; ++fj)
          acc = fma(sL[fj * NP + i], fl[k * E * NFPT + fj], acc);
        if constexpr (EQ == DG_MAXWELL) acc = acc / (k < 3 ? p1 : p2);
        a.rhs[k * nelnp + (e0 + el) * NP + i] = acc;
      }
    }
    __syncthreads();
    // }}}
  }
}

}  // namespace dg
