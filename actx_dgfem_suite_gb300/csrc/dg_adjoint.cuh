// Hand-written adjoint (transpose) of the FP64 wave RHS on affine tetrahedra.
//
// With the forward operator written per element as
//   rhs_u = -sum_r W_r (G v)_r + sum_f s_f LIFT_f F_u
//   rhs_v = -G^T (W_r u)       + sum_f s_f LIFT_f n F_v
//   F_u = 1/2 (v- + v+).n + 1/2 (u+ - u-),   F_v = 1/2 (u- + u+) + 1/2 (v+ - v-).n
// (actx_dgfem_suite/equations/wave.py:80-200, c folded into a per-element
// scale), its transpose y = L^T x is evaluated in two launches:
//
//   1. dg_wave_adjoint_volume: per element, the volume transpose (the forward
//      volume formulas with W_r replaced by W_r^T, which swaps the roles of the
//      divergence and the gradient) into y, and the lifted face adjoints
//        abar_u(f, j) = s_f sum_i LIFT[i][f][j] x_u[i]
//        abar_v(f, j) = s_f sum_i LIFT[i][f][j] (n_f . x_v[i])
//      into a face-point scratch buffer (Nel, 2, 4 Nfp).
//   2. dg_wave_adjoint_surface: per node, the transpose of the flux and of the
//      face gather.  A face point's exterior contribution belongs to the
//      neighbour's node; instead of scattering it (atomics, order-dependent
//      rounding), every node gathers it from the glued partner face point
//      (face_partner index), so the result is deterministic.
//
// The plan's scalar wave speed c and an optional per-element scale c_e
// (variable wave speed, L = c diag(c_e) L_1) are applied to x on load:
// L^T x = L_1^T (c c_e x).
//
// STAGE = true is one stage s of the reverse sweep of a low-storage
// Runge-Kutta step, fused around the transpose (the forward stage is
// r^s = a_s r^{s-1} + dt L(q^(s)), q^(s+1) = q^(s) + b_s r^s):
//   rbar_s   = xscale x                      (the stage's residual adjoint)
//   lam     += dt L^T rbar_s                 (state adjoint, in place)
//   rbar_out = a_s rbar_s + b_{s-1} lam      (the next stage's rbar; may alias x)
//   cbar_e  += dt <rbar_s, lq>_e             (gradient wrt c_e; lq = c L_1 q^(s),
//                                             the forward stage's RHS before c_e)
// The volume kernel reduces each element's inner product in a fixed order
// and the surface kernel applies the epilogue at every node, so the stage is
// deterministic and needs no atomics.
#pragma once

#include "dg_rhs.cuh"

namespace dg {

struct AdjArgs {
  const double* x;          // (4, Nel, Np)
  double* y;                // (4, Nel, Np)
  double* face_scratch;     // (Nel, 2, 4 Nfp)
  const double* elem_scale; // (Nel) or NULL
  double c;                 // the plan's scalar wave speed
  const double* metric;
  const double* face_geom;
  const int32_t* face_partner;  // (Nel, 4, Nfp) flat face-point index, -1 = boundary
  const void* ops;          // adjoint operator block, see AdjOpsLayout
  uint32_t ops_bytes;
  int64_t nel;
  int* status;
  // STAGE (fused reverse RK stage) only
  double xscale;            // rbar_s = xscale x
  double* lam;              // (4, Nel, Np), updated in place
  double* rbar_out;         // (4, Nel, Np) or NULL; may be x itself
  const double* lq;         // (4, Nel, Np) or NULL
  double* cbar;             // (Nel) or NULL
  double rk_a, rk_b, dt;
};

// [W (3 Np Np, [r][i][j]: the forward layout of W^T) | LIFT ([i][fj]) | face_nodes]
template <int N>
struct AdjOpsLayout {
  static constexpr int NP = Shape<N>::NP, NFPT = Shape<N>::NFPT;
  static constexpr int W = 0;
  static constexpr int L = W + pad16(3 * NP * NP * 8);
  static constexpr int FN = L + pad16(NFPT * NP * 8);
  static constexpr int SIZE = FN + pad16(NFPT * 4);
};

template <int N>
struct AdjTile {
  static constexpr int NP = Shape<N>::NP, NFPT = Shape<N>::NFPT;
  static constexpr int E = kBlock / NP;
  static constexpr int X = AdjOpsLayout<N>::SIZE;
  static constexpr int AUX = X + pad16(4 * E * NP * 8);
  static constexpr int GEO = AUX + pad16(3 * E * NP * 8);
  static constexpr int FGEO = GEO + pad16(9 * E * 8);
  static constexpr int VN = FGEO + pad16(16 * E * 8);  // n_f . x_v per face, node
  static constexpr int PART = VN + pad16(4 * E * NP * 8);  // STAGE: <rbar, lq> per node
  static constexpr int SMEM_BYTES = PART + pad16(E * NP * 8);
};

template <int N, bool STAGE>
__global__ void __launch_bounds__(kBlock) dg_wave_adjoint_volume(const AdjArgs a) {
  using T = AdjTile<N>;
  using Ops = AdjOpsLayout<N>;
  constexpr int NP = T::NP, NFPT = T::NFPT, E = T::E;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ int ops_ok;
  const double* sW = reinterpret_cast<const double*>(smem + Ops::W);
  const double* sL = reinterpret_cast<const double*>(smem + Ops::L);
  double* sX = reinterpret_cast<double*>(smem + T::X);
  double* sAux = reinterpret_cast<double*>(smem + T::AUX);
  double* sG = reinterpret_cast<double*>(smem + T::GEO);
  double* sFG = reinterpret_cast<double*>(smem + T::FGEO);
  double* sVN = reinterpret_cast<double*>(smem + T::VN);
  double* sPart = reinterpret_cast<double*>(smem + T::PART);

  const int t = threadIdx.x;
  if (t == 0) {
    mbar_init(&bar, 1);
    mbar_arrive_expect_tx(&bar, a.ops_bytes);
    bulk_g2s(smem, a.ops, a.ops_bytes, &bar);
    const bool ok = mbar_wait_bounded(&bar, 0);
    if (!ok) {
      raise_status(a.status, DG_ERR_TIMEOUT);
      mbar_wait_bounded(&bar, 0);
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

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t e0 = tile * E;
    const int ecount = (nel - e0) < (int64_t)E ? (int)(nel - e0) : E;
    {
      const double* xk = a.x + e0 * NP;
      const double* lk = STAGE && a.lq ? a.lq + e0 * NP : nullptr;
      const double* sc_t = a.elem_scale ? a.elem_scale + e0 : nullptr;
      const double xs = STAGE ? a.xscale : 1.0;
      double part[(E * NP + kBlock - 1) / kBlock];  // this thread's <rbar, lq> terms
#pragma unroll
      for (int r = 0; r < (E * NP + kBlock - 1) / kBlock; ++r) part[r] = 0.0;
#pragma unroll
      for (int k = 0; k < 4; ++k, xk += nelnp) {
#pragma unroll
        for (int r = 0; r < (E * NP + kBlock - 1) / kBlock; ++r) {
          const int rem = t + r * kBlock;
          if (rem >= E * NP) break;
          double v = 0.0;
          if (rem < ecount * NP) {
            const double rb = xs * __ldg(xk + rem);
            if (lk) part[r] = fma(rb, __ldg(lk + k * nelnp + rem), part[r]);
            v = a.c * rb;
            if (sc_t) v *= __ldg(sc_t + rem / NP);
          }
          sX[k * (E * NP) + rem] = v;
        }
      }
      if (STAGE && lk) {
#pragma unroll
        for (int r = 0; r < (E * NP + kBlock - 1) / kBlock; ++r) {
          const int rem = t + r * kBlock;
          if (rem < E * NP) sPart[rem] = part[r];
        }
      }
      const double* mt = a.metric + e0 * 9;
      const double* ft = a.face_geom + e0 * 16;
      for (int idx = t; idx < 9 * E; idx += kBlock)
        sG[idx] = idx < 9 * ecount ? __ldg(mt + idx) : 0.0;
      for (int idx = t; idx < 16 * E; idx += kBlock)
        sFG[idx] = idx < 16 * ecount ? __ldg(ft + idx) : 0.0;
    }
    __syncthreads();

    if (STAGE && a.lq && a.cbar && active && el < ecount && i == 0) {
      double g = 0.0;  // the element's <rbar_s, lq>, fixed order
      for (int j = 0; j < NP; ++j) g += sPart[el * NP + j];
      a.cbar[e0 + el] += a.dt * g;
    }

    if (active && el < ecount) {
      const double* G = sG + el * 9;
      const double v0 = sX[(1 * E + el) * NP + i];
      const double v1 = sX[(2 * E + el) * NP + i];
      const double v2 = sX[(3 * E + el) * NP + i];
#pragma unroll
      for (int r = 0; r < 3; ++r)
        sAux[(r * E + el) * NP + i] =
            fma(G[r * 3 + 0], v0, fma(G[r * 3 + 1], v1, G[r * 3 + 2] * v2));
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        const double* fg = sFG + (el * 4 + f) * 4;
        sVN[(el * 4 + f) * NP + i] = fma(fg[0], v0, fma(fg[1], v1, fg[2] * v2));
      }
    }
    __syncthreads();

    // volume transpose: the forward volume code with W^T
    if (active && el < ecount) {
      const double* G = sG + el * 9;
      const double* u = sX + el * NP;
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
      double* yk = a.y + e0 * NP + (el * NP + i);
      *yk = -dv;
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        yk += nelnp;
        *yk = -fma(G[0 * 3 + x], ur0, fma(G[1 * 3 + x], ur1, G[2 * 3 + x] * ur2));
      }
    }

    // lifted face adjoints
    for (int pidx = t; pidx < ecount * NFPT; pidx += kBlock) {
      const int elp = pidx / NFPT;
      const int fj = pidx - elp * NFPT;
      const int f = fj / Shape<N>::NFP;
      const double s = sFG[(elp * 4 + f) * 4 + 3];
      double au = 0.0, av = 0.0;
      const double* xu = sX + (0 * E + elp) * NP;
      const double* vn = sVN + (elp * 4 + f) * NP;
#pragma unroll 4
      for (int ii = 0; ii < NP; ++ii) {
        const double l = sL[ii * NFPT + fj];
        au = fma(l, xu[ii], au);
        av = fma(l, vn[ii], av);
      }
      double* sc = a.face_scratch + e0 * (2 * NFPT) + elp * (2 * NFPT);
      sc[fj] = s * au;
      sc[NFPT + fj] = s * av;
    }
    __syncthreads();
  }
}

// One thread per node: add the transposed flux and face-gather contributions
// (STAGE: then the reverse-stage epilogue at every node).
// Index arithmetic stays in 32 bits (Nel * 4 Nfp < 2^31 is checked on the
// host): on GB300 wide integer multiplies compete with FP64 for a narrow pipe.
template <int N, bool STAGE>
__global__ void __launch_bounds__(kBlock) dg_wave_adjoint_surface(const AdjArgs a) {
  using Ops = AdjOpsLayout<N>;
  constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP, NFPT = Shape<N>::NFPT;
  // face points of every volume node (a node lies on at most 3 faces)
  __shared__ int sNodeFP[NP][3];
  if (threadIdx.x < NP) {
    const int* gFN = reinterpret_cast<const int*>(
        static_cast<const unsigned char*>(a.ops) + Ops::FN);
    int cnt = 0;
    for (int fj = 0; fj < NFPT; ++fj)
      if (gFN[fj] == (int)threadIdx.x && cnt < 3) sNodeFP[threadIdx.x][cnt++] = fj;
    for (; cnt < 3; ++cnt) sNodeFP[threadIdx.x][cnt] = -1;
  }
  __syncthreads();
  const uint32_t nelnp = (uint32_t)(a.nel * NP);
  const uint32_t nfpt_total = (uint32_t)(a.nel * NFPT);
  double* yu_p = a.y;
  double* y0_p = a.y + nelnp;
  double* y1_p = y0_p + nelnp;
  double* y2_p = y1_p + nelnp;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < nelnp;
       g += gridDim.x * blockDim.x) {
    const uint32_t e = g / NP;
    const int i = (int)(g - e * NP);
    if (!STAGE && sNodeFP[i][0] < 0) continue;  // interior node: volume part only
    double yu = yu_p[g], y0 = y0_p[g], y1 = y1_p[g], y2 = y2_p[g];
    const double* sc = a.face_scratch + e * (2 * NFPT);
    const double* fge = a.face_geom + e * 16;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const int fj = sNodeFP[i][m];
      if (fj < 0) break;
      const double* fg = fge + (fj / NFP) * 4;
      const double au = sc[fj], av = sc[NFPT + fj];
      const int32_t p = a.face_partner[e * NFPT + fj];
      if (p < 0) {
        // own flux with the boundary mirror u+ = -u-, v+ = v- folded in:
        // d/du- = -abar_u, d/dv- = n abar_u
        yu -= au;
        y0 = fma(fg[0], au, y0);
        y1 = fma(fg[1], au, y1);
        y2 = fma(fg[2], au, y2);
      } else if ((uint32_t)p < nfpt_total) {
        // own flux, interior-trace derivatives
        const double d = 0.5 * (av - au);
        yu += d;
        y0 = fma(-fg[0], d, y0);
        y1 = fma(-fg[1], d, y1);
        y2 = fma(-fg[2], d, y2);
        // the glued partner's flux depends on this node as its exterior trace
        const uint32_t pe = (uint32_t)p / NFPT;
        const int pfj = p - (int32_t)(pe * NFPT);
        const double* psc = a.face_scratch + pe * (2 * NFPT);
        const double sp = 0.5 * (psc[pfj] + psc[NFPT + pfj]);
        const double* pg = a.face_geom + pe * 16 + (pfj / NFP) * 4;
        yu += sp;
        y0 = fma(pg[0], sp, y0);
        y1 = fma(pg[1], sp, y1);
        y2 = fma(pg[2], sp, y2);
      } else {
        raise_status(a.status, DG_ERR_INDEX);
      }
    }
    if constexpr (STAGE) {
      // read x and lam of this node before writing: rbar_out may be x and x
      // may be lam (the first reverse stage reads rbar from lam)
      const double y[4] = {yu, y0, y1, y2};
      double rb[4], ln[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        rb[k] = a.xscale * a.x[k * nelnp + g];
        ln[k] = fma(a.dt, y[k], a.lam[k * nelnp + g]);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) a.lam[k * nelnp + g] = ln[k];
      if (a.rbar_out) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          a.rbar_out[k * nelnp + g] = fma(a.rk_a, rb[k], a.rk_b * ln[k]);
      }
    } else {
      yu_p[g] = yu;
      y0_p[g] = y0;
      y1_p[g] = y1;
      y2_p[g] = y2;
    }
  }
}

}  // namespace dg
