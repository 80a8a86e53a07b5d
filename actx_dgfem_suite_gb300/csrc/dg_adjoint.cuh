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
  static constexpr int SMEM_BYTES = VN + pad16(4 * E * NP * 8);
};

template <int N>
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
    for (int idx = t; idx < 4 * E * NP; idx += kBlock) {
      const int k = idx / (E * NP);
      const int rem = idx - k * (E * NP);
      double v = 0.0;
      if (rem < ecount * NP) {
        v = a.c * __ldg(a.x + k * nelnp + e0 * NP + rem);
        if (a.elem_scale) v *= __ldg(a.elem_scale + e0 + rem / NP);
      }
      sX[idx] = v;
    }
    for (int idx = t; idx < 9 * E; idx += kBlock)
      sG[idx] = idx < 9 * ecount ? __ldg(a.metric + e0 * 9 + idx) : 0.0;
    for (int idx = t; idx < 16 * E; idx += kBlock)
      sFG[idx] = idx < 16 * ecount ? __ldg(a.face_geom + e0 * 16 + idx) : 0.0;
    __syncthreads();

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
      const int64_t g = (e0 + el) * NP + i;
      a.y[0 * nelnp + g] = -dv;
#pragma unroll
      for (int x = 0; x < 3; ++x)
        a.y[(1 + x) * nelnp + g] =
            -fma(G[0 * 3 + x], ur0, fma(G[1 * 3 + x], ur1, G[2 * 3 + x] * ur2));
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
      double* sc = a.face_scratch + (e0 + elp) * 2 * NFPT;
      sc[fj] = s * au;
      sc[NFPT + fj] = s * av;
    }
    __syncthreads();
  }
}

// One thread per node: add the transposed flux and face-gather contributions.
template <int N>
__global__ void __launch_bounds__(kBlock) dg_wave_adjoint_surface(const AdjArgs a) {
  using Ops = AdjOpsLayout<N>;
  constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP, NFPT = Shape<N>::NFPT;
  __shared__ int sFN[NFPT];
  const int* gFN = reinterpret_cast<const int*>(
      static_cast<const unsigned char*>(a.ops) + Ops::FN);
  for (int k = threadIdx.x; k < NFPT; k += blockDim.x) sFN[k] = gFN[k];
  __syncthreads();
  const int64_t nelnp = a.nel * NP;
  const int64_t nfpt_total = a.nel * NFPT;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < nelnp;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = g / NP;
    const int i = (int)(g - e * NP);
    double yu = a.y[g], y0 = a.y[nelnp + g], y1 = a.y[2 * nelnp + g],
           y2 = a.y[3 * nelnp + g];
    const double* sc = a.face_scratch + e * 2 * NFPT;
    for (int fj = 0; fj < NFPT; ++fj) {
      if (sFN[fj] != i) continue;
      const int f = fj / NFP;
      const double* fg = a.face_geom + (e * 4 + f) * 4;
      const double nx = fg[0], ny = fg[1], nz = fg[2];
      const double au = sc[fj], av = sc[NFPT + fj];
      // own face point, interior-trace derivatives
      yu += -0.5 * au + 0.5 * av;
      const double cv = 0.5 * au - 0.5 * av;
      y0 += nx * cv;
      y1 += ny * cv;
      y2 += nz * cv;
      const int32_t p = a.face_partner[e * NFPT + fj];
      if (p < 0) {
        // boundary mirror: u+ = -u-, v+ = v-
        yu += -(0.5 * au + 0.5 * av);
        const double cb = 0.5 * au + 0.5 * av;
        y0 += nx * cb;
        y1 += ny * cb;
        y2 += nz * cb;
      } else if ((int64_t)p < nfpt_total) {
        // the partner's flux depends on this node as its exterior trace
        const int64_t pe = p / NFPT;
        const int pfj = p - (int)(pe * NFPT);
        const double* psc = a.face_scratch + pe * 2 * NFPT;
        const double pu = psc[pfj], pv = psc[NFPT + pfj];
        const double* pg = a.face_geom + (pe * 4 + pfj / NFP) * 4;
        yu += 0.5 * pu + 0.5 * pv;
        const double cp = 0.5 * pu + 0.5 * pv;
        y0 += pg[0] * cp;
        y1 += pg[1] * cp;
        y2 += pg[2] * cp;
      } else {
        raise_status(a.status, DG_ERR_INDEX);
      }
    }
    a.y[g] = yu;
    a.y[nelnp + g] = y0;
    a.y[2 * nelnp + g] = y1;
    a.y[3 * nelnp + g] = y2;
  }
}

}  // namespace dg
