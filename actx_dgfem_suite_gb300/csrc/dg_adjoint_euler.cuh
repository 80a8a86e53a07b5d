// Transposed Jacobian of the FP64 Euler RHS: y = (dL/dq (q))^T x.
//
// The forward operator (weak form, per element, Lax-Friedrichs flux and
// inviscid wall as configured at actx_dgfem_suite/equations/euler.py:168-174):
//   L_k(i) = sum_r sum_j W_r[i][j] sum_x G[r][x] F_{k,x}(q_j)
//            + sum_fj LIFT[i][fj] Phi_k(fj),
//   Phi = -s_f f*,  f* = 1/2 (F(q-) + F(q+)).n - 1/2 lam |n|^2 (q+ - q-),
//   lam = max(|u| + c)(q-, q+).
// Its transpose, in four launches:
//   1. dg_euler_aux_kernel (forward code): p, 1/rho, |u| + c per node of q;
//   2. dg_euler_vjp_volume: per element, T_{r,k} = W_r^T x_k, Z_{x,k} =
//      sum_r G[r][x] T_{r,k}, y(j) = sum_x J_x(q_j)^T Z_x(j) (J_x the flux
//      Jacobian in direction x), and the lifted adjoints w_k(fj) = sum_i
//      LIFT[i][fj] x_k(i) into the face scratch;
//   3. dg_euler_vjp_face: one thread per point of an owned face (as the
//      forward face kernel): the flux adjoint fbar = -s_o w_o + s_p w_p (the
//      glued point's LIFT sees -f*), then d f*/d q-^T fbar and d f*/d q+^T
//      fbar written back to the two face points' scratch slots (for a wall,
//      the mirror q+ = M q- folds the exterior part into the interior);
//   4. dg_vjp_node_gather: each volume node adds its face points' slots
//      (deterministic: every slot is written by exactly one thread and
//      gathered, never scattered with atomics).
// The derivative of max(lam-, lam+) follows the side the forward picks
// (lam- >= lam+ takes the interior side).
#pragma once

#include "dg_adjoint.cuh"
#include "dg_face.cuh"

namespace dg {

struct VjpArgs {
  const double* q;          // (5, Nel, Np) linearisation state
  const double* x;          // (5, Nel, Np) adjoint input
  double* y;                // (5, Nel, Np) output
  const double* aux;        // (3, Nel, Np) p, 1/rho, |u| + c of q
  double* scratch;          // (5, Nel, 4 Nfp) face-point scratch
  const double* elem_scale; // (Nel) factor of the forward RHS, or NULL
  const double* metric;
  const double* face_geom;
  const uint32_t* gather;
  const int32_t* partner;
  const int32_t* owned;
  int64_t nowned;
  const void* ops;          // adjoint operator block (AdjOpsLayout)
  uint32_t ops_bytes;
  int64_t nel;
  int* status;
  double gamma;
  // reverse-stage epilogue of the node gather (dg_rhs_vjp_stage): with
  // rbar = xscale x, lam += dt J^T rbar and rbar_out = rk_a rbar + rk_b lam
  double xscale;
  double* lam;
  double* rbar_out;         // or NULL
  double rk_a, rk_b, dt;
};

// g = J_n(q)^T z for the Euler flux F(q).n: q = (rho, E, m), rinv = 1/rho,
// p the pressure; n need not be a unit vector
__device__ __forceinline__ void euler_flux_vjp(const double* q, double rinv, double p,
                                               double nx, double ny, double nz,
                                               const double* z, double gamma,
                                               double* g) {
  const double gm1 = gamma - 1.0;
  const double u0 = q[2] * rinv, u1 = q[3] * rinv, u2 = q[4] * rinv;
  const double un = u0 * nx + u1 * ny + u2 * nz;
  const double q2 = u0 * u0 + u1 * u1 + u2 * u2;
  const double H = (q[1] + p) * rinv;
  const double zmn = z[2] * nx + z[3] * ny + z[4] * nz;
  const double zmu = z[2] * u0 + z[3] * u1 + z[4] * u2;
  const double hq2 = 0.5 * gm1 * q2;
  g[0] = z[1] * un * (hq2 - H) - un * zmu + zmn * hq2;
  g[1] = z[1] * gamma * un + gm1 * zmn;
  const double s = z[0] + z[1] * H + zmu;
  const double a = z[1] * gm1 * un + gm1 * zmn;
  g[2] = nx * s - a * u0 + z[2] * un;
  g[3] = ny * s - a * u1 + z[3] * un;
  g[4] = nz * s - a * u2 + z[4] * un;
}

// gradient of lam = |u| + c with respect to q (|u| = 0: the zero subgradient)
__device__ __forceinline__ void euler_speed_grad(const double* q, double rinv, double p,
                                                 double gamma, double* dl) {
  const double gm1 = gamma - 1.0;
  const double u0 = q[2] * rinv, u1 = q[3] * rinv, u2 = q[4] * rinv;
  const double q2 = u0 * u0 + u1 * u1 + u2 * u2;
  const double speed = sqrt(q2);
  const double c = sqrt(gamma * p * rinv);
  const double kc = 0.5 * gamma / c * rinv;   // d c = kc (dp - p/rho drho)
  const double ks = speed > 0.0 ? rinv / speed : 0.0;
  dl[0] = -speed * rinv + kc * (0.5 * gm1 * q2 - p * rinv);
  dl[1] = kc * gm1;
  dl[2] = ks * u0 - kc * gm1 * u0;
  dl[3] = ks * u1 - kc * gm1 * u1;
  dl[4] = ks * u2 - kc * gm1 * u2;
}

template <int N>
struct VjpTile {
  static constexpr int NP = Shape<N>::NP, NFPT = Shape<N>::NFPT;
  static constexpr int E = kBlock / NP;
  static constexpr int X = AdjOpsLayout<N>::SIZE;
  static constexpr int GEO = X + pad16(5 * E * NP * 8);
  static constexpr int SMEM_BYTES = GEO + pad16(9 * E * 8);
};

template <int N>
__global__ void __launch_bounds__(kBlock) dg_euler_vjp_volume(const VjpArgs a) {
  using T = VjpTile<N>;
  using Ops = AdjOpsLayout<N>;
  constexpr int NP = T::NP, NFPT = T::NFPT, E = T::E;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ int ops_ok;
  const double* sW = reinterpret_cast<const double*>(smem + Ops::W);
  const double* sL = reinterpret_cast<const double*>(smem + Ops::L);
  double* sX = reinterpret_cast<double*>(smem + T::X);
  double* sG = reinterpret_cast<double*>(smem + T::GEO);

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
      // L = diag(s_e) L_1  =>  L^T x = L_1^T (s_e x)
      const double* xk = a.x + e0 * NP;
      const double* sc_t = a.elem_scale ? a.elem_scale + e0 : nullptr;
#pragma unroll
      for (int k = 0; k < 5; ++k, xk += nelnp)
        for (int rem = t; rem < E * NP; rem += kBlock) {
          double v = 0.0;
          if (rem < ecount * NP) {
            v = __ldg(xk + rem);
            if (sc_t) v *= __ldg(sc_t + rem / NP);
          }
          sX[k * (E * NP) + rem] = v;
        }
      const double* mt = a.metric + e0 * 9;
      for (int idx = t; idx < 9 * E; idx += kBlock)
        sG[idx] = idx < 9 * ecount ? __ldg(mt + idx) : 0.0;
    }
    __syncthreads();

    // volume: T_{r,k}(i) = sum_j W_r[j][i] x_k(j), then the flux Jacobians
    if (active && el < ecount) {
      double tr[3][5];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int k = 0; k < 5; ++k) tr[r][k] = 0.0;
#pragma unroll 4
      for (int j = 0; j < NP; ++j) {
        const double w0 = sW[(0 * NP + j) * NP + i];
        const double w1 = sW[(1 * NP + j) * NP + i];
        const double w2 = sW[(2 * NP + j) * NP + i];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const double xj = sX[(k * E + el) * NP + j];
          tr[0][k] = fma(w0, xj, tr[0][k]);
          tr[1][k] = fma(w1, xj, tr[1][k]);
          tr[2][k] = fma(w2, xj, tr[2][k]);
        }
      }
      const double* G = sG + el * 9;
      const int64_t gidx = e0 * NP + (el * NP + i);
      double qn[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) qn[k] = __ldg(a.q + k * nelnp + gidx);
      const double p = __ldg(a.aux + gidx), rinv = __ldg(a.aux + nelnp + gidx);
      double y[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        double z[5], g[5];
#pragma unroll
        for (int k = 0; k < 5; ++k)
          z[k] = fma(G[0 * 3 + x], tr[0][k], fma(G[1 * 3 + x], tr[1][k], G[2 * 3 + x] * tr[2][k]));
        euler_flux_vjp(qn, rinv, p, x == 0 ? 1.0 : 0.0, x == 1 ? 1.0 : 0.0,
                       x == 2 ? 1.0 : 0.0, z, a.gamma, g);
#pragma unroll
        for (int k = 0; k < 5; ++k) y[k] += g[k];
      }
#pragma unroll
      for (int k = 0; k < 5; ++k) a.y[k * nelnp + gidx] = y[k];
    }

    // lifted adjoints w_k(fj) = sum_i LIFT[i][fj] x_k(i) (unscaled)
    const int64_t nfpt_all = nel * NFPT;
    for (int pidx = t; pidx < ecount * NFPT; pidx += kBlock) {
      const int elp = pidx / NFPT;
      const int fj = pidx - elp * NFPT;
      double w[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll 4
      for (int ii = 0; ii < NP; ++ii) {
        const double l = sL[ii * NFPT + fj];
#pragma unroll
        for (int k = 0; k < 5; ++k) w[k] = fma(l, sX[(k * E + elp) * NP + ii], w[k]);
      }
      double* sc = a.scratch + e0 * NFPT + pidx;
#pragma unroll
      for (int k = 0; k < 5; ++k) sc[k * nfpt_all] = w[k];
    }
    __syncthreads();
  }
}

template <int N>
__global__ void __launch_bounds__(kFaceBlock) dg_euler_vjp_face(const VjpArgs a) {
  using Ops = AdjOpsLayout<N>;
  constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP, NFPT = Shape<N>::NFPT;
  __shared__ int sFN[NFPT];
  {
    const int* gFN = reinterpret_cast<const int*>(
        static_cast<const unsigned char*>(a.ops) + Ops::FN);
    for (int t = threadIdx.x; t < NFPT; t += blockDim.x) sFN[t] = gFN[t];
  }
  __syncthreads();
  const uint32_t nelnp = (uint32_t)(a.nel * NP);
  const uint32_t nfp_all = (uint32_t)(a.nel * NFPT);
  const uint32_t total = (uint32_t)(a.nowned * NFP);
  const uint32_t stride = gridDim.x * blockDim.x;
  const double gamma = a.gamma;
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += stride) {
    const uint32_t of = idx / NFP;
    const uint32_t j = idx - of * NFP;
    const uint32_t face = (uint32_t)__ldg(a.owned + of);
    const uint32_t e = face >> 2, f = face & 3u;
    const uint32_t fp = face * NFP + j;
    const uint32_t ii = e * NP + (uint32_t)sFN[f * NFP + j];
    const uint32_t g = __ldg(a.gather + fp);
    const bool bdry = (g >> 31) != 0u;
    uint32_t gi = g & 0x7fffffffu;
    if (gi >= nelnp) {
      raise_status(a.status, DG_ERR_INDEX);
      gi = ii;
    }
    int32_t pp = -1;
    if (!bdry) {
      pp = __ldg(a.partner + fp);
      if (pp < 0 || (uint32_t)pp >= nfp_all) {
        raise_status(a.status, DG_ERR_INDEX);
        pp = -1;
      }
    }
    const double* fg = a.face_geom + face * 4u;
    const double nx = __ldg(fg), ny = __ldg(fg + 1), nz = __ldg(fg + 2);
    const double scale_o = __ldg(fg + 3);
    const double scale_p =
        pp >= 0 ? __ldg(a.face_geom + ((uint32_t)pp / NFP) * 4u + 3) : 0.0;

    double qi[5], qe[5], fbar[5];
    {
      const double* qk = a.q + ii;
      const double* qx = a.q + gi;
#pragma unroll
      for (int k = 0; k < 5; ++k, qk += nelnp, qx += nelnp) {
        qi[k] = __ldg(qk);
        qe[k] = bdry ? 0.0 : __ldg(qx);
      }
      const double* so = a.scratch + fp;
      const double* sp = a.scratch + (pp >= 0 ? (uint32_t)pp : fp);
#pragma unroll
      for (int k = 0; k < 5; ++k, so += nfp_all, sp += nfp_all)
        fbar[k] = -scale_o * so[0] + (pp >= 0 ? scale_p * sp[0] : 0.0);
    }
    const double* an = a.aux;
    const double pi = __ldg(an + ii), ri = __ldg(an + nelnp + ii),
                 li = __ldg(an + 2 * (size_t)nelnp + ii);
    double pe, re, le;
    if (bdry) {  // wall mirror of the normal momentum
      const double mn = qi[2] * nx + qi[3] * ny + qi[4] * nz;
      qe[0] = qi[0];
      qe[1] = qi[1];
      qe[2] = qi[2] - 2.0 * nx * mn;
      qe[3] = qi[3] - 2.0 * ny * mn;
      qe[4] = qi[4] - 2.0 * nz * mn;
      pe = pi;
      re = ri;
      le = li;
    } else {
      pe = __ldg(an + gi);
      re = __ldg(an + nelnp + gi);
      le = __ldg(an + 2 * (size_t)nelnp + gi);
    }
    const bool imax = li >= le;
    const double lam = imax ? li : le;
    const double nn = nx * nx + ny * ny + nz * nz;
    double fd = 0.0;
#pragma unroll
    for (int k = 0; k < 5; ++k) fd = fma(fbar[k], qe[k] - qi[k], fd);
    double gi_[5], ge_[5], dl[5];
    euler_flux_vjp(qi, ri, pi, nx, ny, nz, fbar, gamma, gi_);
    euler_flux_vjp(qe, re, pe, nx, ny, nz, fbar, gamma, ge_);
    euler_speed_grad(imax ? qi : qe, imax ? ri : re, imax ? pi : pe, gamma, dl);
    const double hl = 0.5 * lam * nn, hf = 0.5 * nn * fd;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      gi_[k] = 0.5 * gi_[k] + hl * fbar[k] - (imax ? hf * dl[k] : 0.0);
      ge_[k] = 0.5 * ge_[k] - hl * fbar[k] - (imax ? 0.0 : hf * dl[k]);
    }
    double* so = a.scratch + fp;
    if (bdry) {  // q+ = M q-: add M^T ge (M symmetric) to the interior side
      const double mn = ge_[2] * nx + ge_[3] * ny + ge_[4] * nz;
      gi_[0] += ge_[0];
      gi_[1] += ge_[1];
      gi_[2] += ge_[2] - 2.0 * nx * mn;
      gi_[3] += ge_[3] - 2.0 * ny * mn;
      gi_[4] += ge_[4] - 2.0 * nz * mn;
    }
#pragma unroll
    for (int k = 0; k < 5; ++k, so += nfp_all) so[0] = gi_[k];
    if (pp >= 0) {
      double* sp = a.scratch + (uint32_t)pp;
#pragma unroll
      for (int k = 0; k < 5; ++k, sp += nfp_all) sp[0] = ge_[k];
    }
  }
}

// y_k(e, i) += sum of the face-point slots of node i (a node lies on at most
// 3 faces); 32-bit indices.  STAGE: instead of storing y, every node applies
// the reverse LSRK stage update to lam and rbar_out (x may be lam or
// rbar_out: each node reads its x and lam before it writes either).
template <int N, int NF, bool STAGE = false>
__global__ void __launch_bounds__(kBlock) dg_vjp_node_gather(const VjpArgs a) {
  using Ops = AdjOpsLayout<N>;
  constexpr int NP = Shape<N>::NP, NFPT = Shape<N>::NFPT;
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
  const uint32_t nfp_all = (uint32_t)(a.nel * NFPT);
  for (uint32_t gnode = blockIdx.x * blockDim.x + threadIdx.x; gnode < nelnp;
       gnode += gridDim.x * blockDim.x) {
    const uint32_t e = gnode / NP;
    const int i = (int)(gnode - e * NP);
    if (!STAGE && sNodeFP[i][0] < 0) continue;
#pragma unroll
    for (int k = 0; k < NF; ++k) {
      const size_t o = k * (size_t)nelnp + gnode;
      double acc = a.y[o];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const int fj = sNodeFP[i][m];
        if (fj < 0) break;
        acc += a.scratch[k * (size_t)nfp_all + e * NFPT + fj];
      }
      if constexpr (STAGE) {
        const double rb = a.xscale * a.x[o];
        const double ln = fma(a.dt * a.xscale, acc, a.lam[o]);
        a.lam[o] = ln;
        if (a.rbar_out) a.rbar_out[o] = fma(a.rk_a, rb, a.rk_b * ln);
      } else {
        a.y[o] = acc;
      }
    }
  }
}

}  // namespace dg
