// Face-shared numerical fluxes for the FP64 RHS on sm_103a.
//
// The fused RHS kernel (dg_rhs.cuh) evaluates the numerical flux at every
// element face point: twice per glued pair of face points, once from each
// side, and for Euler it recovers pressure and wave speed of both traces at
// every one of them.  GB300's FP64 pipe issues a small fraction of its FP32
// rate, so on the low orders that repeated FP64 work is a large share of the
// RHS.  The face-shared path splits one RHS into
//
//   (a) Euler only, dg_euler_aux_kernel: pressure, 1/rho and the local wave
//       speed |u| + c of every volume node, once per node;
//   (b) dg_face_flux_kernel: one thread per face point of an OWNED face (a
//       boundary face, or the lower-numbered face of a glued pair) evaluates
//       the flux once and writes the lifted-flux input of BOTH glued face
//       points; the neighbour's value follows from how each flux transforms
//       when the two sides swap (n -> -n, jumps change sign);
//   (c) dg_rhs_kernel with MODE_SPLIT: volume term + LIFT of the stored face
//       values, in the same persistent tile loop as the fused kernel.
//
// Face values live in HBM as (nfields, Nel, 4 Nfp) doubles, face point
// (e, f, j) at e * 4 Nfp + f Nfp + j -- the fused kernel's shared-memory
// flux layout -- already multiplied by sJ/J and signed as that kernel's.
// The flux formulas are the fused kernel's (which follow
// actx_dgfem_suite/equations/wave.py:80-114 and grudge's Euler LF and
// Maxwell alpha fluxes as configured at equations/euler.py:168-174 and
// equations/maxwell.py:55-59).
#pragma once

#include "dg_rhs.cuh"

namespace dg {

constexpr int kFaceBlock = 256;

struct FaceArgs {
  const double* q;            // (NF, Nel, Np) state
  const double* aux;          // euler: (3, Nel, Np) p, 1/rho, |u| + c
  const double* face_geom;    // (Nel, 4, 4) n_x, n_y, n_z, sJ/J
  const uint32_t* gather;     // (Nel, 4, Nfp) exterior node, bit 31 = boundary
  const int32_t* partner;     // (Nel, 4, Nfp) glued face point, -1 on boundary
  const int32_t* owned;       // owned faces e * 4 + f, ascending
  const int32_t* face_nodes;  // (4, Nfp) volume node of each face node
  double* flux;               // (NF, Nel, 4 Nfp) lifted-flux input
  int64_t nel;
  int64_t nowned;
  int* status;
  double p0, p1, p2;          // equation parameters
  double k[6];                // maxwell: z, 1/z, -1/(2z), 1/(2/z), 1/eps, 1/mu
};

// Pressure, 1/rho and |u| + c of every node (the per-trace quantities of the
// Lax-Friedrichs flux), evaluated once per node instead of once per face
// point and side.
template <int EQ>
__global__ void __launch_bounds__(kFaceBlock)
    dg_euler_aux_kernel(const double* __restrict__ q, double* __restrict__ aux,
                        uint32_t nelnp, double gamma) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nelnp;
       idx += stride) {
    const double* qn = q + idx;
    const double rho = __ldg(qn);
    const double en = __ldg(qn + nelnp);
    const double m0 = __ldg(qn + 2 * (size_t)nelnp);
    const double m1 = __ldg(qn + 3 * (size_t)nelnp);
    const double m2 = __ldg(qn + 4 * (size_t)nelnp);
    const double rinv = 1.0 / rho;
    const double mm = fma(m0, m0, fma(m1, m1, m2 * m2));
    const double p = (gamma - 1.0) * fma(-0.5 * mm, rinv, en);
    // |u| + c = sqrt(|m|^2) / rho + sqrt(gamma p / rho)
    const double lam = fma(sqrt(mm), rinv, sqrt(gamma * (p * rinv)));
    double* an = aux + idx;
    an[0] = p;
    an[nelnp] = rinv;
    an[2 * (size_t)nelnp] = lam;
  }
}

template <int N, int EQ>
__global__ void __launch_bounds__(kFaceBlock) dg_face_flux_kernel(const FaceArgs a) {
  constexpr int NP = Shape<N>::NP, NFP = Shape<N>::NFP, NFPT = Shape<N>::NFPT;
  constexpr int NF = EqInfo<EQ>::NF;
  __shared__ int sFN[NFPT];
  for (int t = threadIdx.x; t < NFPT; t += blockDim.x) sFN[t] = __ldg(a.face_nodes + t);
  __syncthreads();

  // 32-bit indices throughout (Nel * 4 Nfp < 2^31 is checked at plan creation)
  const uint32_t nelnp = (uint32_t)(a.nel * NP);
  const uint32_t nfp_all = (uint32_t)(a.nel * NFPT);
  const uint32_t total = (uint32_t)(a.nowned * NFP);
  const uint32_t stride = gridDim.x * blockDim.x;
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
    if (gi >= nelnp) {  // never read out of bounds
      raise_status(a.status, DG_ERR_INDEX);
      gi = ii;
    }
    int32_t pp = -1;
    if (!bdry) {
      pp = __ldg(a.partner + fp);
      if (pp < 0 || (uint32_t)pp >= nfp_all) {  // never write out of bounds
        raise_status(a.status, DG_ERR_INDEX);
        pp = -1;
      }
    }
    // n_x, n_y, n_z, sJ/J of the face: two 16-byte loads (rows of 32 bytes)
    const double2* fg = reinterpret_cast<const double2*>(a.face_geom) + face * 2u;
    const double2 g01 = __ldg(fg), g23 = __ldg(fg + 1);
    const double nx = g01.x, ny = g01.y, nz = g23.x;
    const double scale_o = g23.y;
    const double scale_p =
        pp >= 0 ? __ldg(a.face_geom + ((uint32_t)pp / NFP) * 4u + 3) : 0.0;

    double qi[NF], qe[NF];
    {
      const double* qk = a.q + ii;
      const double* qx = a.q + gi;
#pragma unroll
      for (int k = 0; k < NF; ++k, qk += nelnp, qx += nelnp) {
        qi[k] = __ldg(qk);
        qe[k] = bdry ? 0.0 : __ldg(qx);
      }
    }
    // own[k]: value for this face point; part[k]: for the glued face point
    // (before each side's sJ/J and a common factor fs)
    double own[NF], part[NF];
    double fs = 1.0;

    if constexpr (EQ == DG_WAVE) {
      if (bdry) {  // Dirichlet mirror: exterior (-u, v)
        qe[0] = -qi[0];
        qe[1] = qi[1];
        qe[2] = qi[2];
        qe[3] = qi[3];
      }
      // F_u = c (avg(v).n + (u+ - u-)/2) = c/2 ((v- + v+).n + u+ - u-),
      // F_v = c (avg(u) + (v+ - v-).n/2) n = c/2 (u- + u+ + (v+ - v-).n) n;
      // c/2 goes into the side scales
      const double sv = fma(qi[1] + qe[1], nx, fma(qi[2] + qe[2], ny, (qi[3] + qe[3]) * nz));
      const double dv = fma(qe[1] - qi[1], nx, fma(qe[2] - qi[2], ny, (qe[3] - qi[3]) * nz));
      const double gv = (qi[0] + qe[0]) + dv;
      own[0] = sv + (qe[0] - qi[0]);
      own[1] = gv * nx;
      own[2] = gv * ny;
      own[3] = gv * nz;
#pragma unroll
      for (int k = 0; k < NF; ++k) part[k] = -own[k];
      fs = 0.5 * a.p0;
    } else if constexpr (EQ == DG_EULER) {
      const double* an = a.aux;
      const double pi = __ldg(an + ii), ri = __ldg(an + nelnp + ii),
                   li = __ldg(an + 2 * (size_t)nelnp + ii);
      double pe, re, le;
      if (bdry) {  // InviscidWallBC: mirror the normal momentum; rho, E, |m| kept
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
      // F(q).n of one side: with m.n first, u.n = (m.n) / rho costs one
      // product (the velocity itself is not needed here)
      double fn_i[5], fn_e[5];
      auto side = [&](const double* qq, double p, double rinv, double* fn) {
        const double mn = fma(qq[2], nx, fma(qq[3], ny, qq[4] * nz));
        const double un = mn * rinv;
        fn[0] = mn;
        fn[1] = un * (qq[1] + p);
        fn[2] = fma(qq[2], un, p * nx);
        fn[3] = fma(qq[3], un, p * ny);
        fn[4] = fma(qq[4], un, p * nz);
      };
      side(qi, pi, ri, fn_i);
      side(qe, pe, re, fn_e);
      // f_k = 1/2 (F_i + F_e).n - 1/2 lam (q_e - q_i) n.n = 1/2 t_k; the 1/2
      // and the sign go into the per-side scale factors below
      const double lnn = fmax(li, le) * fma(nx, nx, fma(ny, ny, nz * nz));
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const double tk = fma(-lnn, qe[k] - qi[k], fn_i[k] + fn_e[k]);
        own[k] = -tk;
        part[k] = tk;
      }
      fs = 0.5;
    } else {  // DG_MAXWELL
      if (bdry) {  // PEC: exterior (-E, H)
        qe[0] = -qi[0];
        qe[1] = -qi[1];
        qe[2] = -qi[2];
        qe[3] = qi[3];
        qe[4] = qi[4];
        qe[5] = qi[5];
      }
      const double alpha = a.p0;
      const double z = a.k[0], y = a.k[1], ce = a.k[2], ch = a.k[3];
      const double je[3] = {qe[0] - qi[0], qe[1] - qi[1], qe[2] - qi[2]};
      const double jh[3] = {qe[3] - qi[3], qe[4] - qi[4], qe[5] - qi[5]};
      const double n[3] = {nx, ny, nz};
      auto cross = [](const double* a_, const double* b_, double* c_) {
        c_[0] = a_[1] * b_[2] - a_[2] * b_[1];
        c_[1] = a_[2] * b_[0] - a_[0] * b_[2];
        c_[2] = a_[0] * b_[1] - a_[1] * b_[0];
      };
      // fe = n x (z jh - alpha n x je) = Ae + Be, fh = n x (y je + alpha n x jh)
      // = Ah + Bh; swapping the sides keeps Ae, Ah and negates Be, Bh.  With
      // the constants folded: -ce fe = k1 (n x jh) + k2 (n x n x je),
      // -ch fh = k3 (n x je) + k4 (n x n x jh)
      double nxe[3], nxh[3], nnxe[3], nnxh[3];
      cross(n, je, nxe);
      cross(n, jh, nxh);
      cross(n, nxe, nnxe);
      cross(n, nxh, nnxh);
      const double k1 = -ce * z, k2 = ce * alpha, k3 = -ch * y, k4 = -ch * alpha;
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        const double ae = k1 * nxh[x], be = k2 * nnxe[x];
        const double ah = k3 * nxe[x], bh = k4 * nnxh[x];
        own[x] = ae + be;
        own[3 + x] = ah + bh;
        part[x] = ae - be;
        part[3 + x] = ah - bh;
      }
    }

    const double so = fs * scale_o;
    const double sp = fs * scale_p;
    double* out = a.flux + fp;
#pragma unroll
    for (int k = 0; k < NF; ++k, out += nfp_all) out[0] = so * own[k];
    if (pp >= 0) {
      double* outp = a.flux + (uint32_t)pp;
#pragma unroll
      for (int k = 0; k < NF; ++k, outp += nfp_all) outp[0] = sp * part[k];
    }
  }
}

}  // namespace dg
