// Device-side setup of box meshes: geometry, gather index, face partners and
// node coordinates of the 6 n_x n_y n_z tetrahedra of a box, built in HBM by
// one thread per element.
//
// The host setup (discretization.make_discretization) finds neighbours by
// sorting face keys; for a box the answer is known in closed form: every
// hexahedron is split the same way, so each (tetrahedron type, face) has a
// fixed neighbour -- another tetrahedron of the same hexahedron or of one of
// the six face-adjacent hexahedra -- glued with a fixed vertex permutation.
// The host derives that 6 x 4 table once from a 3 x 3 x 3 box and passes it
// in; a face is on the boundary exactly when its neighbour hexahedron lies
// outside the box.  Element order, vertex order and formulas match the host
// setup, so the arrays agree with it to round-off.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <string>

#include "../../include/dgfem_gb300.h"
#include "dg_launch.h"

namespace {

constexpr int kMaxNp = 35, kMaxNfp = 15;

struct BoxTables {
  int corner[6][4][3];     // corner offsets (0/1 per axis) of each tet's vertices
  int nbr[6][4][6];        // di, dj, dk, tet', face', permutation id
  int face_vert[4][3];     // local vertex indices of each face
  int face_opp[4];         // local vertex opposite each face
  int face_nodes[4][kMaxNfp];
  int perm[6][kMaxNfp];    // face-node map per gluing permutation
  double bary[kMaxNp][4];  // barycentric coordinates of the volume nodes
};

__constant__ BoxTables c_tab;

__global__ void box_setup_kernel(int64_t nx, int64_t ny, int64_t nz, double ax,
                                 double ay, double az, double hx, double hy,
                                 double hz, int np, int nfp, double* metric,
                                 double* face_geom, uint32_t* gather,
                                 int32_t* partner, double* nodes) {
  const int64_t nel = 6 * nx * ny * nz;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nel;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(e % 6);
    const int64_t hex = e / 6;
    const int64_t k = hex % nz, j = (hex / nz) % ny, i = hex / (ny * nz);
    double v[4][3];
    for (int c = 0; c < 4; ++c) {
      v[c][0] = ax + hx * (double)(i + c_tab.corner[t][c][0]);
      v[c][1] = ay + hy * (double)(j + c_tab.corner[t][c][1]);
      v[c][2] = az + hz * (double)(k + c_tab.corner[t][c][2]);
    }
    // dx/dr: columns are half the spanning vectors of the biunit map
    double jm[3][3];
    for (int x = 0; x < 3; ++x)
      for (int r = 0; r < 3; ++r) jm[x][r] = 0.5 * (v[r + 1][x] - v[0][x]);
    const double det = jm[0][0] * (jm[1][1] * jm[2][2] - jm[1][2] * jm[2][1]) -
                       jm[0][1] * (jm[1][0] * jm[2][2] - jm[1][2] * jm[2][0]) +
                       jm[0][2] * (jm[1][0] * jm[2][1] - jm[1][1] * jm[2][0]);
    double g[3][3];  // g[r][x] = d r / d x = inverse(jm)
    g[0][0] = (jm[1][1] * jm[2][2] - jm[1][2] * jm[2][1]) / det;
    g[0][1] = (jm[0][2] * jm[2][1] - jm[0][1] * jm[2][2]) / det;
    g[0][2] = (jm[0][1] * jm[1][2] - jm[0][2] * jm[1][1]) / det;
    g[1][0] = (jm[1][2] * jm[2][0] - jm[1][0] * jm[2][2]) / det;
    g[1][1] = (jm[0][0] * jm[2][2] - jm[0][2] * jm[2][0]) / det;
    g[1][2] = (jm[0][2] * jm[1][0] - jm[0][0] * jm[1][2]) / det;
    g[2][0] = (jm[1][0] * jm[2][1] - jm[1][1] * jm[2][0]) / det;
    g[2][1] = (jm[0][1] * jm[2][0] - jm[0][0] * jm[2][1]) / det;
    g[2][2] = (jm[0][0] * jm[1][1] - jm[0][1] * jm[1][0]) / det;
    for (int r = 0; r < 3; ++r)
      for (int x = 0; x < 3; ++x) metric[e * 9 + r * 3 + x] = g[r][x];

    // barycentric gradients: lambda_1..3 = (r+1)/2, lambda_0 = 1 - sum
    double gb[4][3];
    for (int x = 0; x < 3; ++x) {
      gb[1][x] = 0.5 * g[0][x];
      gb[2][x] = 0.5 * g[1][x];
      gb[3][x] = 0.5 * g[2][x];
      gb[0][x] = -(gb[1][x] + gb[2][x] + gb[3][x]);
    }
    for (int f = 0; f < 4; ++f) {
      const int opp = c_tab.face_opp[f];
      const double nx_ = -gb[opp][0], ny_ = -gb[opp][1], nz_ = -gb[opp][2];
      const double nn = sqrt(nx_ * nx_ + ny_ * ny_ + nz_ * nz_);
      const int a0 = c_tab.face_vert[f][0], a1 = c_tab.face_vert[f][1],
                a2 = c_tab.face_vert[f][2];
      double e1[3], e2[3];
      for (int x = 0; x < 3; ++x) {
        e1[x] = v[a1][x] - v[a0][x];
        e2[x] = v[a2][x] - v[a0][x];
      }
      const double cx = e1[1] * e2[2] - e1[2] * e2[1];
      const double cy = e1[2] * e2[0] - e1[0] * e2[2];
      const double cz = e1[0] * e2[1] - e1[1] * e2[0];
      const double area = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
      double* fg = face_geom + (e * 4 + f) * 4;
      fg[0] = nx_ / nn;
      fg[1] = ny_ / nn;
      fg[2] = nz_ / nn;
      fg[3] = (area / 2.0) / det;

      const int* nb = c_tab.nbr[t][f];
      const int64_t i2 = i + nb[0], j2 = j + nb[1], k2 = k + nb[2];
      const bool inside = i2 >= 0 && i2 < nx && j2 >= 0 && j2 < ny && k2 >= 0 &&
                          k2 < nz;
      const int64_t e2i = ((i2 * ny + j2) * nz + k2) * 6 + nb[3];
      for (int q = 0; q < nfp; ++q) {
        const int64_t fp = (e * 4 + f) * nfp + q;
        if (inside) {
          const int qq = c_tab.perm[nb[5]][q];
          gather[fp] = (uint32_t)(e2i * np + c_tab.face_nodes[nb[4]][qq]);
          if (partner) partner[fp] = (int32_t)((e2i * 4 + nb[4]) * nfp + qq);
        } else {
          gather[fp] = (uint32_t)(e * np + c_tab.face_nodes[f][q]) | 0x80000000u;
          if (partner) partner[fp] = -1;
        }
      }
    }
    if (nodes) {
      for (int n = 0; n < np; ++n)
        for (int x = 0; x < 3; ++x) {
          double s = 0.0;
          for (int c = 0; c < 4; ++c) s += c_tab.bary[n][c] * v[c][x];
          nodes[((int64_t)x * nel + e) * np + n] = s;
        }
    }
  }
}

}  // namespace

extern "C" {

int dg_box_mesh_build(const dg_box_desc* d, void* stream) {
  using dg::set_error;
  if (!d) return set_error(DG_ERR_ARGUMENT, "box description is NULL");
  if (d->order < 1 || d->order > 4)
    return set_error(DG_ERR_UNSUPPORTED, "order must be 1..4");
  if (d->n[0] < 1 || d->n[1] < 1 || d->n[2] < 1)
    return set_error(DG_ERR_ARGUMENT, "need at least one hexahedron per axis");
  const int N = d->order;
  const int np = (N + 1) * (N + 2) * (N + 3) / 6;
  const int nfp = (N + 1) * (N + 2) / 2;
  const int64_t nel = 6 * d->n[0] * d->n[1] * d->n[2];
  if (nel * np >= (int64_t(1) << 31) || nel * 4 * nfp >= (int64_t(1) << 31))
    return set_error(DG_ERR_ARGUMENT, "box too large for 31-bit indices");
  if (!d->metric || !d->face_geom || !d->gather || !d->corner || !d->nbr ||
      !d->face_vert || !d->face_opp || !d->face_nodes || !d->perm || !d->bary)
    return set_error(DG_ERR_ARGUMENT, "a required array pointer is NULL");
  for (int a = 0; a < 3; ++a)
    if (!(d->b[a] > d->a[a])) return set_error(DG_ERR_ARGUMENT, "need b > a");
  for (int k = 0; k < 6 * 4 * 3; ++k)
    if (d->corner[k] != 0 && d->corner[k] != 1)
      return set_error(DG_ERR_ARGUMENT, "corner offsets must be 0 or 1");
  for (int k = 0; k < 12; ++k)
    if (d->face_vert[k] < 0 || d->face_vert[k] > 3)
      return set_error(DG_ERR_ARGUMENT, "face_vert out of range");
  for (int k = 0; k < 4; ++k)
    if (d->face_opp[k] < 0 || d->face_opp[k] > 3)
      return set_error(DG_ERR_ARGUMENT, "face_opp out of range");
  BoxTables tab;
  std::memset(&tab, 0, sizeof(tab));
  std::memcpy(tab.corner, d->corner, sizeof(tab.corner));
  std::memcpy(tab.nbr, d->nbr, sizeof(tab.nbr));
  std::memcpy(tab.face_vert, d->face_vert, sizeof(tab.face_vert));
  std::memcpy(tab.face_opp, d->face_opp, sizeof(tab.face_opp));
  for (int f = 0; f < 4; ++f)
    for (int q = 0; q < nfp; ++q) {
      const int v = d->face_nodes[f * nfp + q];
      if (v < 0 || v >= np) return set_error(DG_ERR_ARGUMENT, "face_nodes out of range");
      tab.face_nodes[f][q] = v;
    }
  for (int p = 0; p < 6; ++p)
    for (int q = 0; q < nfp; ++q) {
      const int v = d->perm[p * nfp + q];
      if (v < 0 || v >= nfp) return set_error(DG_ERR_ARGUMENT, "perm out of range");
      tab.perm[p][q] = v;
    }
  for (int t = 0; t < 6; ++t)
    for (int f = 0; f < 4; ++f) {
      const int* nb = tab.nbr[t][f];
      if (nb[3] < 0 || nb[3] > 5 || nb[4] < 0 || nb[4] > 3 || nb[5] < 0 ||
          nb[5] > 5 || nb[0] < -1 || nb[0] > 1 || nb[1] < -1 || nb[1] > 1 ||
          nb[2] < -1 || nb[2] > 1)
        return set_error(DG_ERR_ARGUMENT, "neighbour table entry out of range");
    }
  for (int n = 0; n < np; ++n)
    for (int c = 0; c < 4; ++c) tab.bary[n][c] = d->bary[n * 4 + c];
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t err =
      cudaMemcpyToSymbolAsync(c_tab, &tab, sizeof(tab), 0, cudaMemcpyHostToDevice, s);
  if (err != cudaSuccess) return set_error(DG_ERR_CUDA, cudaGetErrorString(err));
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int64_t blocks = (nel + 255) / 256;
  if (blocks > (int64_t)nsm * 32) blocks = (int64_t)nsm * 32;
  box_setup_kernel<<<(int)blocks, 256, 0, s>>>(
      d->n[0], d->n[1], d->n[2], d->a[0], d->a[1], d->a[2],
      (d->b[0] - d->a[0]) / (double)d->n[0], (d->b[1] - d->a[1]) / (double)d->n[1],
      (d->b[2] - d->a[2]) / (double)d->n[2], np, nfp, d->metric, d->face_geom,
      d->gather, d->face_partner, d->nodes);
  err = cudaGetLastError();
  if (err != cudaSuccess) return set_error(DG_ERR_CUDA, cudaGetErrorString(err));
  // the constant tables are read asynchronously: keep `tab` alive until the
  // copy has been consumed
  err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return set_error(DG_ERR_CUDA, cudaGetErrorString(err));
  return DG_OK;
}

}  // extern "C"
