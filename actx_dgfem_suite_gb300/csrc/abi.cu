// C ABI of the DG-FEM RHS evaluator (declared in include/dgfem_gb300.h).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/dgfem_gb300.h"
#include "dg_adjoint.cuh"  // AdjArgs, AdjOpsLayout
#include "dg_adjoint_euler.cuh"  // VjpArgs
#include "dg_face.cuh"     // FaceArgs
#include "dg_launch.h"
#include "dg_rhs.cuh"  // RhsArgs, kBlock

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

}  // namespace

namespace dg {
int set_error(int code, const char* msg) {
  g_last_error = msg;
  return code;
}
}  // namespace dg

namespace {

int cuda_fail(cudaError_t err, const char* what) {
  return fail(DG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

int nfields_of(int eq) {
  switch (eq) {
    case DG_WAVE: return 4;
    case DG_EULER: return 5;
    case DG_MAXWELL: return 6;
    default: return 0;
  }
}

int nparams_of(int eq) { return eq == DG_MAXWELL ? 3 : 1; }

cudaError_t shape_of(int eq, int order, int precision, int mode,
                     dg::LaunchShape* out) {
  switch (eq) {
    case DG_WAVE: return dg::shape_wave(order, precision, mode, out);
    case DG_EULER: return dg::shape_euler(order, precision, mode, out);
    case DG_MAXWELL: return dg::shape_maxwell(order, precision, mode, out);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t face_blocks_of(int eq, int order, int* blocks_per_sm) {
  switch (eq) {
    case DG_WAVE: return dg::face_blocks_wave(order, blocks_per_sm);
    case DG_EULER: return dg::face_blocks_euler(order, blocks_per_sm);
    case DG_MAXWELL: return dg::face_blocks_maxwell(order, blocks_per_sm);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t face_launch_of(int eq, int order, const dg::FaceArgs& a, int grid,
                           int aux_grid, cudaStream_t s) {
  switch (eq) {
    case DG_WAVE: return dg::face_launch_wave(order, a, grid, aux_grid, s);
    case DG_EULER: return dg::face_launch_euler(order, a, grid, aux_grid, s);
    case DG_MAXWELL: return dg::face_launch_maxwell(order, a, grid, aux_grid, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_of(int eq, int order, int precision, int mode,
                      const dg::RhsArgs& a, int grid, cudaStream_t s) {
  switch (eq) {
    case DG_WAVE: return dg::launch_wave(order, precision, mode, a, grid, s);
    case DG_EULER: return dg::launch_euler(order, precision, mode, a, grid, s);
    case DG_MAXWELL: return dg::launch_maxwell(order, precision, mode, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

bool overlap(const void* a, const void* b, int64_t bytes) {
  const char* x = static_cast<const char*>(a);
  const char* y = static_cast<const char*>(b);
  return x < y + bytes && y < x + bytes;
}

// [a, a + na) and [b, b + nb) intersect
bool overlap2(const void* a, int64_t na, const void* b, int64_t nb) {
  const char* x = static_cast<const char*>(a);
  const char* y = static_cast<const char*>(b);
  return x < y + nb && y < x + na;
}

// one thread waits on an mbarrier whose single expected arrival never comes
__global__ void wait_probe_kernel(int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    dg::mbar_init(&bar, 1);
    if (!dg::mbar_wait_bounded(&bar, 0)) dg::raise_status(status, DG_ERR_TIMEOUT);
  }
}

// Per block: sum (a - b)^2 and sum b^2 over a grid-stride range, reduced in a
// fixed order (deterministic); partial[2 * block + {0, 1}].
constexpr int kNormBlocks = 512;
__global__ void __launch_bounds__(256) diff_norm_kernel(const double* a, const double* b,
                                                        int64_t n, double* partial) {
  __shared__ double s_d[256], s_b[256];
  double d2 = 0.0, b2 = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double bv = b[k], dv = a[k] - bv;
    d2 = fma(dv, dv, d2);
    b2 = fma(bv, bv, b2);
  }
  s_d[threadIdx.x] = d2;
  s_b[threadIdx.x] = b2;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      s_d[threadIdx.x] += s_d[threadIdx.x + w];
      s_b[threadIdx.x] += s_b[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = s_d[0];
    partial[2 * blockIdx.x + 1] = s_b[0];
  }
}

// dst[k] = src[k] for n 16-byte words, grid-stride, one word per thread and
// step.  Either side may be page-locked host memory: the SMs then load or
// store it through the unified address space over the CPU-GPU link, without
// a copy engine.
__global__ void __launch_bounds__(256) stream_copy_kernel(const uint4* __restrict__ src,
                                                          uint4* __restrict__ dst,
                                                          int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // four independent words in flight per thread
  for (; k + 3 * stride < n; k += 4 * stride) {
    const uint4 a = src[k], b = src[k + stride], c = src[k + 2 * stride],
                d = src[k + 3 * stride];
    dst[k] = a;
    dst[k + stride] = b;
    dst[k + 2 * stride] = c;
    dst[k + 3 * stride] = d;
  }
  for (; k < n; k += stride) dst[k] = src[k];
}

__global__ void fp64_fma_probe_kernel(double* out, int iters) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = 1.0 + 1e-9 * (double)(tid + k);
  // operands in registers (FP64 FMAs with constant-bank operands issue
  // measurably slower on GB300); 32-bit trip count, unrolled loop
  const double b = 1.0 - 1e-7 * (1.0 + 1e-12 * (double)threadIdx.x);
  const double c = 1e-7 * (1.0 + 1e-12 * (double)threadIdx.x);
#pragma unroll 4
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = fma(v[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += v[k];
  out[tid] = s;
}

}  // namespace

struct dg_plan {
  int32_t equation = 0;
  int32_t precision = 0;
  int32_t order = 0;
  int dim = 3;             // 2: triangle mesh (dg_plan_create_2d)
  int grid_stage = 0;      // 2D: persistent grid of the RK-stage kernel (grid: RHS)
  int32_t np = 0, nfp = 0, nfields = 0;
  int64_t nel = 0;
  const double* metric = nullptr;
  const double* face_geom = nullptr;
  const uint32_t* gather = nullptr;
  void* d_ops = nullptr;
  uint32_t ops_bytes = 0;
  int* d_status = nullptr;
  double params[3] = {0, 0, 0};
  int grid = 0;
  int64_t ntiles = 0;      // tiles of the main kernel
  int grid_mtc = 0;        // mixed precision with tensor-core products
  int variant = 0;         // bit 0: tensor-core products (mixed); bit 1: one CTA per
                           // tile; 4-6: the mixed kernel on tcgen05; 7-10: the
                           // mma.sync products at the other tile shapes
  dg::LaunchShape shape;
  int device = 0;
  int nsm = 0;
  const double* elem_scale = nullptr;
  double k[6] = {0, 0, 0, 0, 0, 0};  // derived constants (see RhsArgs::k)
  // face-shared path (FP64, when the mesh carries face_partner)
  bool split = false;
  int32_t* d_owned = nullptr;  // owned faces e * 4 + f
  int64_t nowned = 0;
  double* d_flux = nullptr;    // (NF, Nel, 4 Nfp)
  double* d_aux = nullptr;     // euler: (3, Nel, Np)
  int face_grid = 0, aux_grid = 0;
  const int32_t* d_face_nodes = nullptr;  // inside d_ops
  // tensor-core contractions (DG_FP64_TC on the face-shared path)
  bool tc = false;
  void* d_tc_ops = nullptr;
  uint32_t tc_ops_bytes = 0;
  dg::LaunchShape tc_shape;
  int tc_grid = 0;
  // mixed-precision Euler: per-node FP32 pressure table, filled before each RHS
  float* d_pres = nullptr;
  int pres_grid = 0;
  // mixed precision with tcgen05 contractions: [0] exact digit pairs
  // (variant 4), [1] 3xTF32 products (variant 5), [2] the same with the
  // other CTA size (variant 6); [2] shares [1]'s operator block
  bool tcm[3] = {false, false, false};
  void* d_tcm_ops[3] = {nullptr, nullptr, nullptr};
  uint32_t tcm_ops_bytes[3] = {0u, 0u, 0u};
  dg::LaunchShape tcm_shape[3];
  int tcm_grid[3] = {0, 0, 0};
  // mixed precision, mma.sync products at the other tile shapes: [0] 128
  // threads and 128 / Np elements per tile (variants 7 persistent, 8 one CTA
  // per tile), [1] 512 threads and 512 / Np elements (variants 9, 10)
  bool tcb[2] = {false, false};
  dg::LaunchShape tcb_shape[2];
  int tcb_grid[2] = {0, 0};
  int64_t tcb_ntiles[2] = {0, 0};
  // face-shared path and adjoint (wave, FP64): the mesh's face_partner
  const int32_t* face_partner = nullptr;
  void* d_adj_ops = nullptr;
  uint32_t adj_ops_bytes = 0;
  int adj_grid = 0;
};

namespace {

dg::RhsArgs base_args(const dg_plan* p) {
  dg::RhsArgs a;
  std::memset(&a, 0, sizeof(a));
  a.metric = p->metric;
  a.face_geom = p->face_geom;
  a.gather = p->gather;
  a.ops = p->d_ops;
  a.ops_bytes = p->ops_bytes;
  a.nel = p->nel;
  a.status = p->d_status;
  a.p0 = p->params[0];
  a.p1 = p->params[1];
  a.p2 = p->params[2];
  for (int k = 0; k < 6; ++k) a.k[k] = p->k[k];
  a.elem_scale = p->elem_scale;
  a.flux_in = p->split ? p->d_flux : nullptr;
  a.aux = p->split ? p->d_aux : nullptr;
  a.pres = p->d_pres;
  return a;
}

// Ownership of every face for the face-shared path, with a consistency
// check of face_partner: owned[face] = 1 for a boundary face and for the
// lower-numbered face of a glued pair.  *bad is set unless every interior
// face point's partner lies on one other face, maps back to it, and is the
// face point whose volume node the gather index names.
__global__ void face_owner_kernel(const uint32_t* gather, const int32_t* partner,
                                  const int32_t* face_nodes, int np, int nfp,
                                  int64_t nel, uint8_t* owned, int* bad) {
  const int64_t nfaces = nel * 4;
  const int64_t nfp_all = nfaces * nfp;
  for (int64_t face = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; face < nfaces;
       face += (int64_t)gridDim.x * blockDim.x) {
    const int64_t fp0 = face * nfp;
    const bool bdry = (gather[fp0] >> 31) != 0u;
    int64_t pface = -1;
    bool ok = true;
    for (int j = 0; j < nfp && ok; ++j) {
      const uint32_t g = gather[fp0 + j];
      const int32_t pp = partner[fp0 + j];
      if (((g >> 31) != 0u) != bdry) {
        ok = false;
      } else if (bdry) {
        ok = pp == -1;
      } else if (pp < 0 || pp >= nfp_all) {
        ok = false;
      } else {
        const int64_t pf = pp / nfp;
        if (j == 0) pface = pf;
        const int64_t e2 = pp / (4 * nfp);
        const int fj2 = (int)(pp - e2 * 4 * nfp);
        ok = pf == pface && pf != face && partner[pp] == fp0 + j &&
             (int64_t)(g & 0x7fffffffu) == e2 * np + face_nodes[fj2];
      }
    }
    if (!ok) atomicExch(bad, 1);
    owned[face] = (ok && (bdry || face < pface)) ? 1 : 0;
  }
}

// Build the owned-face list and the buffers of the face-shared path.
int setup_split(dg_plan* p, const int32_t* partner, const int32_t* d_face_nodes) {
  const int64_t nfaces = p->nel * 4;
  uint8_t* d_mask = nullptr;
  int* d_bad = nullptr;
  cudaError_t err = cudaMalloc(&d_mask, nfaces);
  if (err == cudaSuccess) err = cudaMalloc(&d_bad, sizeof(int));
  if (err == cudaSuccess) err = cudaMemset(d_bad, 0, sizeof(int));
  if (err == cudaSuccess) {
    const int64_t blocks = (nfaces + 255) / 256;
    const int grid = (int)(blocks < (int64_t)p->nsm * 16 ? blocks : (int64_t)p->nsm * 16);
    face_owner_kernel<<<grid, 256>>>(p->gather, partner, d_face_nodes, p->np, p->nfp,
                                     p->nel, d_mask, d_bad);
    err = cudaGetLastError();
  }
  std::vector<uint8_t> mask;
  int bad = 0;
  if (err == cudaSuccess) {
    mask.resize(nfaces);
    err = cudaMemcpy(mask.data(), d_mask, nfaces, cudaMemcpyDeviceToHost);
  }
  if (err == cudaSuccess) err = cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost);
  if (d_mask) cudaFree(d_mask);
  if (d_bad) cudaFree(d_bad);
  if (err != cudaSuccess) return cuda_fail(err, "face ownership");
  if (bad)
    return fail(DG_ERR_ARGUMENT,
                "face_partner is not a pairing of whole faces consistent with gather");
  std::vector<int32_t> owned;
  owned.reserve(nfaces / 2 + 1024);
  for (int64_t f = 0; f < nfaces; ++f)
    if (mask[f]) owned.push_back((int32_t)f);
  p->nowned = (int64_t)owned.size();
  const int nfpt = 4 * p->nfp;
  err = cudaMalloc(&p->d_owned, (owned.empty() ? 1 : owned.size()) * sizeof(int32_t));
  if (err == cudaSuccess && !owned.empty())
    err = cudaMemcpy(p->d_owned, owned.data(), owned.size() * sizeof(int32_t),
                     cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMalloc(&p->d_flux, (size_t)p->nfields * p->nel * nfpt * sizeof(double));
  if (err == cudaSuccess && p->equation == DG_EULER)
    err = cudaMalloc(&p->d_aux, (size_t)3 * p->nel * p->np * sizeof(double));
  if (err != cudaSuccess) return cuda_fail(err, "face-shared buffers");
  int fb = 0;
  err = face_blocks_of(p->equation, p->order, &fb);
  if (err != cudaSuccess) return cuda_fail(err, "face kernel configuration");
  if (fb < 1) return fail(DG_ERR_UNSUPPORTED, "face kernel does not fit on an SM");
  const int64_t fthreads = p->nowned * p->nfp;
  const int64_t fblocks = (fthreads + dg::kFaceBlock - 1) / dg::kFaceBlock;
  const int64_t ffull = (int64_t)p->nsm * fb;
  p->face_grid = (int)(fblocks < ffull ? (fblocks > 0 ? fblocks : 1) : ffull);
  const int64_t ablocks = (p->nel * p->np + dg::kFaceBlock - 1) / dg::kFaceBlock;
  const int64_t afull = (int64_t)p->nsm * 8;
  p->aux_grid = (int)(ablocks < afull ? ablocks : afull);
  p->split = true;
  return DG_OK;
}

// Variants 7-10: the mma.sync kernel at tile shape (v - 7) / 2, one CTA per
// tile when v - 7 is odd.
constexpr int kFirstShapeVariant = 7;
bool is_tcm_variant(int v) { return v >= 4 && v < kFirstShapeVariant; }
bool is_shape_variant(int v) { return v >= kFirstShapeVariant && v < DG_NUM_VARIANTS; }
int shape_index(int v) { return (v - kFirstShapeVariant) / 2; }
constexpr int kShapeModeBits[2] = {dg::MODE_B128, dg::MODE_B512};

// Mode bits and grid of the main kernel under the plan's variant.
int main_mode(const dg_plan* p, int base) {
  if (is_shape_variant(p->variant))
    return base | dg::MODE_TC | kShapeModeBits[shape_index(p->variant)];
  return base | ((p->variant & 1) && p->precision == DG_FP32_MIXED ? dg::MODE_TC : 0);
}
int main_grid(const dg_plan* p) {
  if (is_shape_variant(p->variant)) {
    const int k = shape_index(p->variant);
    if ((p->variant - kFirstShapeVariant) & 1)
      return (int)(p->tcb_ntiles[k] < 0x7fffffff ? p->tcb_ntiles[k] : 0x7fffffff);
    return p->tcb_grid[k];
  }
  if (p->variant & 2) return (int)(p->ntiles < 0x7fffffff ? p->ntiles : 0x7fffffff);
  return (p->variant & 1) && p->precision == DG_FP32_MIXED ? p->grid_mtc : p->grid;
}

// The face-shared path's first launches (Euler table, face kernel) for state q.
cudaError_t launch_faces(const dg_plan* p, const double* q, cudaStream_t s) {
  dg::FaceArgs f;
  std::memset(&f, 0, sizeof(f));
  f.q = q;
  f.aux = p->d_aux;
  f.face_geom = p->face_geom;
  f.gather = p->gather;
  f.partner = p->face_partner;
  f.owned = p->d_owned;
  f.face_nodes = p->d_face_nodes;
  f.flux = p->d_flux;
  f.nel = p->nel;
  f.nowned = p->nowned;
  f.status = p->d_status;
  f.p0 = p->params[0];
  f.p1 = p->params[1];
  f.p2 = p->params[2];
  for (int k = 0; k < 6; ++k) f.k[k] = p->k[k];
  return face_launch_of(p->equation, p->order, f, p->face_grid, p->aux_grid, s);
}

// Adjoint operator block: W in [r][i][j] (the forward layout of W^T), LIFT in
// [i][fj], face nodes.
void pack_adj_ops(std::vector<unsigned char>& buf, int np, int nfp,
                  const double* diff, const double* lift,
                  const int32_t* face_nodes, int w_off, int l_off, int fn_off) {
  double* w = reinterpret_cast<double*>(buf.data() + w_off);
  double* l = reinterpret_cast<double*>(buf.data() + l_off);
  int32_t* fn = reinterpret_cast<int32_t*>(buf.data() + fn_off);
  for (int k = 0; k < 3 * np * np; ++k) w[k] = diff[k];
  for (int k = 0; k < np * 4 * nfp; ++k) l[k] = lift[k];
  for (int k = 0; k < 4 * nfp; ++k) fn[k] = face_nodes[k];
}

// FP64: Wt[r][j][i] and Lt[fj][i] (one scalar per thread and step).
void pack_ops_fp64(std::vector<unsigned char>& buf, const dg::OpsOffsets& off,
                   int np, int nfp, const double* diff, const double* lift,
                   const int32_t* face_nodes) {
  double* w = reinterpret_cast<double*>(buf.data() + off.w);
  double* l = reinterpret_cast<double*>(buf.data() + off.l);
  int32_t* fn = reinterpret_cast<int32_t*>(buf.data() + off.fn);
  for (int r = 0; r < 3; ++r)
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j)
        w[(r * np + j) * np + i] = diff[(r * np + i) * np + j];
  for (int i = 0; i < np; ++i)
    for (int fj = 0; fj < 4 * nfp; ++fj)
      l[fj * np + i] = lift[i * 4 * nfp + fj];
  for (int k = 0; k < 4 * nfp; ++k) fn[k] = face_nodes[k];
}

// Mixed: FP32 W[r][i][j] and L[i][fj] with zero-padded rows of pitch
// pitch_host(np) and pitch_host(4 nfp) (four entries per shared load).
void pack_ops_fp32(std::vector<unsigned char>& buf, const dg::OpsOffsets& off,
                   int np, int nfp, const double* diff, const double* lift,
                   const int32_t* face_nodes) {
  float* w = reinterpret_cast<float*>(buf.data() + off.w);
  float* l = reinterpret_cast<float*>(buf.data() + off.l);
  int32_t* fn = reinterpret_cast<int32_t*>(buf.data() + off.fn);
  const int rp = dg::pitch_host(np), fp = dg::pitch_host(4 * nfp);
  for (int r = 0; r < 3; ++r)
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j)
        w[(r * np + i) * rp + j] = (float)diff[(r * np + i) * np + j];
  for (int i = 0; i < np; ++i)
    for (int fj = 0; fj < 4 * nfp; ++fj)
      l[i * fp + fj] = (float)lift[i * 4 * nfp + fj];
  for (int k = 0; k < 4 * nfp; ++k) fn[k] = face_nodes[k];
}

// {{{ operator digits for the tensor-core kernel (layout: tc::Plan in dg_tc.cuh)

int r16h(int x) { return (x + 15) & ~15; }

// IEEE half bits of an integer |d| <= 2048 (exact)
uint16_t half_bits(int d) {
  if (d == 0) return 0;
  const uint16_t sign = d < 0 ? 0x8000 : 0;
  const int a = d < 0 ? -d : d;
  int e = 0;
  while ((a >> (e + 1)) != 0) ++e;                 // 2^e <= a < 2^(e+1)
  const int mant = ((a << 10) >> e) & 0x3ff;
  return static_cast<uint16_t>(sign | ((e + 15) << 10) | mant);
}

// TF32 bits of a finite float: 10 explicit mantissa bits, rounded to
// nearest with ties away from zero (the rounding of cvt.rna.tf32.f32)
uint32_t tf32_rna_bits(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return (u + 0x1000u) & 0xffffe000u;
}

// One product's block: A (m x k, element (r, c) = at(r, c)) as 7 FP16 digit
// slices of its rows' 54-bit fixed-point integers (balanced base-256 digits,
// slice 0 most significant) in the K-major no-swizzle layout of the
// tensor-core descriptors (element (r, c) at (r/8) SBO + (c/8) 128 + (r%8) 16
// + (c%8) 2 bytes, SBO = 128 * k-chunks, rows padded to a multiple of 8),
// then the row exponents.
template <class At>
int pack_gemm(unsigned char* out, int m, int k, At at) {
  const int mr8 = (m + 7) & ~7, kp = r16h(k), kc = kp / 8;
  const int sbo = kc * 128;
  const int slice = (mr8 / 8) * sbo;
  const int digits = 7 * slice;
  const int bytes = (digits + mr8 * 4 + 15) & ~15;
  if (!out) return bytes;
  std::memset(out, 0, bytes);             // FP16 zero
  int32_t* row_exp = reinterpret_cast<int32_t*>(out + digits);
  for (int r = 0; r < m; ++r) {
    double mx = 0.0;
    for (int c = 0; c < k; ++c) mx = std::fmax(mx, std::fabs(at(r, c)));
    int e = 0;
    if (mx > 0.0) std::frexp(mx, &e);    // |A_rc| < 2^e
    row_exp[r] = e;
    for (int c = 0; c < k; ++c) {
      long long x = std::llrint(std::ldexp(at(r, c), 54 - e));
      const int within = (r / 8) * sbo + (c / 8) * 128 + (r % 8) * 16 + (c % 8) * 2;
      for (int sl = 6; sl >= 0; --sl) {   // least significant digit first
        const long long d = ((x + 128) & 255) - 128;
        x = (x - d) >> 8;
        const uint16_t h = half_bits(static_cast<int>(d));
        unsigned char* dst = out + sl * slice + within;
        dst[0] = static_cast<unsigned char>(h & 0xff);
        dst[1] = static_cast<unsigned char>(h >> 8);
      }
    }
  }
  return bytes;
}

}  // namespace

namespace dg {
int pack_tc_ops(int eq, int order, const double* diff, const double* lift,
                unsigned char* out, int out_bytes) {
  const int np = (order + 1) * (order + 2) * (order + 3) / 6;
  const int nfpt = 2 * (order + 1) * (order + 2);
  auto stacked = [&](int r, int c) { return diff[(size_t)r * np + c]; };  // [A_0; A_1; A_2]
  auto concat = [&](int r, int c) {                                      // [A_0 A_1 A_2]
    const int q = c / np;
    return diff[((size_t)q * np + r) * np + (c - q * np)];
  };
  auto gl = [&](int r, int c) { return lift[(size_t)r * nfpt + c]; };
  const bool st = eq != DG_EULER;
  const int gv = st ? pack_gemm(nullptr, 3 * np, np, stacked)
                    : pack_gemm(nullptr, np, 3 * np, concat);
  const int total = gv + pack_gemm(nullptr, np, nfpt, gl);
  if (!out) return total;
  if (out_bytes != total) return -1;
  if (st) pack_gemm(out, 3 * np, np, stacked);
  else pack_gemm(out, np, 3 * np, concat);
  pack_gemm(out + gv, np, nfpt, gl);
  return total;
}

// Operator block of the mixed tcgen05 kernel: B_V = [A_0 A_1 A_2] and
// B_L = LIFT, as four FP16 digit slices each plus row scales, or (tf32) as
// TF32 hi / lo slices (layout: tcm::MPlan).
int pack_tcm_ops(int order, const double* diff, const double* lift,
                 const int32_t* face_nodes, unsigned char* out, int out_bytes, bool tf32) {
  const int np = (order + 1) * (order + 2) * (order + 3) / 6;
  const int nfpt = 2 * (order + 1) * (order + 2);
  const int npp = np + (np & 1);  // node pitch of the volume columns (even)
  const int kg = tf32 ? 4 : 8, kstep = 2 * kg, esz = 16 / kg, ndig = tf32 ? 2 : 4;
  auto rup = [](int x, int m) { return (x + m - 1) / m * m; };
  const int nb = (np + 15) & ~15, kv = rup(3 * npp, kstep), kl = rup(nfpt, kstep);
  const int sbo_v = (kv / kg) * 128, sbo_l = (kl / kg) * 128;
  const int bs_v = (nb / 8) * sbo_v, bs_l = (nb / 8) * sbo_l;
  const int ops_l = ndig * bs_v, ops_ev = ops_l + ndig * bs_l;
  const int ops_el = ops_ev + (tf32 ? 0 : nb * 4);
  const int ops_fn = ops_el + (tf32 ? 0 : nb * 4);
  const int total = ops_fn + ((nfpt * 4 + 15) & ~15);
  if (!out) return total;
  if (out_bytes != total) return -1;
  std::memset(out, 0, total);  // FP16 / TF32 zeros
  auto offset = [&](int i, int k, int sbo) {
    return (i / 8) * sbo + (k / kg) * 128 + (i % 8) * 16 + (k % kg) * esz;
  };
  // digits: rows i < np of at(i, k), k < kk, scaled per row to 31-bit
  // integers (|x| <= 2^31) in four balanced base-256 digits, most significant
  // first; row scales 2^e (FP32) with |at(i, k)| < 2^e
  auto block = [&](int base, int slice, int sbo, int kk, int exp_off, auto at) {
    float* rscale = reinterpret_cast<float*>(out + exp_off);
    for (int i = 0; i < np; ++i) {
      double mx = 0.0;
      for (int k = 0; k < kk; ++k) mx = std::fmax(mx, std::fabs(at(i, k)));
      int e = 0;
      if (mx > 0.0) std::frexp(mx, &e);
      rscale[i] = std::ldexp(1.0f, e);
      for (int k = 0; k < kk; ++k) {
        long long x = std::llrint(std::ldexp(at(i, k), 31 - e));
        const int off = base + offset(i, k, sbo);
        for (int d = 3; d >= 0; --d) {  // least significant digit first
          const long long dig = d == 0 ? x : ((x + 128) & 255) - 128;
          x = (x - dig) >> 8;
          const uint16_t h = half_bits(static_cast<int>(dig));
          std::memcpy(out + off + d * slice, &h, 2);
        }
      }
    }
  };
  // tf32: at(i, k) = hi + lo (+ a remainder below 2^-22 relative), both TF32
  auto block_tf32 = [&](int base, int slice, int sbo, int kk, auto at) {
    for (int i = 0; i < np; ++i)
      for (int k = 0; k < kk; ++k) {
        const double x = at(i, k);
        const uint32_t hi = tf32_rna_bits(static_cast<float>(x));
        float hf;
        std::memcpy(&hf, &hi, 4);
        const uint32_t lo = tf32_rna_bits(static_cast<float>(x - static_cast<double>(hf)));
        const int off = base + offset(i, k, sbo);
        std::memcpy(out + off, &hi, 4);
        std::memcpy(out + off + slice, &lo, 4);
      }
  };
  auto vol = [&](int i, int k) {
    const int r = k / npp, j = k - r * npp;  // column r npp + j; j = np is padding
    return j < np ? diff[((size_t)r * np + i) * np + j] : 0.0;
  };
  auto lft = [&](int i, int k) { return lift[(size_t)i * nfpt + k]; };
  if (tf32) {
    block_tf32(0, bs_v, sbo_v, 3 * npp, vol);
    block_tf32(ops_l, bs_l, sbo_l, nfpt, lft);
  } else {
    block(0, bs_v, sbo_v, 3 * npp, ops_ev, vol);
    block(ops_l, bs_l, sbo_l, nfpt, ops_el, lft);
  }
  std::memcpy(out + ops_fn, face_nodes, (size_t)nfpt * 4);
  return total;
}
}  // namespace dg

namespace {

cudaError_t tc_shape_of(int eq, int order, int mode, dg::LaunchShape* out) {
  switch (eq) {
    case DG_WAVE: return dg::tc_shape_wave(order, mode, out);
    case DG_EULER: return dg::tc_shape_euler(order, mode, out);
    case DG_MAXWELL: return dg::tc_shape_maxwell(order, mode, out);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t tc_launch_of(int eq, int order, int mode, const dg::RhsArgs& a, int grid,
                         cudaStream_t s) {
  switch (eq) {
    case DG_WAVE: return dg::tc_launch_wave(order, mode, a, grid, s);
    case DG_EULER: return dg::tc_launch_euler(order, mode, a, grid, s);
    case DG_MAXWELL: return dg::tc_launch_maxwell(order, mode, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

// launch mode of tcgen05 form k (0 digits, 1 3xTF32, 2 3xTF32 at the other
// CTA size), RHS; | 1 for the RK stage
int tcm_mode(int k) { return k == 0 ? 0 : (k == 1 ? 2 : 6); }

cudaError_t tcm_shape_of(int eq, int order, int mode, dg::LaunchShape* out) {
  switch (eq) {
    case DG_WAVE: return dg::tcm_shape_wave(order, mode, out);
    case DG_EULER: return dg::tcm_shape_euler(order, mode, out);
    case DG_MAXWELL: return dg::tcm_shape_maxwell(order, mode, out);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t tcm_launch_of(int eq, int order, int mode, const dg::RhsArgs& a, int grid,
                          cudaStream_t s) {
  switch (eq) {
    case DG_WAVE: return dg::tcm_launch_wave(order, mode, a, grid, s);
    case DG_EULER: return dg::tcm_launch_euler(order, mode, a, grid, s);
    case DG_MAXWELL: return dg::tcm_launch_maxwell(order, mode, a, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

// }}}

}  // namespace

extern "C" {

const char* dg_last_error(void) { return g_last_error.c_str(); }

int32_t dg_abi_version(void) { return 7; }

int dg_plan_create(dg_plan** plan_out, int32_t equation, int32_t precision,
                   const dg_mesh_desc* mesh, const double* params,
                   int32_t nparams) {
  g_last_error.clear();
  if (!plan_out) return fail(DG_ERR_ARGUMENT, "plan output pointer is NULL");
  *plan_out = nullptr;
  if (!mesh) return fail(DG_ERR_ARGUMENT, "mesh description is NULL");
  const int nf = nfields_of(equation);
  if (nf == 0) return fail(DG_ERR_ARGUMENT, "unknown equation");
  if (precision != DG_FP64 && precision != DG_FP32_MIXED && precision != DG_FP64_TC)
    return fail(DG_ERR_ARGUMENT, "unknown precision");
  const int kprec = precision == DG_FP32_MIXED ? 1 : 0;  // kernel arithmetic type
  if (mesh->order < 1 || mesh->order > 4)
    return fail(DG_ERR_UNSUPPORTED, "order must be 1..4");
  if (mesh->nelements < 1) return fail(DG_ERR_ARGUMENT, "nelements must be >= 1");
  const int N = mesh->order;
  const int np = (N + 1) * (N + 2) * (N + 3) / 6;
  const int nfp = (N + 1) * (N + 2) / 2;
  if (mesh->nelements * (int64_t)np >= (int64_t(1) << 31))
    return fail(DG_ERR_ARGUMENT, "Nel * Np must be < 2^31 (31-bit gather indices)");
  if (!mesh->metric || !mesh->face_geom || !mesh->gather || !mesh->lift ||
      !mesh->face_nodes)
    return fail(DG_ERR_ARGUMENT, "a mesh array pointer is NULL");
  const double* diff =
      equation == DG_MAXWELL ? mesh->strong_diff : mesh->weak_diff;
  if (!diff)
    return fail(DG_ERR_ARGUMENT, equation == DG_MAXWELL ? "strong_diff is NULL"
                                                         : "weak_diff is NULL");
  if (nparams != nparams_of(equation) || (nparams > 0 && !params))
    return fail(DG_ERR_ARGUMENT, "wrong number of equation parameters");
  for (int k = 0; k < 4 * nfp; ++k)
    if (mesh->face_nodes[k] < 0 || mesh->face_nodes[k] >= np)
      return fail(DG_ERR_ARGUMENT, "face_nodes entry out of range");
  if (equation == DG_MAXWELL && (params[1] <= 0 || params[2] <= 0))
    return fail(DG_ERR_ARGUMENT, "epsilon and mu must be positive");
  for (const void* p : {(const void*)mesh->metric, (const void*)mesh->face_geom,
                        (const void*)mesh->gather}) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess ||
        attr.type != cudaMemoryTypeDevice) {
      cudaGetLastError();
      return fail(DG_ERR_ARGUMENT, "metric/face_geom/gather must be device memory");
    }
  }

  // face-shared path: FP64 plans on meshes that carry face_partner and whose
  // face points fit 31-bit indices; the fused kernel serves all others
  const bool split = mesh->face_partner && kprec == 0 &&
                     mesh->nelements * 4 * (int64_t)nfp < (int64_t(1) << 31);
  const bool tc = split && precision == DG_FP64_TC && N >= 3;
  if (mesh->face_partner) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, mesh->face_partner) != cudaSuccess ||
        attr.type != cudaMemoryTypeDevice) {
      cudaGetLastError();
      return fail(DG_ERR_ARGUMENT, "face_partner must be device memory");
    }
  }

  // the persistent grid fits the modes the plan launches: RHS and RK stage,
  // in the face-shared form on the split path
  dg::LaunchShape shape;
  const int base_mode = split ? dg::MODE_SPLIT : dg::MODE_RHS;
  cudaError_t err = shape_of(equation, N, kprec, base_mode, &shape);
  if (err == cudaSuccess) {
    dg::LaunchShape other;
    err = shape_of(equation, N, kprec, base_mode | dg::MODE_STAGE, &other);
    if (other.blocks_per_sm < shape.blocks_per_sm)
      shape.blocks_per_sm = other.blocks_per_sm;
  }
  if (err != cudaSuccess) return cuda_fail(err, "kernel configuration");
  if (shape.blocks_per_sm < 1)
    return fail(DG_ERR_UNSUPPORTED, "kernel does not fit on an SM");
  const int rs = kprec == 0 ? 8 : 4;
  const dg::OpsOffsets off = dg::ops_offsets(np, nfp, rs);
  if (off.size != shape.ops_bytes)
    return fail(DG_ERR_CUDA, "operator layout mismatch between host and kernel");

  std::vector<unsigned char> ops(off.size, 0);
  if (kprec == 0)
    pack_ops_fp64(ops, off, np, nfp, diff, mesh->lift, mesh->face_nodes);
  else
    pack_ops_fp32(ops, off, np, nfp, diff, mesh->lift, mesh->face_nodes);

  dg_plan* p = new dg_plan;
  p->equation = equation;
  p->precision = precision;
  p->order = N;
  p->np = np;
  p->nfp = nfp;
  p->nfields = nf;
  p->nel = mesh->nelements;
  p->metric = mesh->metric;
  p->face_geom = mesh->face_geom;
  p->gather = mesh->gather;
  p->shape = shape;
  p->ops_bytes = static_cast<uint32_t>(off.size);
  for (int k = 0; k < nparams; ++k) p->params[k] = params[k];
  if (equation == DG_MAXWELL) {  // flux and mass constants, once per plan
    const double z = std::sqrt(params[2] / params[1]), y = 1.0 / z;
    p->k[0] = z;
    p->k[1] = y;
    p->k[2] = -1.0 / (z + z);
    p->k[3] = 1.0 / (y + y);
    p->k[4] = 1.0 / params[1];
    p->k[5] = 1.0 / params[2];
  }
  cudaGetDevice(&p->device);

  err = cudaMalloc(&p->d_ops, p->ops_bytes);
  if (err == cudaSuccess) err = cudaMalloc(&p->d_status, sizeof(int));
  if (err == cudaSuccess)
    err = cudaMemcpy(p->d_ops, ops.data(), p->ops_bytes, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemset(p->d_status, 0, sizeof(int));
  if (err != cudaSuccess) {
    dg_plan_destroy(p);
    return cuda_fail(err, "plan buffers");
  }
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device);
  p->nsm = nsm;
  const int64_t ntiles =
      (p->nel + shape.elems_per_tile - 1) / shape.elems_per_tile;
  const int64_t full = (int64_t)nsm * shape.blocks_per_sm;
  p->grid = (int)(ntiles < full ? ntiles : full);
  p->ntiles = ntiles;
  if (kprec == 1) {  // the tensor-core variant of the mixed kernel
    dg::LaunchShape t0, t1;
    err = shape_of(equation, N, 1, dg::MODE_TC, &t0);
    if (err == cudaSuccess) err = shape_of(equation, N, 1, dg::MODE_TC | dg::MODE_STAGE, &t1);
    if (err != cudaSuccess) {
      dg_plan_destroy(p);
      return cuda_fail(err, "tensor-core mixed kernel configuration");
    }
    const int bps = t1.blocks_per_sm < t0.blocks_per_sm ? t1.blocks_per_sm : t0.blocks_per_sm;
    const int64_t tfull = (int64_t)nsm * (bps > 0 ? bps : 1);
    p->grid_mtc = (int)(ntiles < tfull ? ntiles : tfull);
    // the same products at the other tile shapes (variants 7-10); a shape
    // that does not fit on an SM stays unsupported
    for (int k = 0; k < 2; ++k) {
      dg::LaunchShape b0, b1;
      err = shape_of(equation, N, 1, dg::MODE_TC | kShapeModeBits[k], &b0);
      if (err == cudaSuccess)
        err = shape_of(equation, N, 1, dg::MODE_TC | dg::MODE_STAGE | kShapeModeBits[k], &b1);
      if (err != cudaSuccess) {
        dg_plan_destroy(p);
        return cuda_fail(err, "tensor-core mixed kernel tile shapes");
      }
      if (b1.blocks_per_sm < b0.blocks_per_sm) b0.blocks_per_sm = b1.blocks_per_sm;
      if (b0.blocks_per_sm < 1 || b0.elems_per_tile < 1) continue;
      p->tcb[k] = true;
      p->tcb_shape[k] = b0;
      p->tcb_ntiles[k] = (p->nel + b0.elems_per_tile - 1) / b0.elems_per_tile;
      const int64_t bfull = (int64_t)nsm * b0.blocks_per_sm;
      p->tcb_grid[k] = (int)(p->tcb_ntiles[k] < bfull ? p->tcb_ntiles[k] : bfull);
    }
    // the tcgen05 forms (variants 4, 5 and 6)
    for (int k = 0; k < 3; ++k) {
      dg::LaunchShape m0, m1;
      err = tcm_shape_of(equation, N, tcm_mode(k), &m0);
      if (err == cudaSuccess) err = tcm_shape_of(equation, N, tcm_mode(k) | 1, &m1);
      const int mbytes =
          dg::pack_tcm_ops(N, diff, mesh->lift, mesh->face_nodes, nullptr, 0, k >= 1);
      if (err != cudaSuccess || mbytes != m0.ops_bytes) {
        dg_plan_destroy(p);
        return err != cudaSuccess ? cuda_fail(err, "tcgen05 mixed kernel configuration")
                                  : fail(DG_ERR_CUDA, "tcgen05 operator layout mismatch");
      }
      if (m1.blocks_per_sm < m0.blocks_per_sm) m0.blocks_per_sm = m1.blocks_per_sm;
      if (m0.blocks_per_sm < 1) continue;
      if (k == 2 && p->tcm[1]) {  // same operator block as variant 5
        p->d_tcm_ops[2] = p->d_tcm_ops[1];
      } else {
        std::vector<unsigned char> mops(mbytes);
        dg::pack_tcm_ops(N, diff, mesh->lift, mesh->face_nodes, mops.data(), mbytes, k >= 1);
        err = cudaMalloc(&p->d_tcm_ops[k], mbytes);
        if (err == cudaSuccess)
          err = cudaMemcpy(p->d_tcm_ops[k], mops.data(), mbytes, cudaMemcpyHostToDevice);
        if (err != cudaSuccess) {
          dg_plan_destroy(p);
          return cuda_fail(err, "tcgen05 operator buffer");
        }
      }
      p->tcm[k] = true;
      p->tcm_ops_bytes[k] = static_cast<uint32_t>(mbytes);
      p->tcm_shape[k] = m0;
      const int64_t mtiles = (p->nel + m0.elems_per_tile - 1) / m0.elems_per_tile;
      const int64_t mfull = (int64_t)nsm * m0.blocks_per_sm;
      p->tcm_grid[k] = (int)(mtiles < mfull ? mtiles : mfull);
    }
  }
  p->face_partner = mesh->face_partner;

  if (kprec == 1 && equation == DG_EULER) {
    err = cudaMalloc(&p->d_pres, (size_t)p->nel * np * sizeof(float));
    if (err != cudaSuccess) {
      dg_plan_destroy(p);
      return cuda_fail(err, "pressure table");
    }
    const int64_t pblocks = (p->nel * np + dg::kFaceBlock - 1) / dg::kFaceBlock;
    const int64_t pfull = (int64_t)nsm * 8;
    p->pres_grid = (int)(pblocks < pfull ? pblocks : pfull);
  }

  if (split) {
    p->d_face_nodes = reinterpret_cast<const int32_t*>(
        static_cast<const unsigned char*>(p->d_ops) + off.fn);
    const int code = setup_split(p, mesh->face_partner, p->d_face_nodes);
    if (code != DG_OK) {
      dg_plan_destroy(p);
      return code;
    }
  }

  if (tc) {
    dg::LaunchShape ts, ts_stage;
    err = tc_shape_of(equation, N, 0, &ts);
    if (err == cudaSuccess) err = tc_shape_of(equation, N, 1, &ts_stage);
    if (err != cudaSuccess) {
      dg_plan_destroy(p);
      return cuda_fail(err, "tensor-core kernel configuration");
    }
    if (ts_stage.blocks_per_sm < ts.blocks_per_sm) ts.blocks_per_sm = ts_stage.blocks_per_sm;
    const int bytes = dg::pack_tc_ops(equation, N, diff, mesh->lift, nullptr, 0);
    if (bytes != ts.ops_bytes || ts.blocks_per_sm < 1) {
      dg_plan_destroy(p);
      return fail(DG_ERR_CUDA, ts.blocks_per_sm < 1
                                   ? "tensor-core kernel does not fit on an SM"
                                   : "tensor-core operator layout mismatch");
    }
    std::vector<unsigned char> tops(bytes);
    dg::pack_tc_ops(equation, N, diff, mesh->lift, tops.data(), bytes);
    err = cudaMalloc(&p->d_tc_ops, bytes);
    if (err == cudaSuccess)
      err = cudaMemcpy(p->d_tc_ops, tops.data(), bytes, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
      dg_plan_destroy(p);
      return cuda_fail(err, "tensor-core operator buffer");
    }
    p->tc = true;
    p->tc_ops_bytes = static_cast<uint32_t>(bytes);
    p->tc_shape = ts;
    const int64_t tiles = (p->nel + ts.elems_per_tile - 1) / ts.elems_per_tile;
    const int64_t tfull = (int64_t)nsm * ts.blocks_per_sm;
    p->tc_grid = (int)(tiles < tfull ? tiles : tfull);
  }

  // adjoint operators: wave (transpose) and, on the face-shared path, Euler
  // (transposed Jacobian)
  if (mesh->face_partner && kprec == 0 &&
      (equation == DG_WAVE || (equation == DG_EULER && split))) {
    if (p->nel * 8 * (int64_t)nfp >= (int64_t(1) << 32)) {
      dg_plan_destroy(p);
      return fail(DG_ERR_ARGUMENT, "mesh too large for the adjoint's 32-bit face indices");
    }
    dg::LaunchShape ashape;
    err = equation == DG_WAVE ? dg::adjoint_shape_wave(N, &ashape)
                              : dg::vjp_shape_euler(N, &ashape);
    if (err != cudaSuccess || ashape.blocks_per_sm < 1) {
      dg_plan_destroy(p);
      return err != cudaSuccess ? cuda_fail(err, "adjoint configuration")
                                : fail(DG_ERR_UNSUPPORTED, "adjoint does not fit");
    }
    const int w_off = 0;
    const int l_off = dg::pad16_host(3 * np * np * 8);
    const int fn_off = l_off + dg::pad16_host(4 * nfp * np * 8);
    const int size = fn_off + dg::pad16_host(4 * nfp * 4);
    if (size != ashape.ops_bytes) {
      dg_plan_destroy(p);
      return fail(DG_ERR_CUDA, "adjoint operator layout mismatch");
    }
    std::vector<unsigned char> aops(size, 0);
    pack_adj_ops(aops, np, nfp, diff, mesh->lift, mesh->face_nodes, w_off, l_off,
                 fn_off);
    err = cudaMalloc(&p->d_adj_ops, size);
    if (err == cudaSuccess)
      err = cudaMemcpy(p->d_adj_ops, aops.data(), size, cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
      dg_plan_destroy(p);
      return cuda_fail(err, "adjoint buffers");
    }
    p->adj_ops_bytes = static_cast<uint32_t>(size);
    const int64_t atiles = (p->nel + ashape.elems_per_tile - 1) / ashape.elems_per_tile;
    const int64_t afull = (int64_t)nsm * ashape.blocks_per_sm;
    p->adj_grid = (int)(atiles < afull ? atiles : afull);
  }
  *plan_out = p;
  return DG_OK;
}

int dg_plan_create_2d(dg_plan** plan_out, int32_t equation,
                      const dg_mesh2d_desc* mesh, const double* params,
                      int32_t nparams) {
  g_last_error.clear();
  if (!plan_out) return fail(DG_ERR_ARGUMENT, "plan output pointer is NULL");
  *plan_out = nullptr;
  if (!mesh) return fail(DG_ERR_ARGUMENT, "mesh description is NULL");
  const int nf = equation == DG_WAVE ? 3 : (equation == DG_EULER ? 4 : (equation == DG_MAXWELL ? 3 : 0));
  if (nf == 0) return fail(DG_ERR_ARGUMENT, "unknown equation");
  if (mesh->order < 1 || mesh->order > 4)
    return fail(DG_ERR_UNSUPPORTED, "order must be 1..4");
  if (mesh->nelements < 1) return fail(DG_ERR_ARGUMENT, "nelements must be >= 1");
  const int N = mesh->order;
  const int np = (N + 1) * (N + 2) / 2, nfp = N + 1;
  if (mesh->nelements * (int64_t)np >= (int64_t(1) << 31))
    return fail(DG_ERR_ARGUMENT, "Nel * Np must be < 2^31 (31-bit gather indices)");
  if (!mesh->metric || !mesh->face_geom || !mesh->gather || !mesh->lift ||
      !mesh->face_nodes)
    return fail(DG_ERR_ARGUMENT, "a mesh array pointer is NULL");
  const double* diff = equation == DG_MAXWELL ? mesh->strong_diff : mesh->weak_diff;
  if (!diff)
    return fail(DG_ERR_ARGUMENT, equation == DG_MAXWELL ? "strong_diff is NULL"
                                                         : "weak_diff is NULL");
  if (nparams != nparams_of(equation) || (nparams > 0 && !params))
    return fail(DG_ERR_ARGUMENT, "wrong number of equation parameters");
  for (int k = 0; k < 3 * nfp; ++k)
    if (mesh->face_nodes[k] < 0 || mesh->face_nodes[k] >= np)
      return fail(DG_ERR_ARGUMENT, "face_nodes entry out of range");
  if (equation == DG_MAXWELL && (params[1] <= 0 || params[2] <= 0))
    return fail(DG_ERR_ARGUMENT, "epsilon and mu must be positive");
  for (const void* ptr : {(const void*)mesh->metric, (const void*)mesh->face_geom,
                          (const void*)mesh->gather}) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, ptr) != cudaSuccess ||
        attr.type != cudaMemoryTypeDevice) {
      cudaGetLastError();
      return fail(DG_ERR_ARGUMENT, "metric, face_geom and gather must be device memory");
    }
  }
  // each mode's persistent grid from its own occupancy (the RK-stage kernel
  // may hold more registers than the RHS kernel)
  dg::LaunchShape shape, other;
  cudaError_t err = dg::shape_2d(equation, N, dg::MODE_RHS, &shape);
  if (err == cudaSuccess) err = dg::shape_2d(equation, N, dg::MODE_STAGE, &other);
  if (err != cudaSuccess) return cuda_fail(err, "2D kernel configuration");
  if (shape.blocks_per_sm < 1 || other.blocks_per_sm < 1)
    return fail(DG_ERR_UNSUPPORTED, "kernel does not fit on an SM");
  const int ops_bytes = dg::pack_ops_2d(N, diff, mesh->lift, mesh->face_nodes, nullptr, 0);
  if (ops_bytes != shape.ops_bytes)
    return fail(DG_ERR_CUDA, "operator layout mismatch between host and kernel");
  std::vector<unsigned char> ops(ops_bytes, 0);
  dg::pack_ops_2d(N, diff, mesh->lift, mesh->face_nodes, ops.data(), ops_bytes);

  dg_plan* p = new dg_plan;
  p->dim = 2;
  p->equation = equation;
  p->precision = DG_FP64;
  p->order = N;
  p->np = np;
  p->nfp = nfp;
  p->nfields = nf;
  p->nel = mesh->nelements;
  p->metric = mesh->metric;
  p->face_geom = mesh->face_geom;
  p->gather = mesh->gather;
  p->shape = shape;
  p->ops_bytes = static_cast<uint32_t>(ops_bytes);
  for (int k = 0; k < nparams; ++k) p->params[k] = params[k];
  if (equation == DG_MAXWELL) {  // flux and mass constants, as in 3D
    const double z = std::sqrt(params[2] / params[1]), y = 1.0 / z;
    p->k[0] = z;
    p->k[1] = y;
    p->k[2] = -1.0 / (z + z);
    p->k[3] = 1.0 / (y + y);
    p->k[4] = 1.0 / params[1];
    p->k[5] = 1.0 / params[2];
  }
  cudaGetDevice(&p->device);
  err = cudaMalloc(&p->d_ops, p->ops_bytes);
  if (err == cudaSuccess) err = cudaMalloc(&p->d_status, sizeof(int));
  if (err == cudaSuccess)
    err = cudaMemcpy(p->d_ops, ops.data(), p->ops_bytes, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemset(p->d_status, 0, sizeof(int));
  if (err != cudaSuccess) {
    dg_plan_destroy(p);
    return cuda_fail(err, "plan buffers");
  }
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device);
  p->nsm = nsm;
  p->ntiles = (p->nel + shape.elems_per_tile - 1) / shape.elems_per_tile;
  const int64_t full = (int64_t)nsm * shape.blocks_per_sm;
  const int64_t full_stage = (int64_t)nsm * other.blocks_per_sm;
  p->grid = (int)(p->ntiles < full ? p->ntiles : full);
  p->grid_stage = (int)(p->ntiles < full_stage ? p->ntiles : full_stage);
  *plan_out = p;
  return DG_OK;
}

int dg_plan_set_variant(dg_plan* p, int32_t variant) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (p->dim == 2 && variant != 0)
    return fail(DG_ERR_UNSUPPORTED, "triangle-mesh plans have one variant");
  if (variant < 0 || variant >= DG_NUM_VARIANTS)
    return fail(DG_ERR_ARGUMENT, "variant must be 0..10");
  if (((variant & 1) || is_shape_variant(variant)) && p->precision != DG_FP32_MIXED)
    return fail(DG_ERR_UNSUPPORTED, "tensor-core products are a mixed-precision variant");
  if (is_tcm_variant(variant) && !p->tcm[variant - 4])
    return fail(DG_ERR_UNSUPPORTED, "the tcgen05 kernels are mixed-precision variants");
  if (is_shape_variant(variant) && !p->tcb[shape_index(variant)])
    return fail(DG_ERR_UNSUPPORTED, "this tile shape does not fit on an SM");
  if (p->tc) return fail(DG_ERR_UNSUPPORTED, "DG_FP64_TC plans have one variant");
  p->variant = variant;
  return DG_OK;
}

}  // extern "C"

namespace {

// Relative L2 distance ||a - b|| / ||b|| of two device arrays of n doubles
// (deterministic: fixed grid, fixed-order block and host sums).
int rel_l2_device(const double* a, const double* b, int64_t n, cudaStream_t s,
                  double* out) {
  double* d_part = nullptr;
  cudaError_t err = cudaMalloc(&d_part, 2 * kNormBlocks * sizeof(double));
  std::vector<double> part(2 * kNormBlocks, 0.0);
  if (err == cudaSuccess) {
    diff_norm_kernel<<<kNormBlocks, 256, 0, s>>>(a, b, n, d_part);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(part.data(), d_part, part.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (d_part) cudaFree(d_part);
  if (err != cudaSuccess) return cuda_fail(err, "autotune error check");
  double d2 = 0.0, b2 = 0.0;
  for (int k = 0; k < kNormBlocks; ++k) {
    d2 += part[2 * k];
    b2 += part[2 * k + 1];
  }
  *out = b2 > 0.0 ? std::sqrt(d2 / b2) : std::sqrt(d2);
  return DG_OK;
}

// Read and clear the plan's device status word (after the stream drained).
int take_status(dg_plan* p, cudaStream_t s, int* status) {
  cudaError_t err = cudaStreamSynchronize(s);
  if (err == cudaSuccess)
    err = cudaMemcpy(status, p->d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (err == cudaSuccess && *status != 0) err = cudaMemset(p->d_status, 0, sizeof(int));
  if (err != cudaSuccess) return cuda_fail(err, "status read");
  return DG_OK;
}

// Shared by dg_plan_autotune and dg_plan_autotune_bounded: time every
// supported variant; a variant whose launches raised a device status
// (timeout, bad index) is dropped and reported as -1; with `ref`, a
// variant whose result differs from ref by more than max_rel_l2 (relative
// L2) is not chosen unless none meets the bound, in which case the most
// accurate variant is kept.
int autotune_impl(dg_plan* p, const double* q, double* rhs, const double* ref,
                  double max_rel_l2, int32_t reps, void* stream, int32_t* chosen,
                  float* ms_per_variant, double* err_per_variant) {
  if (p->dim == 2) return fail(DG_ERR_UNSUPPORTED, "triangle-mesh plans have one variant");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int nvar = p->tc ? 1 : DG_NUM_VARIANTS;
  const int64_t n = (int64_t)p->nfields * p->nel * p->np;
  cudaEvent_t e0, e1;
  cudaError_t err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  if (err != cudaSuccess) return cuda_fail(err, "autotune events");
  const int saved = p->variant;
  int best = -1, best_acc = -1, first_status = 0;
  float best_ms = 0.f;
  double best_err = 0.0;
  int code = DG_OK;
  for (int v = 0; v < DG_NUM_VARIANTS && code == DG_OK; ++v) {
    float ms = -1.f;
    double rel = -1.0;
    const bool have = v < 4 || (is_tcm_variant(v) && p->tcm[v - 4]) ||
                      (is_shape_variant(v) && p->tcb[shape_index(v)]);
    const bool mixed_only = (v & 1) || is_shape_variant(v);
    if (v < nvar && have && (!mixed_only || p->precision == DG_FP32_MIXED)) {
      p->variant = v;
      code = dg_rhs(p, q, rhs, stream);  // warm-up
      if (code == DG_OK) err = cudaEventRecord(e0, s);
      for (int r = 0; r < reps && code == DG_OK && err == cudaSuccess; ++r)
        code = dg_rhs(p, q, rhs, stream);
      if (code == DG_OK && err == cudaSuccess) err = cudaEventRecord(e1, s);
      if (code == DG_OK && err == cudaSuccess) err = cudaEventSynchronize(e1);
      if (code == DG_OK && err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
      if (code == DG_OK && err != cudaSuccess) code = cuda_fail(err, "autotune timing");
      int status = 0;
      if (code == DG_OK) code = take_status(p, s, &status);
      if (code == DG_OK && status != 0) {  // the variant failed on the device
        if (!first_status) first_status = status;
        ms = -1.f;
      } else if (code == DG_OK) {
        ms /= (float)reps;
        if (ref) code = rel_l2_device(rhs, ref, n, s, &rel);
      }
      if (code == DG_OK && ms >= 0.f) {
        const bool within = !ref || rel <= max_rel_l2;
        if (within && (best < 0 || ms < best_ms)) {
          best = v;
          best_ms = ms;
        }
        if (ref && (best_acc < 0 || rel < best_err)) {
          best_acc = v;
          best_err = rel;
        }
      }
    }
    if (ms_per_variant) ms_per_variant[v] = ms;
    if (err_per_variant) err_per_variant[v] = rel;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best < 0) best = best_acc;
  p->variant = code == DG_OK && best >= 0 ? best : saved;
  if (chosen) *chosen = p->variant;
  if (code == DG_OK && best < 0 && first_status)
    return fail(first_status, "every autotuned variant raised a device-side error");
  return code;
}

dg::VjpArgs vjp_args(const dg_plan* p, const double* q, const double* x, double* y) {
  dg::VjpArgs a;
  std::memset(&a, 0, sizeof(a));
  a.q = q;
  a.x = x;
  a.y = y;
  a.aux = p->d_aux;
  a.scratch = p->d_flux;
  a.elem_scale = p->elem_scale;
  a.metric = p->metric;
  a.face_geom = p->face_geom;
  a.gather = p->gather;
  a.partner = p->face_partner;
  a.owned = p->d_owned;
  a.nowned = p->nowned;
  a.ops = p->d_adj_ops;
  a.ops_bytes = p->adj_ops_bytes;
  a.nel = p->nel;
  a.status = p->d_status;
  a.gamma = p->params[0];
  a.xscale = 1.0;
  return a;
}

}  // namespace

extern "C" {

int dg_plan_autotune(dg_plan* p, const double* q, double* rhs, int32_t reps,
                     void* stream, int32_t* chosen, float* ms_per_variant) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!q || !rhs || reps < 1) return fail(DG_ERR_ARGUMENT, "bad autotune arguments");
  return autotune_impl(p, q, rhs, nullptr, 0.0, reps, stream, chosen, ms_per_variant,
                       nullptr);
}

int dg_plan_autotune_bounded(dg_plan* p, const double* q, double* rhs,
                             const double* ref, double max_rel_l2, int32_t reps,
                             void* stream, int32_t* chosen, float* ms_per_variant,
                             double* err_per_variant) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!q || !rhs || !ref || reps < 1 || !(max_rel_l2 >= 0.0))
    return fail(DG_ERR_ARGUMENT, "bad autotune arguments");
  const int64_t bytes = (int64_t)p->nfields * p->nel * p->np * 8;
  if (overlap(ref, rhs, bytes)) return fail(DG_ERR_ARGUMENT, "ref and rhs overlap");
  return autotune_impl(p, q, rhs, ref, max_rel_l2, reps, stream, chosen, ms_per_variant,
                       err_per_variant);
}

int dg_plan_set_element_scale(dg_plan* p, const double* scale) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (scale) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, scale) != cudaSuccess ||
        attr.type != cudaMemoryTypeDevice) {
      cudaGetLastError();
      return fail(DG_ERR_ARGUMENT, "element scale must be device memory");
    }
  }
  p->elem_scale = scale;
  return DG_OK;
}

int dg_rhs_adjoint(dg_plan* p, const double* x, double* y, double* face_scratch,
                   void* stream) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!p->d_adj_ops || p->equation != DG_WAVE)
    return fail(DG_ERR_UNSUPPORTED,
                "adjoint needs an FP64 wave plan built with face_partner");
  if (!x || !y || !face_scratch)
    return fail(DG_ERR_ARGUMENT, "x, y or face_scratch is NULL");
  const int64_t bytes = (int64_t)p->nfields * p->nel * p->np * 8;
  const int64_t sbytes = p->nel * 2 * 4 * (int64_t)p->nfp * 8;
  if (overlap(x, y, bytes) || overlap2(x, bytes, face_scratch, sbytes) ||
      overlap2(y, bytes, face_scratch, sbytes))
    return fail(DG_ERR_ARGUMENT, "x, y and face_scratch must not overlap");
  dg::AdjArgs a;
  std::memset(&a, 0, sizeof(a));
  a.x = x;
  a.y = y;
  a.face_scratch = face_scratch;
  a.elem_scale = p->elem_scale;
  a.c = p->params[0];
  a.metric = p->metric;
  a.face_geom = p->face_geom;
  a.face_partner = p->face_partner;
  a.ops = p->d_adj_ops;
  a.ops_bytes = p->adj_ops_bytes;
  a.nel = p->nel;
  a.status = p->d_status;
  cudaError_t err = dg::adjoint_launch_wave(p->order, a, p->adj_grid, p->nsm,
                                            reinterpret_cast<cudaStream_t>(stream));
  if (err != cudaSuccess) return cuda_fail(err, "adjoint launch");
  return DG_OK;
}

int dg_rhs_adjoint_stage(dg_plan* p, const double* x, double xscale, double* lam,
                         double* rbar_out, const double* lq, double* cbar, double a_coef,
                         double b_coef, double dt, double* y_scratch, void* stream) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!p->d_adj_ops || p->equation != DG_WAVE || !p->split)
    return fail(DG_ERR_UNSUPPORTED,
                "the adjoint stage needs an FP64 wave plan on the face-shared path "
                "(mesh with face_partner)");
  if (!x || !lam || !y_scratch)
    return fail(DG_ERR_ARGUMENT, "x, lam or y_scratch is NULL");
  if ((cbar != nullptr) != (lq != nullptr))
    return fail(DG_ERR_ARGUMENT, "lq and cbar go together");
  const int64_t bytes = (int64_t)p->nfields * p->nel * p->np * 8;
  // x may be lam or rbar_out itself (each node reads before it writes), but no
  // other overlap is allowed
  auto bad = [&](const void* u, const void* v) { return u != v && overlap(u, v, bytes); };
  if (bad(x, lam) || (rbar_out && (bad(x, rbar_out) || overlap(lam, rbar_out, bytes))) ||
      overlap(y_scratch, x, bytes) || overlap(y_scratch, lam, bytes) ||
      (rbar_out && overlap(y_scratch, rbar_out, bytes)) ||
      (lq && (overlap(lq, lam, bytes) || overlap(lq, y_scratch, bytes) ||
              (rbar_out && overlap(lq, rbar_out, bytes)))) ||
      (cbar && (overlap2(cbar, p->nel * 8, lam, bytes) ||
                overlap2(cbar, p->nel * 8, y_scratch, bytes) ||
                (rbar_out && overlap2(cbar, p->nel * 8, rbar_out, bytes)))))
    return fail(DG_ERR_ARGUMENT, "adjoint stage arrays overlap");
  dg::AdjArgs a;
  std::memset(&a, 0, sizeof(a));
  a.x = x;
  a.y = y_scratch;
  a.face_scratch = p->d_flux;
  a.elem_scale = p->elem_scale;
  a.c = p->params[0];
  a.metric = p->metric;
  a.face_geom = p->face_geom;
  a.face_partner = p->face_partner;
  a.ops = p->d_adj_ops;
  a.ops_bytes = p->adj_ops_bytes;
  a.nel = p->nel;
  a.status = p->d_status;
  a.xscale = xscale;
  a.lam = lam;
  a.rbar_out = rbar_out;
  a.lq = lq;
  a.cbar = cbar;
  a.rk_a = a_coef;
  a.rk_b = b_coef;
  a.dt = dt;
  cudaError_t err = dg::adjoint_stage_launch_wave(p->order, a, p->adj_grid, p->nsm,
                                                  reinterpret_cast<cudaStream_t>(stream));
  if (err != cudaSuccess) return cuda_fail(err, "adjoint stage launch");
  return DG_OK;
}

int dg_rhs_vjp(dg_plan* p, const double* q, const double* x, double* y,
               void* stream) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!q || !x || !y) return fail(DG_ERR_ARGUMENT, "q, x or y is NULL");
  if (!p->d_adj_ops || !p->split)
    return fail(DG_ERR_UNSUPPORTED,
                "the transposed Jacobian needs an FP64 wave or Euler plan built "
                "with face_partner");
  const int64_t bytes = (int64_t)p->nfields * p->nel * p->np * 8;
  if (overlap(y, q, bytes) || overlap(y, x, bytes))
    return fail(DG_ERR_ARGUMENT, "y must not overlap q or x");
  if (p->equation == DG_WAVE)  // linear: the transpose, scratch in the face buffer
    return dg_rhs_adjoint(p, x, y, p->d_flux, stream);
  dg::VjpArgs a = vjp_args(p, q, x, y);
  cudaError_t err = dg::vjp_launch_euler(p->order, a, p->adj_grid, p->nsm, false,
                                         reinterpret_cast<cudaStream_t>(stream));
  if (err != cudaSuccess) return cuda_fail(err, "vjp launch");
  return DG_OK;
}

int dg_rhs_vjp_stage(dg_plan* p, const double* q, const double* x, double xscale,
                     double* lam, double* rbar_out, double a_coef, double b_coef,
                     double dt, double* y_scratch, void* stream) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!p->d_adj_ops || !p->split)
    return fail(DG_ERR_UNSUPPORTED,
                "the reverse stage needs an FP64 wave or Euler plan built with "
                "face_partner");
  if (p->equation == DG_WAVE)  // linear: q is not read
    return dg_rhs_adjoint_stage(p, x, xscale, lam, rbar_out, nullptr, nullptr, a_coef,
                                b_coef, dt, y_scratch, stream);
  if (!q || !x || !lam || !y_scratch)
    return fail(DG_ERR_ARGUMENT, "q, x, lam or y_scratch is NULL");
  const int64_t bytes = (int64_t)p->nfields * p->nel * p->np * 8;
  // x may be lam or rbar_out itself (each node reads before it writes); q is
  // only read, and may not overlap a written array
  auto bad = [&](const void* u, const void* v) { return u != v && overlap(u, v, bytes); };
  if (bad(x, lam) || (rbar_out && (bad(x, rbar_out) || overlap(lam, rbar_out, bytes))) ||
      overlap(y_scratch, x, bytes) || overlap(y_scratch, lam, bytes) ||
      overlap(y_scratch, q, bytes) || overlap(q, lam, bytes) ||
      (rbar_out && (overlap(y_scratch, rbar_out, bytes) || overlap(q, rbar_out, bytes))))
    return fail(DG_ERR_ARGUMENT, "reverse stage arrays overlap");
  dg::VjpArgs a = vjp_args(p, q, x, y_scratch);
  a.xscale = xscale;
  a.lam = lam;
  a.rbar_out = rbar_out;
  a.rk_a = a_coef;
  a.rk_b = b_coef;
  a.dt = dt;
  cudaError_t err = dg::vjp_launch_euler(p->order, a, p->adj_grid, p->nsm, true,
                                         reinterpret_cast<cudaStream_t>(stream));
  if (err != cudaSuccess) return cuda_fail(err, "reverse stage launch");
  return DG_OK;
}

int dg_rhs(dg_plan* p, const double* q, double* rhs, void* stream) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!q || !rhs) return fail(DG_ERR_ARGUMENT, "state or rhs pointer is NULL");
  const int64_t bytes = (int64_t)p->nfields * p->nel * p->np * 8;
  if (overlap(q, rhs, bytes)) return fail(DG_ERR_ARGUMENT, "state and rhs overlap");
  dg::RhsArgs a = base_args(p);
  a.q = q;
  a.rhs = rhs;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (p->dim == 2) {
    cudaError_t err = dg::launch_2d(p->equation, p->order, dg::MODE_RHS, a, p->grid, s);
    if (err != cudaSuccess) return cuda_fail(err, "rhs launch");
    return DG_OK;
  }
  if (p->split) {
    cudaError_t err = launch_faces(p, q, s);
    if (err != cudaSuccess) return cuda_fail(err, "face kernel launch");
  }
  if (p->d_pres) {
    cudaError_t err = dg::pressure_launch_euler(q, p->d_pres, p->nel * p->np,
                                                p->params[0], p->pres_grid, s);
    if (err != cudaSuccess) return cuda_fail(err, "pressure kernel launch");
  }
  cudaError_t err;
  if (p->tc) {
    a.ops = p->d_tc_ops;
    a.ops_bytes = p->tc_ops_bytes;
    err = tc_launch_of(p->equation, p->order, 0, a, p->tc_grid, s);
  } else if (is_tcm_variant(p->variant)) {
    const int k = p->variant - 4;
    a.ops = p->d_tcm_ops[k];
    a.ops_bytes = p->tcm_ops_bytes[k];
    err = tcm_launch_of(p->equation, p->order, tcm_mode(k), a, p->tcm_grid[k], s);
  } else {
    err = launch_of(p->equation, p->order, p->precision == DG_FP32_MIXED ? 1 : 0,
                    main_mode(p, p->split ? dg::MODE_SPLIT : dg::MODE_RHS), a,
                    main_grid(p), s);
  }
  if (err != cudaSuccess) return cuda_fail(err, "rhs launch");
  return DG_OK;
}

int dg_rk_stage(dg_plan* p, const double* q_in, double* q_out, double* res,
                double a_coef, double b_coef, double dt, double* rhs_unscaled,
                void* stream) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!q_in || !q_out || !res)
    return fail(DG_ERR_ARGUMENT, "state, output or residual pointer is NULL");
  const int64_t bytes = (int64_t)p->nfields * p->nel * p->np * 8;
  if (overlap(q_in, q_out, bytes) || overlap(q_in, res, bytes) ||
      overlap(q_out, res, bytes))
    return fail(DG_ERR_ARGUMENT, "q_in, q_out and res must not overlap");
  dg::RhsArgs a = base_args(p);
  a.q = q_in;
  a.q_out = q_out;
  a.res = res;
  a.rk_a = a_coef;
  a.rk_b = b_coef;
  a.rk_dt = dt;
  if (rhs_unscaled) {
    if (overlap(rhs_unscaled, q_in, bytes) || overlap(rhs_unscaled, q_out, bytes) ||
        overlap(rhs_unscaled, res, bytes))
      return fail(DG_ERR_ARGUMENT, "rhs_unscaled overlaps another array");
    a.rhs_unscaled = rhs_unscaled;
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (p->dim == 2) {
    cudaError_t err = dg::launch_2d(p->equation, p->order, dg::MODE_STAGE, a, p->grid_stage, s);
    if (err != cudaSuccess) return cuda_fail(err, "rk stage launch");
    return DG_OK;
  }
  if (p->split) {
    cudaError_t err = launch_faces(p, q_in, s);
    if (err != cudaSuccess) return cuda_fail(err, "face kernel launch");
  }
  if (p->d_pres) {
    cudaError_t err = dg::pressure_launch_euler(q_in, p->d_pres, p->nel * p->np,
                                                p->params[0], p->pres_grid, s);
    if (err != cudaSuccess) return cuda_fail(err, "pressure kernel launch");
  }
  cudaError_t err;
  if (p->tc) {
    a.ops = p->d_tc_ops;
    a.ops_bytes = p->tc_ops_bytes;
    err = tc_launch_of(p->equation, p->order, 1, a, p->tc_grid, s);
  } else if (is_tcm_variant(p->variant)) {
    const int k = p->variant - 4;
    a.ops = p->d_tcm_ops[k];
    a.ops_bytes = p->tcm_ops_bytes[k];
    err = tcm_launch_of(p->equation, p->order, tcm_mode(k) | 1, a, p->tcm_grid[k], s);
  } else {
    err = launch_of(p->equation, p->order, p->precision == DG_FP32_MIXED ? 1 : 0,
                    main_mode(p, dg::MODE_STAGE | (p->split ? dg::MODE_SPLIT : 0)), a,
                    main_grid(p), s);
  }
  if (err != cudaSuccess) return cuda_fail(err, "rk stage launch");
  return DG_OK;
}

}  // extern "C"

// Face-point scratch of dg_rhs_adjoint_noalloc, one per device that loads the
// library.  In host code this name is only a stand-in for the device array:
// its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double
    g_noalloc_scratch[DG_NOALLOC_SCRATCH_BYTES / sizeof(double)];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
// the scratch's device address per device, and the context it belongs to
double* g_noalloc_addr[kMaxDevices] = {};
void* g_noalloc_ctx[kMaxDevices] = {};

// The calling thread's current CUDA context (driver handle), or NULL.  The
// driver entry point is looked up through the runtime, so the library does
// not link libcuda directly.
void* current_context() {
  using CtxGetCurrent = int (*)(void**);
  static CtxGetCurrent fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<CtxGetCurrent>(f);
  }();
  void* ctx = nullptr;
  if (!fn || fn(&ctx) != 0) return nullptr;
  return ctx;
}

// Device address of the static scratch on `device` (which must be current).
// The address belongs to the context it was looked up in: a context that is
// destroyed and created again (cudaDeviceReset) loads the library's device
// code anew, possibly elsewhere, so the cache is keyed by the current
// context and looked up again when that changes.
int noalloc_scratch(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  void* ctx = current_context();
  if (!g_noalloc_addr[device] || !ctx || ctx != g_noalloc_ctx[device]) {
    void* ptr = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (err != cudaSuccess)
      return cuda_fail(err, "looking up the static adjoint scratch");
    g_noalloc_addr[device] = static_cast<double*>(ptr);
    g_noalloc_ctx[device] = current_context();  // current once the lookup ran
  }
  *out = g_noalloc_addr[device];
  return DG_OK;
}

}  // namespace

extern "C" {

int dg_rhs_adjoint_noalloc(dg_plan* p, const double* x, double* y,
                           void* stream) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!p->d_adj_ops || p->equation != DG_WAVE)
    return fail(DG_ERR_UNSUPPORTED,
                "adjoint needs an FP64 wave plan built with face_partner");
  if (!x || !y) return fail(DG_ERR_ARGUMENT, "x or y is NULL");
  const int64_t need = p->nel * 2 * 4 * (int64_t)p->nfp * 8;
  if (need > (int64_t)DG_NOALLOC_SCRATCH_BYTES)
    return fail(DG_ERR_ARGUMENT,
                "mesh too large for the static adjoint scratch: needs " +
                    std::to_string(need) + " bytes, the buffer holds " +
                    std::to_string(DG_NOALLOC_SCRATCH_BYTES));
  int dev = -1;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return cuda_fail(err, "cudaGetDevice");
  if (dev != p->device)
    return fail(DG_ERR_ARGUMENT, "the plan's device must be current");
  if (dev < 0 || dev >= kMaxDevices)
    return fail(DG_ERR_UNSUPPORTED, "device ordinal out of range");
  double* scratch = nullptr;
  const int code = noalloc_scratch(dev, &scratch);
  if (code != DG_OK) return code;
  return dg_rhs_adjoint(p, x, y, scratch, stream);
}

int dg_finish(dg_plan* p, void* stream) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return cuda_fail(err, "stream synchronize");
  int status = 0;
  err = cudaMemcpy(&status, p->d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (err != cudaSuccess) return cuda_fail(err, "status read");
  if (status != 0) {
    cudaMemset(p->d_status, 0, sizeof(int));
    return fail(status, status == DG_ERR_INDEX ? "a gather index was out of range"
                                               : "a device-side wait timed out");
  }
  return DG_OK;
}

int dg_plan_destroy(dg_plan* p) {
  if (!p) return DG_OK;
  int code = DG_OK;
  if (p->d_ops && cudaFree(p->d_ops) != cudaSuccess) code = DG_ERR_CUDA;
  if (p->d_status && cudaFree(p->d_status) != cudaSuccess) code = DG_ERR_CUDA;
  if (p->d_adj_ops && cudaFree(p->d_adj_ops) != cudaSuccess) code = DG_ERR_CUDA;
  for (void* b : {(void*)p->d_owned, (void*)p->d_flux, (void*)p->d_aux,
                  (void*)p->d_tc_ops, p->d_tcm_ops[0], p->d_tcm_ops[1],
                  p->d_tcm_ops[2] != p->d_tcm_ops[1] ? p->d_tcm_ops[2] : nullptr,
                  (void*)p->d_pres})
    if (b && cudaFree(b) != cudaSuccess) code = DG_ERR_CUDA;
  delete p;
  if (code != DG_OK) return fail(code, "cudaFree failed");
  return DG_OK;
}

int dg_stream_copy(void* dst, const void* src, int64_t bytes, int32_t ctas, void* stream) {
  if (!dst || !src || bytes < 0 || ctas < 1)
    return fail(DG_ERR_ARGUMENT, "bad stream copy arguments");
  if ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) |
       static_cast<uintptr_t>(bytes)) & 15u)
    return fail(DG_ERR_ARGUMENT, "stream copy needs 16-byte aligned addresses and sizes");
  if (overlap(dst, src, bytes)) return fail(DG_ERR_ARGUMENT, "source and destination overlap");
  // both addresses as the device sees them (page-locked host memory must be
  // mapped into the unified address space)
  const void* ptrs[2] = {src, dst};
  void* dev[2] = {nullptr, nullptr};
  for (int k = 0; k < 2; ++k) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, ptrs[k]) != cudaSuccess) {
      cudaGetLastError();
      return fail(DG_ERR_ARGUMENT, "stream copy: unknown pointer");
    }
    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) {
      dev[k] = const_cast<void*>(ptrs[k]);
    } else if (attr.type == cudaMemoryTypeHost && attr.devicePointer) {
      dev[k] = attr.devicePointer;
    } else {
      return fail(DG_ERR_ARGUMENT,
                  "stream copy: host memory must be page-locked and mapped");
    }
  }
  if (bytes == 0) return DG_OK;
  const int64_t n = bytes / 16;
  const int64_t need = (n + 255) / 256;
  const int grid = (int)(need < ctas ? (need > 0 ? need : 1) : ctas);
  stream_copy_kernel<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      static_cast<const uint4*>(dev[0]), static_cast<uint4*>(dev[1]), n);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return cuda_fail(err, "stream copy launch");
  return DG_OK;
}

int dg_wait_probe(int32_t* status, void* stream) {
  if (!status) return fail(DG_ERR_ARGUMENT, "status is NULL");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int* d = nullptr;
  cudaError_t err = cudaMalloc(&d, sizeof(int));
  if (err == cudaSuccess) err = cudaMemsetAsync(d, 0, sizeof(int), s);
  if (err == cudaSuccess) {
    wait_probe_kernel<<<1, 32, 0, s>>>(d);
    err = cudaGetLastError();
  }
  int h = 0;
  if (err == cudaSuccess) err = cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (d) cudaFree(d);
  if (err != cudaSuccess) return cuda_fail(err, "wait probe");
  *status = h;
  return DG_OK;
}

int dg_fp64_fma_probe(double* out, int64_t iters, int32_t grid, int32_t block,
                      void* stream) {
  if (!out || iters < 1 || iters > INT32_MAX || grid < 1 || block < 1 || block > 1024)
    return fail(DG_ERR_ARGUMENT, "bad probe arguments");
  fp64_fma_probe_kernel<<<grid, block, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      out, (int)iters);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return cuda_fail(err, "probe launch");
  return DG_OK;
}

int dg_plan_path(const dg_plan* p, int32_t* face_shared, int32_t* tensor_cores,
                 int32_t* launches_per_rhs, int64_t* owned_faces) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (face_shared) *face_shared = p->split ? 1 : 0;
  if (tensor_cores)
    *tensor_cores =
        (p->tc || p->variant >= 4 || ((p->variant & 1) && p->precision == DG_FP32_MIXED)) ? 1 : 0;
  if (launches_per_rhs)
    *launches_per_rhs = p->split ? (p->equation == DG_EULER ? 3 : 2) : (p->d_pres ? 2 : 1);
  if (owned_faces) *owned_faces = p->split ? p->nowned : 0;
  return DG_OK;
}

int dg_plan_info(const dg_plan* p, int64_t* nelements, int32_t* order,
                 int32_t* nfields, int32_t* grid, int32_t* block,
                 int32_t* smem_bytes) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (nelements) *nelements = p->nel;
  if (order) *order = p->order;
  if (nfields) *nfields = p->nfields;
  const bool m4 = !p->tc && is_tcm_variant(p->variant);
  const bool mb = !p->tc && is_shape_variant(p->variant);
  const int k = m4 ? p->variant - 4 : 0;
  const int kb = mb ? shape_index(p->variant) : 0;
  if (grid) *grid = p->tc ? p->tc_grid : (m4 ? p->tcm_grid[k] : main_grid(p));
  if (block)
    *block = p->tc ? p->tc_shape.threads
                   : (m4 ? p->tcm_shape[k].threads
                         : (mb ? p->tcb_shape[kb].threads : dg::kBlock));
  if (smem_bytes)
    *smem_bytes = p->tc ? p->tc_shape.smem_bytes
                        : (m4 ? p->tcm_shape[k].smem_bytes
                              : (mb ? p->tcb_shape[kb].smem_bytes : p->shape.smem_bytes));
  return DG_OK;
}

}  // extern "C"
