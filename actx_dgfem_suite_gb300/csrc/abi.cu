// C ABI of the DG-FEM RHS evaluator (declared in include/dgfem_gb300.h).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dgfem_gb300.h"
#include "dg_launch.h"
#include "dg_rhs_fp64.cuh"  // RhsArgs, kBlock

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t err, const char* what) {
  return fail(DG_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(err));
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

__global__ void fp64_fma_probe_kernel(double* out, int64_t iters) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-9 * (double)(tid + k);
  const double b = 0.9999999, c = 1e-7;
  for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[tid] = s;
}

}  // namespace

struct dg_plan {
  int32_t equation = 0;
  int32_t order = 0;
  int32_t np = 0, nfp = 0, nfields = 0;
  int64_t nel = 0;
  const double* metric = nullptr;
  const double* face_geom = nullptr;
  const uint32_t* gather = nullptr;
  double* d_ops = nullptr;
  uint32_t ops_bytes = 0;
  int* d_status = nullptr;
  double params[3] = {0, 0, 0};
  int grid = 0;
  dg::LaunchShape shape;
  int device = 0;
};

extern "C" {

const char* dg_last_error(void) { return g_last_error.c_str(); }

int32_t dg_abi_version(void) { return 1; }

int dg_plan_create(dg_plan** plan_out, int32_t equation,
                   const dg_mesh_desc* mesh, const double* params,
                   int32_t nparams) {
  g_last_error.clear();
  if (!plan_out) return fail(DG_ERR_ARGUMENT, "plan output pointer is NULL");
  *plan_out = nullptr;
  if (!mesh) return fail(DG_ERR_ARGUMENT, "mesh description is NULL");
  const int nf = nfields_of(equation);
  if (nf == 0) return fail(DG_ERR_ARGUMENT, "unknown equation");
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
    return fail(DG_ERR_ARGUMENT,
                equation == DG_MAXWELL ? "strong_diff is NULL"
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

  dg::LaunchShape shape;
  cudaError_t err = cudaErrorInvalidValue;
  switch (equation) {
    case DG_WAVE: err = dg::fp64_shape_wave(N, &shape); break;
    case DG_EULER: err = dg::fp64_shape_euler(N, &shape); break;
    case DG_MAXWELL: err = dg::fp64_shape_maxwell(N, &shape); break;
  }
  if (err != cudaSuccess) return cuda_fail(err, "kernel configuration");
  if (shape.blocks_per_sm < 1)
    return fail(DG_ERR_UNSUPPORTED, "kernel does not fit on an SM");
  const dg::OpsOffsets off = dg::ops_offsets(np, nfp);
  if (off.size != shape.ops_doubles)
    return fail(DG_ERR_CUDA, "operator layout mismatch between host and kernel");

  // pack [Wt | Lt | face_nodes]
  std::vector<double> ops(off.size, 0.0);
  for (int r = 0; r < 3; ++r)
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j)
        ops[off.w + (r * np + j) * np + i] = diff[(r * np + i) * np + j];
  for (int i = 0; i < np; ++i)
    for (int fj = 0; fj < 4 * nfp; ++fj)
      ops[off.l + fj * np + i] = mesh->lift[i * 4 * nfp + fj];
  int32_t* fn = reinterpret_cast<int32_t*>(ops.data() + off.fn);
  for (int k = 0; k < 4 * nfp; ++k) fn[k] = mesh->face_nodes[k];

  dg_plan* p = new dg_plan;
  p->equation = equation;
  p->order = N;
  p->np = np;
  p->nfp = nfp;
  p->nfields = nf;
  p->nel = mesh->nelements;
  p->metric = mesh->metric;
  p->face_geom = mesh->face_geom;
  p->gather = mesh->gather;
  p->shape = shape;
  p->ops_bytes = static_cast<uint32_t>(off.size * sizeof(double));
  for (int k = 0; k < nparams; ++k) p->params[k] = params[k];
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
  const int64_t ntiles =
      (p->nel + shape.elems_per_tile - 1) / shape.elems_per_tile;
  const int64_t full = (int64_t)nsm * shape.blocks_per_sm;
  p->grid = (int)(ntiles < full ? ntiles : full);
  *plan_out = p;
  return DG_OK;
}

int dg_rhs(dg_plan* p, const double* q, double* rhs, void* stream) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (!q || !rhs) return fail(DG_ERR_ARGUMENT, "state or rhs pointer is NULL");
  const int64_t n = (int64_t)p->nfields * p->nel * p->np;
  const char* qb = reinterpret_cast<const char*>(q);
  const char* rb = reinterpret_cast<const char*>(rhs);
  if (qb < rb + n * 8 && rb < qb + n * 8)
    return fail(DG_ERR_ARGUMENT, "state and rhs overlap");
  dg::RhsArgs a;
  a.q = q;
  a.rhs = rhs;
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
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t err = cudaErrorInvalidValue;
  switch (p->equation) {
    case DG_WAVE: err = dg::fp64_launch_wave(p->order, a, p->grid, s); break;
    case DG_EULER: err = dg::fp64_launch_euler(p->order, a, p->grid, s); break;
    case DG_MAXWELL: err = dg::fp64_launch_maxwell(p->order, a, p->grid, s); break;
  }
  if (err != cudaSuccess) return cuda_fail(err, "rhs launch");
  return DG_OK;
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
    return fail(status, status == DG_ERR_INDEX
                            ? "a gather index was out of range"
                            : "a device-side wait timed out");
  }
  return DG_OK;
}

int dg_plan_destroy(dg_plan* p) {
  if (!p) return DG_OK;
  int code = DG_OK;
  if (p->d_ops && cudaFree(p->d_ops) != cudaSuccess) code = DG_ERR_CUDA;
  if (p->d_status && cudaFree(p->d_status) != cudaSuccess) code = DG_ERR_CUDA;
  delete p;
  if (code != DG_OK) return fail(code, "cudaFree failed");
  return DG_OK;
}

int dg_fp64_fma_probe(double* out, int64_t iters, int32_t grid, int32_t block,
                      void* stream) {
  if (!out || iters < 1 || grid < 1 || block < 1 || block > 1024)
    return fail(DG_ERR_ARGUMENT, "bad probe arguments");
  fp64_fma_probe_kernel<<<grid, block, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      out, iters);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return cuda_fail(err, "probe launch");
  return DG_OK;
}

int dg_plan_info(const dg_plan* p, int64_t* nelements, int32_t* order,
                 int32_t* nfields, int32_t* grid, int32_t* block,
                 int32_t* smem_bytes) {
  if (!p) return fail(DG_ERR_ARGUMENT, "plan is NULL");
  if (nelements) *nelements = p->nel;
  if (order) *order = p->order;
  if (nfields) *nfields = p->nfields;
  if (grid) *grid = p->grid;
  if (block) *block = dg::kBlock;
  if (smem_bytes) *smem_bytes = p->shape.smem_bytes;
  return DG_OK;
}

}  // extern "C"
