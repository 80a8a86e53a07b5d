/*
 * dgfem_gb300.h -- C ABI of the GB300 (sm_103a) DG-FEM right-hand-side evaluator.
 *
 * The suite evaluates an RHS as `compiled = actx.compile(rhs); out = compiled(*args)`
 * (actx_dgfem_suite/run/__main__.py:73-76).  This library is what sits behind
 * such a compiled callable: a plan built once per (equation, mesh, order) and
 * one call per RHS evaluation.  All device arrays are borrowed; the caller keeps
 * them alive for the plan's lifetime.  No function here allocates per RHS call.
 *
 * Data layouts (FP64, C order; Nel elements, Np = (N+1)(N+2)(N+3)/6 volume nodes,
 * Nfp = (N+1)(N+2)/2 nodes per face, 4 faces):
 *   state / rhs : (nfields, Nel, Np)   field-major, one meshmode DOFArray per field
 *                 wave:    u, v_x, v_y, v_z                    (nfields = 4)
 *                 euler:   mass, energy, momentum_x, _y, _z    (nfields = 5)
 *                 maxwell: E_x, E_y, E_z, H_x, H_y, H_z        (nfields = 6)
 *   metric      : (Nel, 3, 3)  dr_r/dx_x per element (affine simplices)
 *   face_geom   : (Nel, 4, 4)  outward normal n_x, n_y, n_z and sJ/J per face
 *   gather      : (Nel, 4, Nfp) uint32 flat index e'*Np + i' of the exterior
 *                 node of every face node; bit 31 set on boundary faces (the low
 *                 bits then name the element's own node)
 *
 * Return values: DG_OK (0) or one of the dg_status codes; dg_last_error()
 * returns a message for the calling thread's last failure.
 */
#ifndef DGFEM_GB300_H
#define DGFEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum dg_status {
  DG_OK = 0,
  DG_ERR_ARGUMENT = 1,     /* null pointer, bad size, bad enum value */
  DG_ERR_UNSUPPORTED = 2,  /* order or equation not compiled in */
  DG_ERR_CUDA = 3,         /* a CUDA runtime call failed */
  DG_ERR_TIMEOUT = 4,      /* a bounded device-side wait gave up */
  DG_ERR_INDEX = 5         /* a gather index was out of range (device-detected) */
};

enum dg_equation { DG_WAVE = 0, DG_EULER = 1, DG_MAXWELL = 2 };

/* Arithmetic of a plan.  DG_FP64: every operation in FP64 (the plain path).
 * DG_FP32_MIXED: derivative, flux and LIFT arithmetic in FP32 with FP32
 * operators and geometry, while the state stays FP64 in memory, the Euler
 * pressure is recovered from total energy in FP64, and RK stage updates
 * accumulate in FP64. */
/* DG_FP64: FP64 arithmetic throughout (contractions as FP64 FMAs).
 * DG_FP32_MIXED: FP32 derivative/flux/LIFT arithmetic, FP64 state, FP64
 *   Euler pressure recovery and FP64 RK accumulation.
 * DG_FP64_TC: FP64 state and results with the volume and LIFT contractions
 *   on the tcgen05 tensor cores as an exact FP64 emulation by FP16 digit
 *   slices (54-bit row/column scaling, exact FP32 level sums in tensor
 *   memory; error of the order of FP64's own accumulation error); orders 3
 *   and 4 on the face-shared path (see dg_plan_create), other plans fall
 *   back to DG_FP64 arithmetic. */
enum dg_precision { DG_FP64 = 0, DG_FP32_MIXED = 1, DG_FP64_TC = 2 };

typedef struct dg_plan dg_plan;

typedef struct dg_mesh_desc {
  int32_t order;             /* polynomial degree N, 1..4 */
  int64_t nelements;         /* Nel >= 1, Nel * Np < 2^31 */
  const double* metric;      /* device, (Nel, 3, 3) */
  const double* face_geom;   /* device, (Nel, 4, 4) */
  const uint32_t* gather;    /* device, (Nel, 4, Nfp) */
  const double* weak_diff;   /* host, (3, Np, Np): M^-1 S_r^T (wave, euler) */
  const double* strong_diff; /* host, (3, Np, Np): D_r (maxwell) */
  const double* lift;        /* host, (Np, 4, Nfp): M^-1 E */
  const int32_t* face_nodes; /* host, (4, Nfp): volume node of each face node */
  const int32_t* face_partner; /* device, (Nel, 4, Nfp): flat face-point index
                                  (e'*4 + f')*Nfp + j' of the glued face point,
                                  -1 on the boundary; optional.  FP64 plans use
                                  it for the face-shared path (see
                                  dg_plan_create); dg_rhs_adjoint needs it */
} dg_mesh_desc;

/* Build a plan: validate the description, stage the reference operators in
 * device memory (in the plan's precision) and size the persistent launch.
 * params: wave {c}; euler {gamma}; maxwell {alpha, epsilon, mu}.
 *
 * FP64 plans on meshes with face_partner (and Nel * 4 * Nfp < 2^31) take the
 * face-shared path: each glued pair of face points has its numerical flux
 * evaluated once (for Euler, pressure and wave speed once per node) by one
 * or two extra launches before the volume/LIFT kernel; face_partner must then
 * pair whole faces consistently with gather, which plan creation checks
 * (DG_ERR_ARGUMENT otherwise).  Such a plan keeps face values in its own
 * device buffers, so its dg_rhs / dg_rk_stage calls must not run
 * concurrently with each other (issue them on one stream).  All other plans
 * evaluate the RHS in one fused launch and have no such restriction.
 *
 * Replaces the compile step of the reference's array contexts:
 * actx.compile(rhs) (actx_dgfem_suite/run/__main__.py:74) and the DAG/loopy
 * pipeline behind it (actx_dgfem_suite/arraycontext/dgfem_optimizer.py:182-245). */
int dg_plan_create(dg_plan** plan, int32_t equation, int32_t precision,
                   const dg_mesh_desc* mesh, const double* params,
                   int32_t nparams);

/* Triangle meshes (the suite's dim = 2 runs).  Layouts (FP64, C order;
 * Np = (N+1)(N+2)/2 nodes, Nfp = N+1 nodes per edge, 3 edges):
 *   state / rhs : (nfields, Nel, Np)
 *                 wave:    u, v_x, v_y                         (nfields = 3)
 *                 euler:   mass, energy, momentum_x, _y        (nfields = 4)
 *                 maxwell: E_z, H_x, H_y (TM fields, grudge's
 *                          subset for dimensions = 2)          (nfields = 3)
 *   metric      : (Nel, 2, 2)  dr_r/dx_x per element
 *   face_geom   : (Nel, 3, 4)  n_x, n_y, sJ/J and a zero pad per edge
 *   gather      : (Nel, 3, Nfp) uint32, as in 3D (bit 31 = boundary) */
typedef struct dg_mesh2d_desc {
  int32_t order;             /* polynomial degree N, 1..4 */
  int64_t nelements;         /* Nel >= 1, Nel * Np < 2^31 */
  const double* metric;      /* device, (Nel, 2, 2) */
  const double* face_geom;   /* device, (Nel, 3, 4) */
  const uint32_t* gather;    /* device, (Nel, 3, Nfp) */
  const double* weak_diff;   /* host, (2, Np, Np): M^-1 S_r^T (wave, euler) */
  const double* strong_diff; /* host, (2, Np, Np): D_r (maxwell) */
  const double* lift;        /* host, (Np, 3, Nfp): M^-1 E */
  const int32_t* face_nodes; /* host, (3, Nfp): volume node of each edge node */
} dg_mesh2d_desc;

/* Build a plan for a triangle mesh: FP64 arithmetic, one fused persistent
 * launch per RHS (dg_rhs2d_kernel).  params as for dg_plan_create.  The plan
 * works with dg_rhs, dg_rk_stage, dg_plan_set_element_scale, dg_finish,
 * dg_plan_info, dg_plan_path and dg_plan_destroy; dg_plan_set_variant
 * accepts variant 0 only, and the adjoint entry points and autotuners return
 * DG_ERR_UNSUPPORTED.  Replaces actx.compile(rhs) for the builders' dim = 2
 * meshes (actx_dgfem_suite/equations/wave.py:248-285, euler.py:140-186,
 * maxwell.py:43-74). */
int dg_plan_create_2d(dg_plan** plan, int32_t equation,
                      const dg_mesh2d_desc* mesh, const double* params,
                      int32_t nparams);

/* One RHS evaluation: rhs = L(q), state and result FP64.  Enqueued on `stream` (a cudaStream_t,
 * NULL = legacy default stream); returns without synchronising.
 * q and rhs are device arrays of nfields * Nel * Np doubles and must not overlap.
 * Replaces the call of the compiled RHS, compiled_rhs(*args)
 * (actx_dgfem_suite/run/__main__.py:76,109,126). */
int dg_rhs(dg_plan* plan, const double* q, double* rhs, void* stream);

/* One stage of a low-storage Runge-Kutta method fused into the RHS kernel:
 *   res   = a * res + dt * L(q_in)      (res is not read when a == 0)
 *   q_out = q_in + b * res
 * All arrays are device (nfields, Nel, Np) FP64 and must not overlap; q_out
 * must differ from q_in because other elements still read q_in's face values
 * during the stage.  rhs_unscaled (optional, NULL to skip) receives L(q_in)
 * before the per-element scale (what an adjoint needs for the gradient with
 * respect to that scale).  The reference evaluates the RHS only; its RK hook
 * is estimate_rk4_timestep (actx_dgfem_suite/equations/wave.py:206-213). */
int dg_rk_stage(dg_plan* plan, const double* q_in, double* q_out, double* res,
                double a, double b, double dt, double* rhs_unscaled,
                void* stream);

/* Multiply the RHS of every element e by scale[e] in dg_rhs / dg_rk_stage /
 * dg_rhs_adjoint (a variable wave speed c_e for the wave operator, whose RHS
 * is linear in c).  scale: device array of Nel doubles kept alive by the
 * caller, or NULL to clear.  No counterpart in the reference (its wave speed
 * is a scalar, actx_dgfem_suite/equations/wave.py:279). */
int dg_plan_set_element_scale(dg_plan* plan, const double* scale);

/* Transpose of the plan's operator: y = L^T x (Euclidean inner product over
 * all DOFs), for FP64 wave plans built with mesh->face_partner.  The face
 * gather's transpose is computed as a gather over glued face points, so the
 * result is deterministic.  face_scratch: device buffer of Nel * 2 * 4 * Nfp
 * doubles.  x, y, face_scratch must not overlap.  No counterpart in the
 * reference (which has no adjoint); it is the building block of the
 * gradient of a misfit with respect to the initial state and wave speed. */
int dg_rhs_adjoint(dg_plan* plan, const double* x, double* y,
                   double* face_scratch, void* stream);

/* One stage of the reverse sweep of a low-storage Runge-Kutta step, fused
 * around the transpose (FP64 wave plans on the face-shared path).  For the
 * forward stage r^s = a_s r^{s-1} + dt L(q^(s)), q^(s+1) = q^(s) + b_s r^s
 * with L = c diag(c_e) L_1 (c_e from dg_plan_set_element_scale), and the
 * stage's residual adjoint rbar_s = xscale * x:
 *   lam      += dt L^T rbar_s                        (in place)
 *   rbar_out  = a * rbar_s + b * lam                 (skipped if NULL)
 *   cbar[e]  += dt <rbar_s, lq>_e   for every element (skipped if NULL)
 * where a = a_s, b = b_{s-1} (the next stage's b) and lq = c L_1 q^(s), the
 * forward stage's RHS before the element scale as dg_rk_stage wrote it to
 * rhs_unscaled, so that cbar accumulates the gradient with respect to c_e.  x may be lam itself (the
 * first reverse stage of a step, rbar = b_4 lam: xscale = b_4) and rbar_out
 * may be x itself; no other arrays may overlap.  y_scratch: device buffer of
 * nfields * Nel * Np doubles; the plan's face buffers are used too, so do
 * not run this concurrently with other calls on the plan.  Every sum has a
 * fixed order: the result is deterministic.  No counterpart in the
 * reference (which has no adjoint): it is the reverse step of the gradient
 * of a misfit with respect to the initial state and wave speed. */
int dg_rhs_adjoint_stage(dg_plan* plan, const double* x, double xscale, double* lam,
                         double* rbar_out, const double* lq, double* cbar,
                         double a, double b, double dt, double* y_scratch,
                         void* stream);

/* Transposed Jacobian of the plan's operator at state q: y = (dL/dq (q))^T x
 * (the vector-Jacobian product; for the linear wave operator, L^T x).
 * FP64 wave and Euler plans on the face-shared path (mesh with
 * face_partner).  Euler: transposed weak derivatives and LIFT, the flux
 * Jacobians J_x(q)^T at every node, the Lax-Friedrichs flux's Jacobians
 * (including the derivative of its wave-speed maximum, taken on the side
 * the forward picks) and the wall mirror, all computed deterministically
 * (gathers over glued face points, no atomics).  A per-element scale set
 * with dg_plan_set_element_scale is honoured.  Works in the plan's own
 * face buffers: do not run it concurrently with other calls on the plan.
 * No counterpart in the reference (which has no adjoint); it is the Euler
 * part of the adjoint RHS. */
int dg_rhs_vjp(dg_plan* plan, const double* q, const double* x, double* y,
               void* stream);

/* One reverse LSRK stage of a nonlinear operator, fused: for the forward
 * stage r^s = a_s r^{s-1} + dt L(q^(s)), q^(s+1) = q^(s) + b_s r^s and the
 * stage's residual adjoint rbar_s = xscale * x:
 *   lam      += dt (dL/dq (q^(s)))^T rbar_s          (in place)
 *   rbar_out  = a * rbar_s + b * lam                 (skipped if NULL)
 * with q = q^(s), the stage's input state, a = a_s and b = b_{s-1}.  The
 * launches of dg_rhs_vjp, whose last one (the node gather) applies the two
 * updates instead of storing the product, so that the stage reads and
 * writes each state-sized array once.  x may be lam itself (the first
 * reverse stage of a step: rbar_4 = b_4 lam, xscale = b_4) and rbar_out may
 * be x itself; q and y_scratch (nfields * Nel * Np doubles) may overlap
 * nothing that is written.  For a wave plan q is not read and the call is
 * dg_rhs_adjoint_stage without the element-scale gradient.  Uses the plan's
 * face buffers: do not run it concurrently with other calls on the plan.
 * No counterpart in the reference (which has no adjoint). */
int dg_rhs_vjp_stage(dg_plan* plan, const double* q, const double* x, double xscale,
                     double* lam, double* rbar_out, double a, double b, double dt,
                     double* y_scratch, void* stream);

/* Size of the device buffer that dg_rhs_adjoint_noalloc works in. */
#define DG_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)

/* dg_rhs_adjoint without a caller-supplied scratch buffer and without any
 * allocation.  It has no counterpart in the reference.
 *
 * Who needs it: callers that are not allowed to call cudaMalloc while they
 * run -- for example a host application that reserves the whole device
 * memory budget for its own pool at start-up and forbids allocations behind
 * its back, or code on a latency-critical path where cudaMalloc could
 * synchronise the device and stall work on other streams.
 *
 * How it works: the face-point scratch lives in one file-scope __device__
 * array of DG_NOALLOC_SCRATCH_BYTES (64 MiB) that every GPU loading this
 * library holds until the process exits.  The plan's mesh must fit:
 * Nel * 2 * 4 * Nfp * 8 bytes <= 64 MiB, i.e. at most 349,525 / 174,762 /
 * 104,857 / 69,905 elements at P1 / P2 / P3 / P4; larger meshes are
 * rejected with DG_ERR_ARGUMENT.  The plan's device must be current.
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * The address is cached for the CUDA context it was looked up in and looked
 * up again when the current context changes (a context destroyed by
 * cudaDeviceReset and created again holds the array elsewhere).
 * Memory: the 64 MiB are part of the library's device code, so they are
 * committed on a device when that code is loaded there -- with CUDA's
 * default lazy module loading at the latest by the first call of this
 * function (plan creation on a mesh with face_partner loads it too).  A
 * caller that reserves the rest of the device for its own pool should make
 * one call (any small wave plan will do) before taking that reservation,
 * or the first call may fail with DG_ERR_CUDA (out of memory).
 * Nothing in the array needs to start at zero: each call writes every entry
 * it later reads.  All calls share the one array, so calls that overlap on
 * the GPU (concurrent streams) race and must be serialised by the caller. */
int dg_rhs_adjoint_noalloc(dg_plan* plan, const double* x, double* y,
                           void* stream);

/* Block until `stream` has drained, then report any device-side error flag
 * the plan's kernels raised (DG_ERR_INDEX, DG_ERR_TIMEOUT) and clear it.
 * Replaces finish_command_queue(actx) (actx_dgfem_suite/measure.py:48-55). */
int dg_finish(dg_plan* plan, void* stream);

/* Box mesh built on the device: the 6 n[0] n[1] n[2] tetrahedra of the box
 * [a, b] (hexahedra in C order, six tetrahedra each), written straight into
 * the plan's input arrays.  Replaces the host-side mesh generation and
 * connectivity of the suite's builders (generate_regular_rect_mesh and
 * DiscretizationCollection, actx_dgfem_suite/equations/wave.py:250-270).
 * The small tables describe the hexahedron split and the reference element;
 * the host derives them once (see actx_dgfem_suite_gb300/device_setup.py). */
typedef struct dg_box_desc {
  int32_t order;                /* 1..4 */
  int64_t n[3];                 /* hexahedra per axis */
  double a[3], b[3];            /* box corners, b > a */
  const int32_t* corner;        /* host (6, 4, 3): corner offsets of each tet */
  const int32_t* nbr;           /* host (6, 4, 6): di, dj, dk, tet', face', perm */
  const int32_t* face_vert;     /* host (4, 3) */
  const int32_t* face_opp;      /* host (4) */
  const int32_t* face_nodes;    /* host (4, Nfp) */
  const int32_t* perm;          /* host (6, Nfp) */
  const double* bary;           /* host (Np, 4) */
  double* metric;               /* device out (Nel, 3, 3) */
  double* face_geom;            /* device out (Nel, 4, 4) */
  uint32_t* gather;             /* device out (Nel, 4, Nfp) */
  int32_t* face_partner;        /* device out (Nel, 4, Nfp), optional */
  double* nodes;                /* device out (3, Nel, Np), optional */
} dg_box_desc;

int dg_box_mesh_build(const dg_box_desc* desc, void* stream);

/* Number of launch variants (0 .. DG_NUM_VARIANTS - 1). */
#define DG_NUM_VARIANTS 11

/* Launch variant of the plan's main kernel: bit 0 = contractions on the
 * tensor cores (DG_FP32_MIXED plans: 3xTF32 split with FP32 accumulation,
 * i.e. FP32 accuracy, as warp-level mma.sync), bit 1 = one CTA per tile
 * instead of the persistent grid; 4 and 5 = the DG_FP32_MIXED kernel with
 * its volume and LIFT contractions as one tcgen05 product per 128-row tile
 * (persistent grid): 4 with rows scaled to 31-bit integers in four FP16
 * digits and the digit-pair products accumulated exactly in tensor memory
 * (the most accurate mixed variant), 5 with both operands split into TF32
 * pairs hi + lo and the products hi hi + hi lo + lo hi accumulated in FP32
 * (FP32 accuracy, far fewer instructions per tile); 6 = variant 5 with the
 * other CTA size for the same 128-row tile (128 threads at orders 2-3, so
 * that more tiles are in flight per SM, 256 at orders 1 and 4): the tile
 * shape the autotuner chooses along with the variant; 7-10 = variant 1's
 * mma.sync products at the two other tile shapes of that kernel, one
 * thread per (element, node) of the tile: 7 (persistent) and 8 (one CTA
 * per tile) with 128 threads and 128 / Np elements per tile, 9 and 10 with
 * 512 threads and 512 / Np elements (variants 1 and 3: 256 / Np).  A
 * variant the plan does not support (a precision it does not apply to, or
 * a tile that does not fit on an SM) is refused with DG_ERR_UNSUPPORTED.
 * Default 0.  No counterpart in the reference. */
int dg_plan_set_variant(dg_plan* plan, int32_t variant);

/* Time every variant the plan supports (after one warm-up launch, `reps`
 * launches of dg_rhs(q -> rhs) each, CUDA events on `stream`), keep the
 * fastest and report it in *chosen (may be NULL); ms_per_variant (may be
 * NULL) receives DG_NUM_VARIANTS floats, -1 for variants the plan does
 * not support and for variants whose launches raised a device-side status
 * (DG_ERR_TIMEOUT, DG_ERR_INDEX; read and cleared after each variant, and
 * such a variant is never chosen).
 * Writes rhs.  The autotuner of the batched (ensemble) path: the reference
 * fixes its loop-nest tiling in its loopy transforms instead
 * (actx_dgfem_suite/arraycontext/batched_einsum_loop_transforms.py:142). */
int dg_plan_autotune(dg_plan* plan, const double* q, double* rhs, int32_t reps,
                     void* stream, int32_t* chosen, float* ms_per_variant);

/* dg_plan_autotune under an accuracy bound: `ref` (device, the plan's state
 * shape) holds a trusted RHS of q, typically the DG_FP64 plan's; after its
 * timed launches each variant's result is compared with ref, and only
 * variants with ||rhs - ref|| / ||ref|| <= max_rel_l2 compete on time.  If
 * none meets the bound, the most accurate variant is kept.  err_per_variant
 * (may be NULL) receives DG_NUM_VARIANTS doubles, -1 where ms_per_variant
 * is -1.  The
 * reference checks every array context against its numpy context after the
 * first call (actx_dgfem_suite/run/__main__.py:87-96); this applies such a
 * tolerance to the choice of kernel. */
int dg_plan_autotune_bounded(dg_plan* plan, const double* q, double* rhs,
                             const double* ref, double max_rel_l2, int32_t reps,
                             void* stream, int32_t* chosen, float* ms_per_variant,
                             double* err_per_variant);

/* Release the plan's device buffers.  Replaces dropping the compiled program
 * and freeing the memory pool (actx_dgfem_suite/tools/wave_dof_scaling.py:108-126). */
int dg_plan_destroy(dg_plan* plan);

/* Which path the plan takes: face_shared 1 for the face-shared path, 0 for
 * the single fused launch; tensor_cores 1 when the contractions run on the
 * tensor cores (DG_FP64_TC on the face-shared path, or a DG_FP32_MIXED plan
 * under variant 1, 3 or 4); launches_per_rhs = kernel launches of one dg_rhs
 * or dg_rk_stage; owned_faces = faces whose flux the face kernel evaluates.
 * Any output pointer may be NULL. */
int dg_plan_path(const dg_plan* plan, int32_t* face_shared, int32_t* tensor_cores,
                 int32_t* launches_per_rhs, int64_t* owned_faces);

/* Describe a plan: any output pointer may be NULL.  grid/block/smem are the
 * persistent launch shape chosen at plan creation. */
int dg_plan_info(const dg_plan* plan, int64_t* nelements, int32_t* order,
                 int32_t* nfields, int32_t* grid, int32_t* block,
                 int32_t* smem_bytes);

/* Measurement helper (no counterpart in the reference, which hard-codes
 * datasheet peaks in actx_dgfem_suite/consts.py:1-12): runs `grid` x `block`
 * threads, each issuing 8 independent FP64 FMA chains of `iters` steps, and
 * writes one double per thread to `out` (device, grid*block doubles).
 * FP64 work = 16 * iters * grid * block flops; time it with events. */
int dg_fp64_fma_probe(double* out, int64_t iters, int32_t grid, int32_t block,
                      void* stream);

/* Copy `bytes` from src to dst with the SMs (a streaming kernel of at most
 * `ctas` CTAs on `stream`) instead of a copy engine.  Either side may be
 * page-locked, mapped host memory (cudaHostAlloc / pinned tensors), which
 * the kernel reads or writes over the CPU-GPU link; the array context uses
 * it to move host states and results.  Addresses and size must be 16-byte
 * aligned and the ranges must not overlap.  No counterpart in the reference
 * (its states live in the array context's device memory pool). */
int dg_stream_copy(void* dst, const void* src, int64_t bytes, int32_t ctas, void* stream);

/* Failure-detection check (no counterpart in the reference): one thread
 * waits on an mbarrier that nothing arrives at, through the same bounded
 * wait the kernels use (1 s), and reports through *status the code that
 * wait raises (DG_ERR_TIMEOUT), read back to the host after the launch.
 * The context stays usable.  Returns DG_OK when the launch and the read
 * succeeded. */
int dg_wait_probe(int32_t* status, void* stream);

/* Thread-local message for the last failing call, "" if none. */
const char* dg_last_error(void);

/* ABI version, bumped on any incompatible change (3: dg_plan_autotune
 * writes 5 floats to ms_per_variant, variant 4 added; 4: variants that
 * raise a device-side status report -1, dg_plan_autotune_bounded and
 * dg_rhs_adjoint_stage added; 5: dg_rhs_vjp_stage and variants 5 and 6
 * added, the autotuners write DG_NUM_VARIANTS = 7 entries; 6: the tile-shape
 * variants 7-10, DG_NUM_VARIANTS = 11; 7: dg_plan_create_2d). */
int32_t dg_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DGFEM_GB300_H */
