/*
 * quijibo_gpu.h -- C ABI of the GB300 implementation of QUIJIBO's hot path.
 *
 * The reference exposes this path as C++ class methods; each entry point
 * below names the reference interface it replaces (paths inside the QUIJIBO
 * project).  All entry points return QJG_OK (0) or a negative QJG_ERR_* code
 * and never exit the process; qjg_last_error() describes the last failure on
 * a context.  Device pointers are plain CUDA device addresses; `stream` is a
 * cudaStream_t (NULL = the legacy default stream).  A context serves one host
 * thread at a time: its scratch buffers are shared by its calls.
 */
#ifndef QUIJIBO_GPU_H
#define QUIJIBO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QJG_OK 0
#define QJG_ERR_ARG (-1)      /* invalid argument (sizes, handles, null pointers) */
#define QJG_ERR_CUDA (-2)     /* a CUDA call failed */
#define QJG_ERR_NOMEM (-3)    /* device memory could not be allocated */
#define QJG_ERR_HANDLE (-4)   /* unknown or freed root set */
#define QJG_ERR_CAPACITY (-5) /* an output buffer is too small; the counts say how much is needed */

#define QJG_MAX_ROOTS 128 /* top + bottom roots of one root set */

/* Precision forms of the field. */
#define QJG_FP64 0        /* plain form: FP64 with the reference's QUATERNION::pow per root term */
#define QJG_FP32 1        /* FP32 only */
#define QJG_FP32_REFINE 2 /* FP32 bulk, FP64 re-evaluation of the band |d| < band_h * h */

/* How FP64 re-evaluation raises roots to powers. */
#define QJG_FORM_QUOTIENT 0
#define QJG_FORM_LAGRANGE 1
#define QJG_REFINE_POW 0 /* the reference's polar QUATERNION::pow (reference rounding) */
#define QJG_REFINE_INT 1 /* repeated products when every exponent is an integer */

/* Transcendentals of the reference's QUATERNION::pow in the FP64 forms. */
#define QJG_LIBM_DEVICE 0 /* the CUDA device library's acos/log/exp/sin/cos */
#define QJG_LIBM_CR 1     /* correctly rounded acos/log/exp/sin/cos (slower): the values a C
                             library with correctly rounded functions gives */

typedef struct qjg_ctx qjg_ctx;
typedef int32_t qjg_rootset;

/* Cell-centred grid = FIELD_3D geometry (src/geometry/FIELD_3D.h:55-120):
 * res, center, lengths (spacing lengths/res), rotation quaternion (w,x,y,z)
 * about center, and the 4D slice coordinate of every start point. */
typedef struct {
  int32_t res[3];
  double center[3];
  double lengths[3];
  double rot[4];
  double slice;
} qjg_grid;

/* Escape-time iteration settings. */
typedef struct {
  int32_t max_it;    /* OPTIMIZE_3D::_maxIterations */
  int32_t precision; /* QJG_FP64 / QJG_FP32 / QJG_FP32_REFINE */
  int32_t refine_pow;/* QJG_REFINE_POW / QJG_REFINE_INT */
  int32_t want_de;   /* also produce the distance estimate |q| log|q| / |q'| */
  double escape;     /* escape radius (the reference uses 2000) */
  double band_h;     /* refine band half-width in voxel spacings (2.0 = |d| < 2h) */
  double field_tol;  /* voxels with |log|q|| < field_tol are refined too */
  double rel_tol;    /* QJG_FP32_REFINE: target relative field error (e.g. 1e-6); voxels whose
                        tracked FP32 error exceeds it are re-run with a double-float head and,
                        if still above it, in FP64.  0 = the band rule alone. */
  int32_t form;      /* QJG_FORM_QUOTIENT: T(q) / B(q) (computeLogScaledPowerRationalMap);
                        QJG_FORM_LAGRANGE: RATIONAL_4D::evaluateLagrange order, top and bottom
                        factors interleaved (RATIONAL_4D.cpp:27-73), in every precision form */
  int32_t libm;      /* QJG_LIBM_DEVICE / QJG_LIBM_CR: the transcendentals of every FP64
                        QUATERNION::pow (plain FP64 form, FP64 refine with QJG_REFINE_POW,
                        the meshers' FP64 evaluations) and the final log|q_N| of those
                        evaluations */
} qjg_iter;

typedef struct {
  int64_t voxels;        /* voxels computed */
  int64_t voxel_iters;   /* executed map applications (bulk pass) */
  int64_t root_terms;    /* voxel_iters x (n_top + n_bottom) */
  int64_t refined;       /* voxels re-evaluated in FP64 */
  int64_t refined_iters; /* map applications of the FP64 re-evaluation */
  int64_t nonfinite;     /* FP32 voxels that overflowed or underflowed */
  int64_t lane_iters;    /* FP32 bulk: lane slots spent (32 x the longest orbit of each warp) */
  int64_t rerun;         /* voxels re-run with a double-float head (rel_tol) */
  int64_t rerun_iters;   /* map applications of those re-runs */
} qjg_field_stats;

/* ---- context and root sets ------------------------------------------- */

/* A context's calls take their device scratch from the context's own
 * stream-ordered memory pool, which keeps freed memory for later calls
 * (re-mapping it at every call cost 0.4 ms of a 2 ms energy + gradient
 * call); qjg_trim returns the kept memory to the device, qjg_destroy all
 * of it.  The server's worker contexts return it after every request. */
int qjg_create(int device, qjg_ctx** out);
void qjg_destroy(qjg_ctx* ctx);
int qjg_trim(qjg_ctx* ctx);
const char* qjg_last_error(qjg_ctx* ctx);

/* Upload a rational map and keep it resident.  Replaces building the
 * OPTIMIZE_3D top/bottom POLYNOMIAL_4D state (src/algebra/POLYNOMIAL_4D.cpp:40-60,
 * POLYNOMIAL_4D.h:137-150) plus _expScaling.  roots are n x (w,x,y,z);
 * effective exponents are sigma * powers[i]; n_top >= 1; n_bot may be 0. */
int qjg_rootset_upload(qjg_ctx* ctx, int32_t n_top, const double* top_roots,
                       const double* top_powers, double sigma_top, int32_t n_bot,
                       const double* bot_roots, const double* bot_powers, double sigma_bot,
                       double scale, qjg_rootset* out);
int qjg_rootset_free(qjg_ctx* ctx, qjg_rootset rs);

/* ---- field ------------------------------------------------------------ */

/* Escape-time field log|q_N| of slices [z0, z1) into device memory:
 * d_field[(z - z0) * X * Y + y * X + x]; d_de (optional, may be NULL) gets
 * the distance estimate.  Replaces OPTIMIZE_3D::computeLogScaledPowerRationalMap
 * (src/solvers/OPTIMIZE_3D.cpp:1272-1370, declared OPTIMIZE_3D.h:167) and
 * TRIANGLE_MESH::computeNonlinearSlice (src/geometry/TRIANGLE_MESH.cpp:330-381). */
int qjg_field(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
              int32_t z0, int32_t z1, double* d_field, float* d_de, void* stream);

/* The same with host buffers: host_field receives the full X*Y*Z field
 * (the FIELD_3D data array), host_de (optional) the distance estimate.
 * Inputs and outputs cross PCIe/NVLink-C2C inside the call. */
int qjg_field_host(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
                   double* host_field, float* host_de, qjg_field_stats* stats);

/* Counters of the last qjg_field call on ctx; synchronizes `stream`. */
int qjg_field_stats_read(qjg_ctx* ctx, void* stream, qjg_field_stats* out);

/* The field, for callers that cannot allocate device memory: plugins whose
 * host application owns every device allocation (its own pool, nothing left
 * for a library to cudaMalloc), real-time loops that must not reach the
 * allocator, processes held to a fixed device-memory quota.  No counterpart
 * in the reference.  The map comes as host arrays
 * (as in qjg_rootset_upload), the output is a device buffer as in qjg_field;
 * no context is needed and nothing is allocated: the counters, the FP64
 * refine list and the double-float re-run list live in a fixed scratch array
 * inside the library (about 32 MiB, held on every device that loads the
 * library until the process exits).  The field has the bits of qjg_field's
 * for the same inputs, rel_tol included.  One call covers at most QJG_NOALLOC_MAX_VOXELS voxels (X*Y*(z1-z0));
 * larger slab ranges return QJG_ERR_CAPACITY before anything is launched.
 * The first call on a device looks up the scratch array's device address
 * (with that device current), so make that first call before any stream
 * capture.  Every call shares the scratch array:
 * calls whose work overlaps on the GPU (different streams or host threads)
 * race on it and must be serialised by the caller. */
#define QJG_NOALLOC_MAX_VOXELS (1 << 22)
int qjg_field_noalloc(int32_t n_top, const double* top_roots, const double* top_powers,
                      double sigma_top, int32_t n_bot, const double* bot_roots,
                      const double* bot_powers, double sigma_bot, double scale,
                      const qjg_grid* grid, const qjg_iter* iter, int32_t z0, int32_t z1,
                      double* d_field, float* d_de, void* stream);

/* ---- marching cubes ---------------------------------------------------- */

/* Edge-vertex placement. */
#define QJG_EDGE_LINEAR 0 /* p0 + d0/(d0-d1) (p1-p0) from stored values */
#define QJG_EDGE_BISECT 1 /* bisection of the map, <= 6 levels, FP64 */

typedef struct {
  int64_t n_verts;       /* vertices (written, or needed when a capacity is short) */
  int64_t n_tris;        /* triangles after the degenerate filter (or needed before it) */
  int64_t n_degenerate;  /* triangles dropped by the degenerate filter (edge < 1e-7) */
  int64_t n_unbracketed; /* edges whose end values do not bracket zero (the reference exits) */
  int64_t map_evals;     /* FP64 map evaluations of the edge bisection */
  int64_t map_evals_fp32;/* FP32 evaluations whose sign was trusted (precision form only) */
  int64_t map_evals_ff;  /* double-float evaluations that decided a point FP32 could not
                            (precision form, integer exponents) */
  int64_t slabs;         /* z-slabs processed */
  qjg_field_stats field; /* the field pass of qjg_mesh_stream */
  /* with qjg_set_timing on (else 0): device milliseconds of each phase, summed over slabs */
  double ms_field;       /* slab fields (qjg_mesh_stream) */
  double ms_classify;    /* cube flags, edge masks, vertex ids */
  double ms_vertices;    /* vertex placement (interpolation or bisection) */
  double ms_triangles;   /* triangle emission */
  double ms_filter;      /* degenerate-triangle filter and output conversion */
  double ms_field_bulk;  /* qjg_mesh_stream: the FP32 bulk kernel's part of ms_field */
} qjg_mesh_stats;

/* Marching cubes on a stored device field (X*Y*Z doubles).  Corners are
 * inside when the stored value is > 0.  edge_mode QJG_EDGE_LINEAR replaces
 * TRIANGLE_MESH(const FIELD_3D&) / computeStagedMarchingCubes
 * (src/geometry/TRIANGLE_MESH.cpp:48-57, 989-1114); QJG_EDGE_BISECT replaces
 * TRIANGLE_MESH(field, top, bottom, expScaling, maxIterations, slice, iso)
 * / computeNonlinearMarchingCubes (TRIANGLE_MESH.cpp:62-76, 152-275), whose
 * bisection evaluates the map (rs, iter: max_it, escape, refine_pow) minus iso.
 * Outputs in device memory: vertices as 3 doubles (d_verts64) and/or 3
 * floats (d_verts32), triangles as 3 int32 vertex indices; vertex order and
 * triangle order are the reference's.  slab_nz cube layers per pass (<= 0: 64).
 * Returns QJG_ERR_CAPACITY, with the needed counts in *stats, when vert_cap
 * or tri_cap is too small.  Synchronizes `stream`. */
int qjg_mesh_field(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
                   const double* d_field, int32_t edge_mode, double iso, int32_t slab_nz,
                   double* d_verts64, float* d_verts32, int64_t vert_cap, int32_t* d_tris,
                   int64_t tri_cap, qjg_mesh_stats* stats, void* stream);

/* Streaming marching cubes: the field (iter->precision) is computed slab by
 * slab, corners are classified by log|q| > 0, and vertices are placed by
 * bisection of log|q| - iso: in FP64 for QJG_FP64; for the precision form
 * each evaluation is tried in FP32 first and kept only when its value clears
 * its error bound, so every bisection decision is the one FP64 makes.  Replaces the two-slab streaming
 * TRIANGLE_MESH(center, lengths, res, top, bottom, expScaling, maxIterations,
 * slice, isosurface, rotation, cacheFile) constructor /
 * computeNonlinearMarchingCubesLowMemoryHuge (TRIANGLE_MESH.cpp:84-101,
 * 681-768).  Outputs and capacities as qjg_mesh_field. */
int qjg_mesh_stream(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
                    double iso, int32_t slab_nz, double* d_verts64, float* d_verts32,
                    int64_t vert_cap, int32_t* d_tris, int64_t tri_cap, qjg_mesh_stats* stats,
                    void* stream);

/* qjg_mesh_stream as a fixed launch sequence: every count stays in device
 * memory, so no host read, host wait or allocation sits between its kernels
 * and a caller may capture the call into a CUDA graph (same vertices and
 * triangles as qjg_mesh_stream).  qjg_mesh_prepare sizes the context for
 * meshes up to the grid's X, Y, the slab depth and the capacities (device
 * allocations: call it before a capture); qjg_mesh_stream_async enqueues one
 * mesh on `stream` and returns (vert_cap and tri_cap > 0, at most the
 * prepared ones; d_tris also holds the unfiltered triangles);
 * qjg_mesh_async_result reads its stats once the stream (or graph) has run.
 * A mesh that outgrows a capacity stops writing and reads back as
 * QJG_ERR_CAPACITY without the counts it needs (qjg_mesh_stream reports
 * them).  No edge-cache capture or phase timing on this path.  A captured
 * graph holds the context's buffers: a later call on the context that grows
 * them (qjg_mesh_prepare with larger sizes, qjg_mesh_stream or qjg_field on
 * more voxels) leaves the graph pointing at freed memory, so capture again
 * after such a call. */
int qjg_mesh_prepare(qjg_ctx* ctx, const qjg_grid* grid, int32_t slab_nz, int64_t vert_cap,
                     int64_t tri_cap);
int qjg_mesh_stream_async(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid,
                          const qjg_iter* iter, double iso, int32_t slab_nz, double* d_verts64,
                          float* d_verts32, int64_t vert_cap, int32_t* d_tris, int64_t tri_cap,
                          void* stream);
int qjg_mesh_async_result(qjg_ctx* ctx, qjg_mesh_stats* stats);

/* Edge-cache bookkeeping of the meshers.  With capture on, qjg_mesh_stream
 * and qjg_mesh_field keep, per call, the edge of every vertex (its two grid
 * corners, in vertex order) and every cube whose corners are neither all
 * inside nor all outside (flag and corner index, in scan order): the two
 * lists of the reference's edge cache.  qjg_mesh_edge_cache_write writes the
 * last captured call in the reference's cache-file format, byte for byte
 * (TRIANGLE_MESH::writeEdgeCacheHuge, src/geometry/TRIANGLE_MESH.cpp:535-586,
 * the file computeNonlinearMarchingCubesLowMemoryHuge (:681-768) leaves at
 * the streaming constructor's cacheFilename): int count, 6 ints per edge;
 * int count, 4 ints (flag, x, y, z) per cube.  qjg_mesh_edge_cache_read reads
 * such a file (TRIANGLE_MESH::readEdgeCacheHuge, :431-482) into caller
 * arrays (NULL arrays: counts only).  Capture costs one device-to-host copy
 * of the vertices' edges and the cubes per slab. */
int qjg_mesh_capture(qjg_ctx* ctx, int32_t on);
int qjg_mesh_edge_cache_write(qjg_ctx* ctx, const char* path);
int qjg_mesh_edge_cache_read(const char* path, int32_t* edges, int64_t edge_cap, int64_t* n_edges,
                             int32_t* cubes, int64_t cube_cap, int64_t* n_cubes);

/* ---- fitting energy and gradients ------------------------------------- */

typedef struct {
  int64_t voxels;
  int64_t overflowed;  /* voxels whose map overflowed; the reference recomputes them
                          in long double, here their gradient terms are left out */
  int64_t bad_terms;   /* NaN/inf gradient terms left out (the reference's _nans/_infs) */
  int64_t band_voxels; /* voxels whose per-parameter terms were computed; the others' are exact
                          zeros (saturated tanh or zero weight) */
} qjg_tanh_stats;

/* Tanh-weighted fitting score of the map on a grid and its analytic
 * one-application gradients, in one pass.  Replaces OPTIMIZE_3D::computeScoreAP
 * (src/solvers/OPTIMIZE_3D.cpp:3563-3569: computeRationalMapAP + weightScore),
 * computeExpGradientAP (:3589-3625), computeBottomGradientAP (:10012-10218),
 * computeTopGradientAP (:8905-9106) and compute{Top,Bottom}BulkScalarGradientAP
 * (:9250-9478, :10360-10602).  grad (host, 3 + n_bottom + n_top entries) has
 * the layout of toothOptimizer's FormScaledFunctionGradient
 * (projects/toothOptimizer/toothOptimizer.cpp:65-109): [d/d log s,
 * d/d bottom exponents, d/d top exponents, d/d sigma_top, d/d sigma_bottom].
 * The weight field (d_weights, device, FIELD_3D layout on weight_grid) is
 * looked up trilinearly at cell centres; alpha/threshold are _tanhAlpha and
 * _tanhThreshold (10, 0 in the reference).  max_it as _maxIterations (the
 * gradient is exact for max_it = 1, as toothOptimizer runs it).  d_field
 * (optional, device) receives the map's log|q|.  Synchronizes `stream`. */
int qjg_tanh_score_grad(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, int32_t max_it,
                        const qjg_grid* weight_grid, const double* d_weights, double alpha,
                        double threshold, double* score, double* grad, double* d_field,
                        qjg_tanh_stats* stats, void* stream);

/* Squared-error fitting energy E = sum_k (D tanh(d(x_k)/D) - t_k)^2 of the
 * distance estimate d = |q_N| log|q_N| / |q_N'| at sample points x_k, with
 * D = d_sat (d_sat <= 0: E = sum (d - t)^2; samples deep inside, where
 * |q_N'| contracts to zero and d grows without bound, saturate at +-D and
 * add no gradient once |d| > 20 D) (no reference
 * counterpart: the reference fits exponents and scales with the tanh score;
 * this form also fits root positions).  The map's parameters live in a
 * device vector d_params of 5 * (n_top + n_bot) + 1 doubles:
 * [top roots (w,x,y,z) x n_top | bottom roots x n_bot | top exponents |
 *  bottom exponents | log s] (effective exponents, sigma folded in).
 * d_xyz: n x 3 device doubles; d_target: n device doubles; slice is the
 * fourth coordinate; precision QJG_FP32 or QJG_FP64.  max_it <= 256.
 * qjg_energy_forward writes E to *energy (host); qjg_energy_backward also
 * writes dE/dparams into d_grad (device, same layout), computed by a
 * hand-written adjoint that runs back over the orbit points the forward pass
 * kept (one quaternion per sample and iteration in the call's device
 * scratch: n x max_it x 16 bytes in FP32, 32 in FP64).  d_iters (optional, device) receives
 * each sample's iteration count.  Both synchronize `stream`. */
int qjg_energy_forward(qjg_ctx* ctx, const double* d_params, int32_t n_top, int32_t n_bot,
                       int64_t n, const double* d_xyz, const double* d_target, double slice,
                       int32_t max_it, double escape, double d_sat, int32_t precision,
                       double* energy, int32_t* d_iters, void* stream);
int qjg_energy_backward(qjg_ctx* ctx, const double* d_params, int32_t n_top, int32_t n_bot,
                        int64_t n, const double* d_xyz, const double* d_target, double slice,
                        int32_t max_it, double escape, double d_sat, int32_t precision,
                        double* energy, double* d_grad, void* stream);

/* Several squared-error energy + gradient calls in one pass (FP32 only; no
 * reference counterpart: the serving form's batches).  Each item is the
 * argument set of a qjg_energy_backward call; the items' samples are
 * iterated by one persistent forward kernel and their gradient samples by
 * one persistent adjoint kernel, and each item's energy and gradient are
 * summed in a fixed order (the same values on every run, within FP32
 * rounding of the item's own qjg_energy_backward).  Writes each item's
 * energy and d_grad; synchronizes `stream`. */
typedef struct {
  const double* d_params; /* 5 (n_top + n_bot) + 1 doubles, layout of qjg_energy_backward */
  int32_t n_top, n_bot;
  int64_t n;              /* samples */
  const double* d_xyz;    /* n x 3 */
  const double* d_target; /* n */
  double slice;
  int32_t max_it;
  int32_t pad_;
  double escape, d_sat;
  double* d_grad;         /* device output */
  double energy;          /* output */
} qjg_energy_item;
int qjg_energy_backward_batch(qjg_ctx* ctx, int32_t n_items, qjg_energy_item* items, void* stream);

typedef struct {
  int32_t steps;          /* L-BFGS iterations taken */
  int32_t energy_evals;   /* forward evaluations (line search) */
  int32_t gradient_evals; /* forward + adjoint evaluations */
  double energy0;         /* energy at the start */
  double energy;          /* energy at the end */
} qjg_fit_stats;

/* Fit the map's parameters (d_params, layout of qjg_energy_backward, updated
 * in place on the device) to the sample targets with `steps` iterations of
 * L-BFGS (history `history` pairs, Armijo backtracking).  The parameters,
 * gradients and history stay on the device; only scalar energies reach the
 * host.  Replaces the role of toothOptimizer's TAO_SOLVER::optimizeBLMVM
 * loop (src/TOUPEE/TAO_SOLVER.h:41-43) for this energy; no bounds.
 * energies (optional, host, steps + 1 doubles) receives the energy after
 * each step.  Synchronizes `stream`. */
int qjg_fit_lbfgs(qjg_ctx* ctx, double* d_params, int32_t n_top, int32_t n_bot, int64_t n,
                  const double* d_xyz, const double* d_target, double slice, int32_t max_it,
                  double escape, double d_sat, int32_t precision, int32_t steps, int32_t history,
                  double* energies, qjg_fit_stats* stats, void* stream);

/* ---- serving ----------------------------------------------------------- */

/* A continuous-batching request server (no reference counterpart: the
 * reference runs one driver per job).  Requests are admitted as soon as a
 * worker slot is free and their device-memory estimate fits the HBM budget;
 * admitted requests run concurrently on their own streams, so work submitted
 * while others run overlaps with them.  Field requests in the precision form
 * with integer exponents and at most 2^26 voxels are served by a batch
 * worker instead: every such request waiting when it becomes free (up to 64
 * and the batch arena) runs in one multi-request pass, replayed from a
 * captured CUDA graph.  Mesh requests of the same form with at most 2^22
 * voxels take their field from that pass as well; a worker then meshes that
 * field (qjg_mesh_field with the map's bisection: the vertices and triangles
 * qjg_mesh_stream gives them).  FP32 energy + gradient requests go to an energy
 * batch worker, which runs every such request waiting when it is free as
 * one qjg_energy_backward_batch pass.  Inputs are copied at submission; output buffers
 * (host) must stay valid until the request completes. */
#define QJG_REQ_FIELD 0  /* field of a map on a grid (out_field: X*Y*Z doubles, optional) */
#define QJG_REQ_MESH 1   /* streaming field + marching cubes (out_verts / out_tris optional) */
#define QJG_REQ_ENERGY 2 /* squared-error energy + gradient (params/xyz/target; out_grad) */

#define QJG_STATUS_QUEUED 0
#define QJG_STATUS_RUNNING 1
#define QJG_STATUS_DONE 2
#define QJG_STATUS_FAILED 3

typedef struct qjg_server qjg_server;

typedef struct {
  int32_t kind;      /* QJG_REQ_* */
  int32_t precision; /* field/mesh: QJG_FP64 or QJG_FP32_REFINE; energy: QJG_FP32 or QJG_FP64 */
  int32_t n_top, n_bot;
  const double* top_roots; /* field / mesh: the map as in qjg_rootset_upload */
  const double* top_powers;
  const double* bot_roots;
  const double* bot_powers;
  double sigma_top, sigma_bot, scale;
  qjg_grid grid;    /* field / mesh; energy uses grid.slice only */
  int32_t max_it;
  double escape;
  double iso;       /* mesh */
  int64_t vert_cap, tri_cap; /* mesh output capacities */
  const double* params; /* energy: parameter vector (layout of qjg_energy_backward) */
  double d_sat;         /* energy: saturation distance D (as qjg_energy_backward) */
  int64_t n_samples;
  const double* xyz;
  const double* target;
  double* out_field;  /* host outputs, optional */
  double* out_verts;
  int32_t* out_tris;
  double* out_grad;
  double rel_tol;     /* field / mesh in QJG_FP32_REFINE: as qjg_iter.rel_tol (0: band rule) */
} qjg_request;

typedef struct {
  int32_t status; /* QJG_STATUS_* */
  int32_t error;  /* QJG_OK or the failing entry point's code */
  double latency_ms, queue_ms, run_ms;
  double t_admit_ms, t_done_ms; /* since the server was created */
  int64_t voxel_iters, refined;
  int64_t n_verts, n_tris;
  double energy;
} qjg_result;

typedef struct {
  int64_t completed, failed;
  double p50_ms, p99_ms, max_ms; /* submission-to-completion latency of completed requests */
  double span_s;                 /* first submission to last completion */
  int64_t in_use_bytes;          /* device-memory estimate of the running requests */
  int64_t peak_in_use_bytes;
  int32_t peak_running;          /* most requests running at once */
  int32_t pad_;
  int64_t batched;               /* field (and mesh) requests served inside multi-request batches */
  int64_t batches;               /* batch passes (one CUDA-graph replay each) */
  int64_t max_batch;             /* most requests in one batch */
  int64_t energy_batched;        /* FP32 energy requests served inside energy batches */
  int64_t energy_batches;        /* energy batch passes */
  int64_t max_energy_batch;      /* most requests in one energy batch */
  int64_t mesh_batched;          /* mesh requests among `batched` (field from the batch pass) */
} qjg_server_stats;

int qjg_server_create(int device, int32_t workers, int64_t hbm_budget_bytes, qjg_server** out);
void qjg_server_destroy(qjg_server* srv); /* drains first */
int qjg_server_submit(qjg_server* srv, const qjg_request* req, int64_t* ticket);
int qjg_server_poll(qjg_server* srv, int64_t ticket, qjg_result* out);
/* waits for the ticket, returns its result and forgets it */
int qjg_server_wait(qjg_server* srv, int64_t ticket, qjg_result* out);
int qjg_server_drain(qjg_server* srv);
int qjg_server_read_stats(qjg_server* srv, qjg_server_stats* out);

/* ---- finite-difference root gradients ---------------------------------- */

/* Central differences, step eps = lengths[0] / res[0], of OPTIMIZE_3D's
 * binary-score objectives with respect to every root component (entry
 * 4 k + c for root k, component c of (w, x, y, z)); every moved map is
 * evaluated in one pass, FP64 in the reference's operation order, so the
 * scores and gradients are the reference's.  The map takes the root set's
 * roots and scale s (_expScaling); exponents and power scalars are unused.
 * d_dist (and d_curv) are X*Y*Z device doubles on `grid` (the reference's
 * _distanceField and _curvatureField share the fractal's grid).  grad is a
 * host array; *score (optional) receives the unmoved map's score. */
#define QJG_FD_LOG_RATIONAL 0        /* computeLogRationalCenteredGradient
                                        (src/solvers/OPTIMIZE_3D.cpp:2872-2951): binary score
                                        (:2275-2297) of computeLogRationalMap (:1907-1985);
                                        4 (nt + nb) entries, top roots first */
#define QJG_FD_LOG_RATIONAL_BOTTOM 1 /* computeLogRationalBottomCenteredGradient (:2956-3008):
                                        the same, bottom roots only; 4 nb entries */
#define QJG_FD_POLYNOMIAL 2          /* computeCenteredGradient (:2761-2812): (binary + curvature
                                        score (:2497-2537)) / 2 of computeMap (:853-980), the
                                        top polynomial alone; 4 nt entries; needs d_curv */
int qjg_centered_gradient(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, int32_t max_it,
                          int32_t kind, const double* d_dist, const double* d_curv, double* grad,
                          double* score, void* stream);

/* ---- optimizer set-up passes ------------------------------------------ */

/* The weight field of a signed distance field (X*Y*Z doubles, device):
 * 1 / (breadth-first layer from the sign-change shells), negated inside and
 * quartered outside; with `normalized`, scaled to sum |w| = 1 and 0.5 per
 * side.  Replaces FIELD_3D::invertedDistance / invertedDistanceNormalized
 * (src/geometry/FIELD_3D.cpp:5241-5352).  QJG_ERR_ARG when the field has no
 * sign change that reaches every cell (the reference loops forever). */
int qjg_inverted_distance(qjg_ctx* ctx, const int32_t res[3], const double* d_dist,
                          int32_t normalized, double* d_out, void* stream);
/* The conformal-radius scan: the one-application field log|T/B| of `rs` with
 * the roots' own exponents (no power scalar), s = 1, escape 20 on `grid`;
 * scores sum -tanh(alpha (F - x)) W over four passes of ~100 thresholds x,
 * W = the inverted distance of d_dist (on dist_grid) at the cell centres.
 * Returns the lowest score, its threshold and exp(-threshold), the scale the
 * optimizer starts from.  Replaces OPTIMIZE_3D::estimateConformalRadius
 * (src/solvers/OPTIMIZE_3D.cpp:4693-4772; alpha is _tanhAlpha = 10). */
int qjg_conformal_radius(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid,
                         const qjg_grid* dist_grid, const double* d_dist, double alpha,
                         double* min_score, double* threshold, double* exp_scaling, void* stream);

/* ---- optimizer ---------------------------------------------------------- */

/* Objective of qjg_blmvm: *f = f(x) and g = its gradient (n entries).  A
 * non-zero return stops the solver, which returns that value. */
typedef int (*qjg_objective_fn)(void* user, int32_t n, const double* x, double* f, double* g);
/* Called after every iteration; a non-zero return ends the run
 * (reason QJG_BLMVM_CONVERGED_USER). */
typedef int (*qjg_monitor_fn)(void* user, int32_t iter, double f, double gnorm, const double* x);

/* Solver settings; qjg_blmvm_defaults gives TAO_SOLVER's defaults with the
 * tolerances toothOptimizer sets (src/TOUPEE/TAO_SOLVER.cpp:40-63,
 * projects/toothOptimizer/toothOptimizer.cpp:150-160). */
typedef struct {
  int32_t max_it;       /* iterations (2000) */
  int32_t ls_max_funcs; /* trial points per line search (30) */
  double fatol;         /* stop when |g|^2 <= fatol (1e-8) */
  double frtol;         /* ... |g|^2 / |f| <= frtol (1e-8) */
  double gatol;         /* ... |g| <= gatol (1e-8) */
  double grtol;         /* ... |g / f| <= grtol (1e-8) */
  double gttol;         /* ... |g| / |g_0| <= gttol (0) */
} qjg_blmvm_settings;

/* Why the solver stopped: TAO's SOLVER_STATE codes (TAO_SOLVER.h:62-81). */
#define QJG_BLMVM_CONVERGED_FATOL 1
#define QJG_BLMVM_CONVERGED_FRTOL 2
#define QJG_BLMVM_CONVERGED_GATOL 3
#define QJG_BLMVM_CONVERGED_GRTOL 4
#define QJG_BLMVM_CONVERGED_GTTOL 5
#define QJG_BLMVM_CONVERGED_MINF 7
#define QJG_BLMVM_CONVERGED_USER 8
#define QJG_BLMVM_DIVERGED_MAXITS (-2)
#define QJG_BLMVM_DIVERGED_NAN (-4)
#define QJG_BLMVM_DIVERGED_LS_FAILURE (-6)

typedef struct {
  int32_t reason;      /* QJG_BLMVM_* */
  int32_t iterations;
  int32_t evaluations; /* objective calls */
  int32_t grad_steps;  /* quasi-Newton directions that were not descent (scaled gradient used) */
  int32_t resets;      /* failed line searches retried along the scaled gradient */
  int32_t pad_;
  double f;            /* objective at the returned x */
  double gnorm;        /* norm of the bound-projected gradient there */
} qjg_blmvm_stats;

void qjg_blmvm_defaults(qjg_blmvm_settings* out);

/* Minimise fg over lower <= x <= upper from x (the result is written back):
 * BLMVM with the Moré-Thuente line search, as QUIJIBO's TAO port runs it.
 * Replaces TAO_SOLVER::optimizeBLMVM (src/TOUPEE/TAO_SOLVER.h:41-43,
 * TAO_SOLVER.cpp:72-341).  Host only: the objective may launch GPU work.
 * settings NULL = qjg_blmvm_defaults.  Returns QJG_OK, QJG_ERR_ARG, or the
 * objective's non-zero status. */
int qjg_blmvm(int32_t n, double* x, const double* lower, const double* upper, qjg_objective_fn fg,
              void* fg_user, qjg_monitor_fn monitor, void* monitor_user,
              const qjg_blmvm_settings* settings, qjg_blmvm_stats* stats);

/* The optimizer's map: OPTIMIZE_3D's top/bottom POLYNOMIAL_4D and
 * _expScaling.  The roots stay fixed; fits update the exponents, the power
 * scalars and the scale in place. */
typedef struct {
  int32_t n_top;
  int32_t n_bot;
  const double* top_roots; /* n_top x (w,x,y,z) */
  const double* bot_roots; /* n_bot x (w,x,y,z) */
  double* top_powers;      /* n_top */
  double* bot_powers;      /* n_bot */
  double sigma_top;        /* powerScalar() */
  double sigma_bot;
  double scale;            /* expScaling() */
} qjg_map_state;

#define QJG_FIT_SCALED_ONLY 0 /* variables [log s, sigma_top, sigma_bot] */
#define QJG_FIT_SCALED 1      /* [log s, bottom exponents, top exponents, sigma_top, sigma_bot] */

/* One BLMVM solve of the tanh score of qjg_tanh_score_grad on `grid`
 * (max_it map applications, weights on weight_grid): every objective
 * evaluation is one GPU pass over the grid.  Bounds as the reference's: log s
 * free, every other variable >= 0.  Replaces callConstrainedScaledOnlyTao /
 * callConstrainedScaledTao with FormScaledOnlyFunctionGradient /
 * FormScaledFunctionGradient (projects/toothOptimizer/toothOptimizer.cpp:
 * 65-229).  The monitor (optional) sees the solver's variables after each
 * iteration; d_field (optional, device) receives the field of the last
 * evaluation, as OPTIMIZE_3D::_fractal holds it.  settings NULL = defaults. */
int qjg_tanh_fit(qjg_ctx* ctx, int32_t mode, qjg_map_state* state, const qjg_grid* grid,
                 int32_t max_it, const qjg_grid* weight_grid, const double* d_weights, double alpha,
                 double threshold, const qjg_blmvm_settings* settings, qjg_monitor_fn monitor,
                 void* monitor_user, double* d_field, qjg_blmvm_stats* stats, void* stream);

/* sum |w| over the cell centres of grid, the weights looked up trilinearly:
 * OPTIMIZE_3D::computeMaximumScaledPowerRationalScore
 * (src/solvers/OPTIMIZE_3D.cpp:4484-4497). */
int qjg_tanh_max_score(qjg_ctx* ctx, const qjg_grid* grid, const qjg_grid* weight_grid,
                       const double* d_weights, double* out, void* stream);

/* buildReweightedInsideField's arithmetic (projects/toothOptimizer/
 * toothOptimizer.cpp:302-381) on device fields of n cells: md = the target's
 * signed distance, fd = the fitted shape's, w = the weights.  Target-inside
 * cells (md < 0) the shape misses (fd > 0) share 0.25 of the weight, those it
 * covers (fd < 0) another 0.25, each region scaled uniformly; every other
 * cell gets 0.5 / (number of cells with md > 0).  *poor_sum / *well_sum (may
 * be NULL) get the two regions' weight sums before scaling. */
int qjg_reweight_inside(qjg_ctx* ctx, int64_t n, const double* d_md, const double* d_fd,
                        const double* d_w, double* d_out, double* poor_sum, double* well_sum,
                        void* stream);

/* Signed distance (negative inside), on `grid`, of a closed triangle mesh
 * given in host buffers: what toothOptimizer obtains from its external sdfGen
 * program (toothOptimizer.cpp:285-300).  Returns 0 on success. */
typedef int (*qjg_sdf_fn)(void* user, const double* verts, int64_t n_verts, const int32_t* tris,
                          int64_t n_tris, const qjg_grid* grid, double* out);

/* toothOptimizer's run (projects/toothOptimizer/toothOptimizer.cpp:462-530):
 * read the state file, take the weights from the normalized inverted distance
 * of its distance field, move a unit-cube problem to the fractal's frame
 * (translate all but the first root by -1/2, scale by fractal_radius, when
 * the field is smaller than 0.95 fractal_radius), multiply every exponent but
 * the first of each polynomial by amp, set both power scalars to 1, then
 * optimizeSpecificResolution (:385-457) per level: the conformal-radius scan
 * (first level only), the scaled-only solve, the scaled solve, the reweighted
 * solve (when `sdf` is given: the level's field, infinities clamped to the
 * mean and borders set as computeFractal does, meshed by linear marching
 * cubes and handed to sdf), the unweighted solve, and <output_prefix>_res_<res>.o3d.
 * Every solve is qjg_tanh_fit on the level's grid at maxIterations 1. */
typedef struct {
  const char* input_path;      /* the .o3d state to start from */
  const char* checkpoint_path; /* state written every 10th solver iteration of the run (the
                                  monitor's output.o3d, toothOptimizer.cpp:48-61); NULL: none */
  const char* output_prefix;   /* NULL: no per-level state files */
  double fractal_radius;       /* "fractal radius" (4) */
  double amp;                  /* "initial bulk scalar amplitude" (-1) */
  int32_t n_levels;            /* entries of levels[] (the reference: 3) */
  int32_t levels[8];           /* grid resolution per level (25, 50, 97) */
  int32_t pad_;
  qjg_sdf_fn sdf;              /* NULL: the reweighted solve is skipped */
  void* sdf_user;
  const qjg_blmvm_settings* settings; /* NULL: qjg_blmvm_defaults */
} qjg_tooth_config;

typedef struct {
  int32_t res;
  int32_t reweighted;       /* 1 when the reweighted solve ran */
  int64_t mesh_tris;        /* triangles handed to sdf */
  double conformal_score;   /* the scan's lowest score (first level; else 0) */
  double initial_score;     /* the tanh score at the level's start */
  double max_score;         /* computeMaximumScaledPowerRationalScore, original weights */
  double final_score;       /* the tanh score after the last solve */
  double poor_sum, well_sum;/* buildReweightedInsideField's region sums */
  qjg_blmvm_stats solve[4]; /* scaled-only, scaled, reweighted, unweighted */
  double ms;                /* wall time of the level */
  int32_t checkpoints;      /* state files written by the monitor during the level */
  int32_t pad_;
} qjg_tooth_level;

/* Runs cfg->n_levels levels; levels_out gets one entry per level.  Each
 * level's map (roots in the fractal frame) is in its state file. */
int qjg_tooth_optimize(qjg_ctx* ctx, const qjg_tooth_config* cfg, qjg_tooth_level* levels_out,
                       void* stream);

/* ---- file formats ------------------------------------------------------ */

/* FIELD_3D's binary stream: int xRes, yRes, zRes; double center[3], lengths[3];
 * double data[X*Y*Z] (x fastest).  Replaces FIELD_3D::write(string) / write(FILE*)
 * (src/geometry/FIELD_3D.cpp:280-300, 4371-4393).  `field` is host or device memory. */
int qjg_field3d_write(const char* path, const int32_t res[3], const double center[3],
                      const double lengths[3], const double* field);
/* The header of such a file, and its data into `field` (host or device, at
 * least X*Y*Z doubles, else QJG_ERR_CAPACITY).  Replace FIELD_3D::read(FILE*)
 * (FIELD_3D.cpp:4398-4450). */
int qjg_field3d_read_header(const char* path, int32_t res[3], double center[3],
                            double lengths[3]);
int qjg_field3d_read(const char* path, double* field, int64_t capacity);
/* TRIANGLE_MESH's raw stream (int V, int T, V x 3 doubles, T x 3 ints), the
 * format TRIANGLE_MESH::read(FILE*) loads.  Replaces TRIANGLE_MESH::write(FILE*)
 * (src/geometry/TRIANGLE_MESH.cpp:4502-4522).  Buffers host or device. */
int qjg_mesh_write_raw(const char* path, const double* verts, int64_t n_verts,
                       const int32_t* tris, int64_t n_tris);
/* OBJ text as TRIANGLE_MESH::writeOBJ prints it ("v %.16f %.16f %.16f", then
 * "f %i %i %i" 1-based; TRIANGLE_MESH.cpp:2762-2800), from FP64 or FP32
 * vertices (exactly one of verts64 / verts32), host or device buffers. */
int qjg_mesh_write_obj(const char* path, const double* verts64, const float* verts32,
                       int64_t n_verts, const int32_t* tris, int64_t n_tris);

/* The optimizer state file (.o3d): OPTIMIZE_3D::write / read
 * (src/solvers/OPTIMIZE_3D.cpp:3253-3360).  Roots are n x (w,x,y,z); the
 * fields are the fractal, distance and curvature FIELD_3D streams, in that
 * order.  The writer stores empty coefficient lists (the power-factored
 * path never reads them; OPTIMIZE_3D::read accepts them). */
typedef struct {
  int32_t res[3];
  double center[3], lengths[3];
  int32_t n_top, n_bot;
  double sigma_top, sigma_bot; /* the polynomials' power scalars */
  double exp_scaling;
  int32_t history;             /* length of the (unwritten) optimizer history */
  int32_t field_res[3][3];
  double field_center[3][3], field_lengths[3][3];
} qjg_o3d_info;
int qjg_o3d_read_info(const char* path, qjg_o3d_info* info);
/* Host buffers sized from the info; any may be NULL to skip it. */
int qjg_o3d_read(const char* path, double* top_roots, double* top_powers, double* bot_roots,
                 double* bot_powers, double* fractal, double* distance, double* curvature);
int qjg_o3d_write(const char* path, const qjg_o3d_info* info, const double* top_roots,
                  const double* top_powers, const double* bot_roots, const double* bot_powers,
                  const double* fractal, const double* distance, const double* curvature);

#ifdef __cplusplus
}
#endif
#endif
