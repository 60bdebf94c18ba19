/*
 * quijibo_gpu_bench.h -- measurement hooks of the GB300 library.  These have
 * no counterpart in the reference: they expose per-kernel CUDA-event timings
 * and launch counts so that a benchmark can attribute time to kernels, and an
 * FP32 FMA-throughput probe used as the roofline denominator of the field
 * kernel.
 */
#ifndef QUIJIBO_GPU_BENCH_H
#define QUIJIBO_GPU_BENCH_H

#include <stdint.h>

#include "quijibo_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Record CUDA events around each kernel a context launches (off by default). */
int qjg_set_timing(qjg_ctx* ctx, int on);

/* Milliseconds of the bulk and FP64-refine kernels of the last field call
 * (synchronizes with it); a kernel that did not run reports 0. */
int qjg_last_timings(qjg_ctx* ctx, float* ms_bulk, float* ms_refine);

/* Kernels this context has launched since it was created. */
int64_t qjg_launch_count(qjg_ctx* ctx);

/* Process-wide choice of the FP32 bulk field kernel, for A/B timing and the
 * bit-equality test of the two forms: 1 (the default) two voxels per lane on
 * the packed f32x2 instructions, 0 one voxel per lane.  Both give the same
 * bits.  Set it while no field call is in flight. */
int qjg_set_field32_pairs(int on);

/* Process-wide choice of the squared-error energy's forward kernel, for A/B
 * timing: 1 two samples per lane sharing one walk over the roots, 0 (the
 * default) one sample per lane.  Set it while no energy call is in flight. */
int qjg_set_energy_pairs(int on);

/* Process-wide form of the FP32 adjoint of qjg_energy_backward and of
 * qjg_energy_backward_batch, for A/B timing: 1 (the default) each gradient
 * sample taken by a group of 16 lanes, every lane owning a run of at most 4
 * roots of each side (the products over the roots as scans over the lanes),
 * for maps of at most 64 top and 64 bottom roots (larger maps keep the
 * one-lane form); 0 one lane per sample walking the roots in series.  The
 * two agree to FP32 rounding (the products and sums run in different
 * orders).  Set it while no energy call is in flight. */
int qjg_set_energy_adjoint_roots(int on);

/* Process-wide form of the FP32 energy's arithmetic: 1 (the default) the
 * fast form (the PTX approximations of log2, exp2, sin/cos, the reciprocal
 * for every division and the reciprocal square root, denormals flushed, and
 * a polynomial atan: about 1e-6 relative per power), 0 the accurate device
 * library functions and IEEE divisions.  Set it while no energy call is in
 * flight. */
int qjg_set_energy_fast(int on);

/* Process-wide block count of the energy forward kernel, for sweeps: 0 (the
 * default) the sizing rule (at least 3 blocks of 128 lanes per SM, more when
 * each lane would otherwise take more than about four samples), else that
 * many blocks per SM, capped by residency.  With the one-sample kernel (the
 * default) results do not depend on it (each sample's value is its own; sums
 * run in sample order).  Set it while no energy call is in flight; a
 * negative count returns QJG_ERR_ARG. */
int qjg_set_energy_forward_blocks(int per_sm);

/* Work of the last qjg_energy_forward/backward call on ctx: the map
 * applications of its forward pass (orbit steps of every sample) and the
 * orbit steps its adjoint ran back over (gradient samples only; 0 for a
 * forward call): the units of the energy kernels' algorithmic FLOP counts. */
int qjg_energy_last_work(qjg_ctx* ctx, int64_t* applications, int64_t* steps);

/* The correctly rounded FP64 transcendentals of the QJG_LIBM_CR form, element
 * by element on the device: y[i] = f(x[i]) for n device doubles on `stream`
 * (for bit-for-bit comparison with the same functions built for the host). */
#define QJG_CRM_EXP 0
#define QJG_CRM_LOG 1
#define QJG_CRM_SIN 2
#define QJG_CRM_COS 3
#define QJG_CRM_ACOS 4
int qjg_crmath_eval(int fn, const double* d_x, double* d_y, int64_t n, void* stream);

/* FP32 FMA-pipe probe: runs a kernel of independent FMA chains on every SM
 * of `device` and returns the achieved FP32 TFLOP/s (2 flops per FMA). */
int qjg_fma_probe(int device, double* tflops);

#ifdef __cplusplus
}
#endif
#endif
