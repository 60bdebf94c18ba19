// Host-side launchers of the energy kernels (energy.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "qj_params.h"

namespace qj {

// A FIELD_3D weight grid for trilinear lookups (FIELD_3D.cpp:966-1029):
// corner = center - lengths/2 + dx/2, inv = 1/dx.

int tanh_blocks();
// out[] of launch_tanh_grad: [d log s, d bottom exps, d top exps, d sigma_t,
// d sigma_b, score, overflowed voxels, non-finite terms left out, scratch,
// voxels with per-parameter terms]
int tanh_slots(int nt, int nb);
cudaError_t launch_tanh_grad(const MapParams& m, const GridParams& g, const WeightGrid& wg,
                             const double* weights, int max_it, double alpha, double thr,
                             bool pow_ref, double* field, double* partials, int nblocks,
                             double* out, cudaStream_t s);

int sq_max_iterations();
// Device scratch of one energy call (forward, or forward + gradient).
size_t sq_scratch_bytes(bool fp64, bool grad, long long n, int max_it, int nt, int nb);
// *out (in the scratch): [energy, gradient (5 (nt + nb) + 1), samples left
// out of the gradient]; *launches: kernels launched.
// process-wide choice of the energy forward kernel: 1 two samples per lane
void set_energy_pairs(int on);
// process-wide choice of the FP32 adjoint: 1 (default) the roots of a step
// spread over a group of lanes where the map fits, 0 one lane per sample
void set_energy_adjoint_roots(int on);
// FP32/FP64 forward blocks per SM (0: the sizing rule).
void set_energy_forward_blocks(int per_sm);
// the FP32 polar power's fast form (hardware log2 and sin/cos, polynomial atan)
cudaError_t set_energy_fast(int on);
// *work: two counters in the scratch, the map applications of the forward
// pass and the orbit steps of the adjoint (read after the call completes).
// steps_hint: the forward map applications of an earlier call on the same
// samples (0 if none), which sizes the FP32 forward grid.
cudaError_t launch_sq_energy(bool fp64, bool grad, const double* params, int nt, int nb,
                             const double* xyz, const double* target, long long n, double slice,
                             int max_it, double escape, double d_sat, void* scratch,
                             double** out, int* iters, cudaStream_t s, int* launches,
                             unsigned long long** work, long long steps_hint);

// One request of a batch of FP32 energy + gradient calls: device pointers
// as for launch_sq_energy.
struct SqBatchReq {
  const double* params;
  int nt, nb;
  long long n;
  const double* xyz;
  const double* target;
  double slice;
  int max_it;
  double escape, d_sat;
};
size_t sq_batch_scratch_bytes(const SqBatchReq* r, int K);
// The K requests in one pass (FP32 forward and adjoint); outs[i] (in the
// scratch) receives request i's [energy, gradient, samples left out], as
// launch_sq_energy's out.
cudaError_t launch_sq_energy_batch(const SqBatchReq* r, int K, void* scratch, double** outs,
                                   cudaStream_t s, int* launches);

}  // namespace qj
