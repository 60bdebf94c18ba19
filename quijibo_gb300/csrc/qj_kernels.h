// Host-side launchers of the CUDA kernels (implemented in the .cu files).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qj_params.h"

namespace qj {

// field.cu
cudaError_t launch_field64(const MapParams& m, const GridParams& g, const IterParams& it,
                           bool pow_ref, double* field, float* de, DevStats* st, cudaStream_t s);
// FP32 bulk pass; with refine, appends the voxels to re-evaluate in FP64 to
// `list` (with each one's FP32 orbit length in `keys` when not null) and,
// when `ff_list` is not null, it.est_tol > 0 and the exponents are integers,
// the voxels for the double-float re-run to `ff_list`.
cudaError_t launch_field32(const MapParams& m, const GridParams& g, const IterParams& it,
                           bool refine, double* field, float* de, uint32_t* list, uint8_t* keys,
                           uint32_t* ff_list, DevStats* st, cudaStream_t s);
// Double-float re-run of `ff_list`; appends what still needs FP64 to `list`.
cudaError_t launch_rerun_ff(const MapParams& m, const GridParams& g, const IterParams& it,
                            const uint32_t* ff_list, double* field, float* de, uint32_t* list,
                            uint8_t* keys, DevStats* st, cudaStream_t s);
// process-wide choice of the FP32 bulk kernel: 1 two voxels per lane
// (field32x2_kernel, the default), 0 one voxel per lane (field32_kernel)
void set_field32_pairs(int on);
// FP64 re-evaluation of the listed voxels.  With `keys`, the list is first
// counting-sorted by key into `sorted` (capacity of the list; `hist` holds
// REFINE_KEYS counters) so that each warp gets orbits of one length.
constexpr int REFINE_KEYS = 256;
cudaError_t launch_refine64(const MapParams& m, const GridParams& g, const IterParams& it,
                            bool pow_ref, const uint32_t* list, const uint8_t* keys,
                            uint32_t* sorted, unsigned* hist, double* field, float* de,
                            DevStats* st, cudaStream_t s);

}  // namespace qj
