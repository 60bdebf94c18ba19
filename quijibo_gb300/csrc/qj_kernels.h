// Host-side launchers of the CUDA kernels (implemented in the .cu files).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qj_params.h"

namespace qj {

// field.cu
cudaError_t launch_field64(const MapParams& m, const GridParams& g, const IterParams& it,
                           bool pow_ref, double* field, float* de, DevStats* st, cudaStream_t s);
cudaError_t launch_field32(const MapParams& m, const GridParams& g, const IterParams& it,
                           bool refine, double* field, float* de, uint32_t* list, DevStats* st,
                           cudaStream_t s);
cudaError_t launch_refine64(const MapParams& m, const GridParams& g, const IterParams& it,
                            bool pow_ref, const uint32_t* list, double* field, float* de,
                            DevStats* st, cudaStream_t s);

}  // namespace qj
