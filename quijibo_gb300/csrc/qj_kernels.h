// Host-side launchers of the CUDA kernels (implemented in the .cu files).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qj_params.h"

namespace qj {

// Lists a bulk pass fills (device pointers; keys and ff may be null).
struct RefineLists {
  uint32_t* list;  // voxels for the FP64 re-evaluation (length in DevStats::refined)
  uint8_t* keys;   // their FP32 orbit lengths, the sort key of the FP64 pass
  uint32_t* ff;    // voxels for the double-float re-run (length in DevStats::rerun)
};

// A batch of field requests run as one pass (field.cu, batch kernels).
constexpr int BATCH_MAX = 64;                    // items per batch
constexpr int BATCH_SHIFT = 26;                  // list entry = item << 26 | local voxel
constexpr uint32_t BATCH_MASK = (1u << BATCH_SHIFT) - 1u;
constexpr long long BATCH_ITEM_VOXELS = 1ll << BATCH_SHIFT;  // largest item

struct BatchItem {
  GridParams g;      // the item's grid, z-range [0, Z)
  IterParams it;
  double* field;     // device output, X*Y*Z doubles
  float* de;         // optional
  long long tile0;   // first tile of the item in the batch's tile queue
  int refine;        // FP32 bulk + re-run/FP64 passes (else FP32 only)
  int pad_;
};

struct BatchTable {
  int n;
  int pad_;
  long long total_tiles;
  BatchItem items[BATCH_MAX];
};

struct BatchCounts {
  unsigned long long voxel_iters;  // bulk map applications of the item
};

// Device buffers of a batch pass; entries of `rl` and `sorted` hold up to
// the batch's total voxels.
struct BatchBuffers {
  const BatchTable* tab;
  const MapParams* maps;
  RefineLists rl;
  uint32_t* sorted;
  unsigned* hist;
  BatchCounts* counts;
  DevStats* st;
};

// Launch shapes of the batch kernels on the current device (computed once,
// outside any stream capture).
struct BatchShapes {
  int bulk, rerun, sort, refine;
};
BatchShapes batch_shapes();
// Tiles of one item (the unit of the batch's work queue).
long long batch_item_tiles(int X, int Y, int Z);
// The whole batch pass: fixed launch shapes and no host synchronisation, so
// the sequence can be captured into a CUDA graph once and replayed for every
// batch with a new table in the same buffers.
cudaError_t launch_field_batch(const BatchBuffers& b, const BatchShapes& sh, cudaStream_t s);

// field.cu
// pow_mode of the FP64 kernels: 0 integer powers as repeated products, 1 the
// reference's polar QUATERNION::pow with the device library's transcendentals,
// 2 the same with correctly rounded ones (qj_crmath.h).
cudaError_t launch_field64(const MapParams& m, const GridParams& g, const IterParams& it,
                           int pow_mode, double* field, float* de, DevStats* st, cudaStream_t s);
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
                            int pow_mode, const uint32_t* list, const uint8_t* keys,
                            uint32_t* sorted, unsigned* hist, double* field, float* de,
                            DevStats* st, cudaStream_t s);

}  // namespace qj
