// Field entry point that allocates no device memory.
//
// Some callers of this library cannot allocate device memory on the path
// that computes a field: plugins hosted by an application that owns every
// device allocation (its own memory pool, no room for a library's
// cudaMalloc), real-time loops that must not reach the allocator, and
// processes held to a fixed device-memory quota.  qjg_field_noalloc serves them.  The caller passes the map
// (host arrays), the grid, the iteration settings and a device output
// buffer; the only device memory the call touches besides that buffer is a
// fixed scratch array of this file (the counters, the FP64 refine list and
// the double-float re-run list of the FP32 + FP64-refine form, about 32 MiB),
// which lives for as long as the library is loaded on a device.  Every call shares that array, so calls whose work overlaps
// on the GPU (different streams, or different host threads) race on it and
// must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/quijibo_gpu.h"
#include "qj_ctx.h"
#include "qj_kernels.h"

namespace {

constexpr int kMaxDevices = 64;

// [0, 256): the counters (qj::DevStats, padded); then two lists of one
// uint32 entry per voxel of the largest launch: the FP64 refine list and the
// double-float re-run list (the same two lists qjg_field fills).
constexpr size_t kStatsBytes = 256;
static_assert(sizeof(qj::DevStats) <= kStatsBytes, "the counters overlap the refine list");
constexpr size_t kListBytes = sizeof(uint32_t) * (size_t)QJG_NOALLOC_MAX_VOXELS;
constexpr size_t kScratchBytes = kStatsBytes + 2 * kListBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// The device address of the scratch array for the current device, looked up
// once per device (host code must not use the symbol itself as an address).
int scratch_for_current_device(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return QJG_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return QJG_ERR_CUDA;
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_addr[dev];
  return QJG_OK;
}

}  // namespace

extern "C" int qjg_field_noalloc(int32_t n_top, const double* top_roots, const double* top_powers,
                                 double sigma_top, int32_t n_bot, const double* bot_roots,
                                 const double* bot_powers, double sigma_bot, double scale,
                                 const qjg_grid* grid, const qjg_iter* iter, int32_t z0, int32_t z1,
                                 double* d_field, float* d_de, void* stream) {
  if (n_top < 1 || n_bot < 0 || n_top + n_bot > QJG_MAX_ROOTS) return QJG_ERR_ARG;
  if (!top_roots || !top_powers || (n_bot > 0 && (!bot_roots || !bot_powers)) || !d_field)
    return QJG_ERR_ARG;
  int rc;
  if ((rc = qj_check_grid(nullptr, grid)) || (rc = qj_check_iter(nullptr, iter))) return rc;
  if (z0 < 0 || z1 > grid->res[2] || z0 >= z1) return QJG_ERR_ARG;
  const int64_t n = (int64_t)grid->res[0] * grid->res[1] * (z1 - z0);
  if (n > (int64_t)QJG_NOALLOC_MAX_VOXELS) return QJG_ERR_CAPACITY;

  // the map's launch parameters, built on the host stack
  qj::MapParams m;
  if (qj_fill_map(&m, n_top, top_roots, top_powers, sigma_top, n_bot, bot_roots, bot_powers,
                  sigma_bot, scale) >= 0)
    return QJG_ERR_ARG;

  m.lagrange = iter->form == QJG_FORM_LAGRANGE ? 1 : 0;

  unsigned char* scratch = nullptr;
  if ((rc = scratch_for_current_device(&scratch))) return rc;
  qj::DevStats* st = reinterpret_cast<qj::DevStats*>(scratch);
  uint32_t* list = reinterpret_cast<uint32_t*>(scratch + kStatsBytes);
  uint32_t* ff_list = reinterpret_cast<uint32_t*>(scratch + kStatsBytes + kListBytes);

  cudaStream_t s = (cudaStream_t)stream;
  const qj::GridParams g = qj_grid_params(grid, z0, z1);
  const qj::IterParams it = qj_iter_params(iter, grid);
  const bool refine = iter->precision == QJG_FP32_REFINE;
  const int pow_mode = qj_pow_mode(iter, m.all_int);
  // the counters (work-queue position, refine-list length) start at zero
  if (cudaMemsetAsync(st, 0, sizeof(qj::DevStats), s) != cudaSuccess) return QJG_ERR_CUDA;
  // voxels whose tracked FP32 error exceeds rel_tol are re-run with a
  // double-float head first, as in qjg_field, so both give the same bits
  const bool rerun = refine && it.est_tol > 0.0 && m.all_int;
  cudaError_t e;
  if (iter->precision == QJG_FP64)
    e = qj::launch_field64(m, g, it, pow_mode, d_field, d_de, st, s);
  else
    e = qj::launch_field32(m, g, it, refine, d_field, d_de, list, nullptr,
                           rerun ? ff_list : nullptr, st, s);
  if (e == cudaSuccess && rerun)
    e = qj::launch_rerun_ff(m, g, it, ff_list, d_field, d_de, list, nullptr, st, s);
  if (e == cudaSuccess && refine)
    e = qj::launch_refine64(m, g, it, pow_mode, list, nullptr, nullptr, nullptr, d_field, d_de, st,
                            s);
  return e == cudaSuccess ? QJG_OK : QJG_ERR_CUDA;
}
