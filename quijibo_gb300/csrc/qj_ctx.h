// Internal context of the C ABI, shared by the host translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "../../include/quijibo_gpu.h"
#include "qj_mesh.h"
#include "qj_params.h"

struct qjg_ctx {
  int device = 0;
  std::string err;
  // stream-ordered memory of the calls' scratch; keeps what they free for
  // the next calls (qjg_trim returns it to the device)
  cudaMemPool_t pool = nullptr;
  std::vector<std::unique_ptr<qj::MapParams>> rootsets;
  qj::DevStats* d_stats = nullptr;  // counters of the current call
  uint32_t* d_list = nullptr;   // FP64 refine list
  size_t list_cap = 0;
  uint32_t* d_sorted = nullptr; // the refine list in orbit-length order
  size_t sorted_cap = 0;
  uint8_t* d_keys = nullptr;    // FP32 orbit length of each refine entry
  size_t keys_cap = 0;
  unsigned* d_hist = nullptr;   // counting-sort counters
  size_t hist_cap = 0;
  uint32_t* d_ff = nullptr;     // double-float re-run list
  size_t ff_cap = 0;
  double* d_field = nullptr;    // staging for host-buffer calls: two chunk buffers
  float* d_de = nullptr;
  size_t buf_cap = 0;
  size_t de_cap = 0;
  cudaStream_t copy_stream = nullptr;  // host-buffer calls: copies beside the compute stream
  cudaEvent_t chunk_ev[4] = {nullptr, nullptr, nullptr, nullptr};  // computed / copied, per buffer
  qj::DevStats* h_stats = nullptr;     // pinned per-chunk counters
  size_t h_stats_cap = 0;
  cudaStream_t stream = nullptr;  // internal stream of host-buffer calls
  // bookkeeping of the last field call, for qjg_field_stats_read
  int64_t last_voxels = 0;
  int last_roots = 0;
  // measurement hooks
  bool timing = false;
  bool timed_refine = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t mev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // mesher phases
  int64_t launches = 0;
  int64_t sq_applications = 0;  // work of the last energy call: forward map applications
  int64_t sq_steps = 0;         // ... and adjoint orbit steps
  int64_t sq_last_n = -1;       // sample count and iteration cap of that call
  int32_t sq_last_max_it = -1;
  // marching-cubes scratch
  qj::DevStats* d_mstats = nullptr;
  double* m_field = nullptr;    // slab field window
  size_t m_field_cap = 0;
  uint32_t* m_bits = nullptr;   // activity bits of the classified planes
  size_t m_bits_cap = 0;
  uint32_t* m_sign = nullptr;   // sign words of the window's planes
  size_t m_sign_cap = 0;
  uint32_t* m_ucount = nullptr; // unit counts
  size_t m_ucount_cap = 0;
  qj::McTotals* m_tot = nullptr;
  size_t m_tot_cap = 0;
  qj::McCube* m_cubes[2] = {nullptr, nullptr};  // cube lists of alternate slabs
  size_t m_cubes_cap[2] = {0, 0};
  uint8_t* m_masks = nullptr;
  size_t m_masks_cap = 0;
  int32_t* m_vbase = nullptr;
  size_t m_vbase_cap = 0;
  uint32_t* m_list = nullptr;
  size_t m_list_cap = 0;
  long long* m_bsum = nullptr;
  size_t m_bsum_cap = 0;
  double* m_verts = nullptr;    // FP64 vertex store when the caller gives none
  size_t m_verts_cap = 0;
  int32_t* m_tris = nullptr;    // compaction target of the degenerate filter
  size_t m_tris_cap = 0;
  uint8_t* m_estate = nullptr;  // bisection state per edge (FP32-first mesher)
  size_t m_estate_cap = 0;
  uint32_t* m_epark = nullptr;  // two parking lists of edges waiting for FP64
  size_t m_epark_cap = 0;
  unsigned long long* m_ecount = nullptr;
  size_t m_ecount_cap = 0;
  // the fixed launch sequence (qjg_mesh_prepare / qjg_mesh_stream_async)
  qj::McRun* m_run = nullptr;        // device counts of the run
  qj::DevStats* m_fstats = nullptr;  // the slab fields' counters, summed on the device
  long long m_prep_X = 0, m_prep_Y = 0, m_prep_nz = 0;  // what qjg_mesh_prepare sized for
  int64_t m_prep_vcap = 0, m_prep_tcap = 0;
  int32_t m_async_slabs = -1;  // slabs of the last enqueued run (-1: none)
  int64_t m_async_voxels = 0;  // its field voxels
  int m_async_roots = 0;       // its map's roots
  // edge-cache capture (qjg_mesh_capture): per vertex its edge's two corners
  // (6 ints), per mixed cube (flag, x, y, z), of the last mesher call
  bool m_capture = false;
  std::vector<int32_t> cap_edges;
  std::vector<int32_t> cap_cubes;
};


inline int fail(qjg_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

#define QJ_CUDA(ctx, call)                                                                 \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? QJG_ERR_NOMEM : QJG_ERR_CUDA,     \
                  "%s failed: %s", #call, cudaGetErrorString(e_));                         \
  } while (0)

template <class T>
inline int ensure(qjg_ctx* ctx, T** buf, size_t* cap, size_t n) {
  if (*cap >= n && *buf) return QJG_OK;
  if (*buf) cudaFree(*buf);
  *buf = nullptr;
  *cap = 0;
  QJ_CUDA(ctx, cudaMalloc((void**)buf, n * sizeof(T)));
  *cap = n;
  return QJG_OK;
}


// shared by the field and mesh entry points (api.cpp)
// Fills the launch parameters of the map s * prod (q - t_i)^(sigma_t e_i) /
// prod (q - b_j)^(sigma_b f_j).  Returns -1 when every value is finite, else
// the index of the first root (coordinate or exponent) that is not.
int qj_fill_map(qj::MapParams* m, int n_top, const double* top_roots, const double* top_powers,
                double sigma_top, int n_bot, const double* bot_roots, const double* bot_powers,
                double sigma_bot, double scale);
int qj_check_grid(qjg_ctx* ctx, const qjg_grid* g);
int qj_check_iter(qjg_ctx* ctx, const qjg_iter* it);
// pow_mode of the FP64 kernels (qj_kernels.h) for these settings: the
// reference's polar pow unless integer products were asked for and apply
// Stream-ordered allocation from the context's pool.
template <class T>
inline cudaError_t qj_malloc_async(qjg_ctx* ctx, T** p, size_t bytes, cudaStream_t s) {
  return cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), bytes, ctx->pool, s);
}

// Whether the context's pool keeps freed memory past a synchronization (the
// default) or returns it to the device then.
inline cudaError_t qj_pool_keep(qjg_ctx* ctx, bool keep) {
  uint64_t thr = keep ? ~0ull : 0ull;
  return cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &thr);
}

inline int qj_pow_mode(const qjg_iter* it, bool all_int) {
  const bool pow_ref = !it || it->refine_pow == QJG_REFINE_POW || !all_int;
  return pow_ref ? (it && it->libm == QJG_LIBM_CR ? 2 : 1) : 0;
}
qj::GridParams qj_grid_params(const qjg_grid* g, int z0, int z1);
qj::IterParams qj_iter_params(const qjg_iter* it, const qjg_grid* g);
qj::MapParams* qj_lookup(qjg_ctx* ctx, qjg_rootset rs);
// trilinear-lookup geometry of a FIELD_3D on grid g (energy_api.cpp)
qj::WeightGrid qj_weight_grid(const qjg_grid* g);
