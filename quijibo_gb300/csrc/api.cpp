// C ABI of the QUIJIBO hot path: contexts, resident root sets, field calls.
// Compiled with -ffp-contract=off: the rotation matrix and exponent products
// computed here must round like the reference's host code.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/quijibo_gpu.h"
#include "../../include/quijibo_gpu_bench.h"
#include "qj_ctx.h"
#include "qj_kernels.h"

using qj::DevStats;
using qj::GridParams;
using qj::IterParams;
using qj::MapParams;

namespace {

// QUATERNION::toRotationMatrix, src/algebra/QUATERNION.cpp:395-411.
void rotation_matrix(const double q[4], double R[3][3]) {
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  R[0][0] = 1 - 2 * y * y - 2 * z * z;
  R[0][1] = 2 * x * y - 2 * w * z;
  R[0][2] = 2 * x * z + 2 * w * y;
  R[1][0] = 2 * x * y + 2 * w * z;
  R[1][1] = 1 - 2 * x * x - 2 * z * z;
  R[1][2] = 2 * y * z - 2 * w * x;
  R[2][0] = 2 * x * z - 2 * w * y;
  R[2][1] = 2 * y * z + 2 * w * x;
  R[2][2] = 1 - 2 * x * x - 2 * y * y;
}

// The device address of a page-locked (cudaHostAlloc / cudaHostRegister)
// host buffer, or null for other memory.
void* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

}  // namespace

// scratch target for stats nobody asked for
static qjg_field_stats& total_sink(qjg_ctx*) {
  static thread_local qjg_field_stats sink;
  return sink;
}

int qj_check_grid(qjg_ctx* ctx, const qjg_grid* g) {
  if (!g) return fail(ctx, QJG_ERR_ARG, "grid is NULL");
  for (int c = 0; c < 3; c++) {
    if (g->res[c] < 1) return fail(ctx, QJG_ERR_ARG, "grid res[%d] = %d < 1", c, g->res[c]);
    if (!(g->lengths[c] > 0) || !std::isfinite(g->lengths[c]))
      return fail(ctx, QJG_ERR_ARG, "grid lengths[%d] must be finite and > 0", c);
  }
  return QJG_OK;
}

GridParams qj_grid_params(const qjg_grid* g, int z0, int z1) {
  GridParams p;
  p.X = g->res[0];
  p.Y = g->res[1];
  p.Z = g->res[2];
  p.z0 = z0;
  p.z1 = z1;
  for (int c = 0; c < 3; c++) {
    p.center[c] = g->center[c];
    p.half[c] = g->lengths[c] * 0.5;  // (Real)0.5 * _lengths
    p.dx[c] = g->lengths[c] / g->res[c];
  }
  rotation_matrix(g->rot, p.R);
  p.slice = g->slice;
  // cell centre = center + R (center - half + (idx + 0.5) dx - center)
  auto split = [](double v, float out[2]) {
    out[0] = (float)v;
    out[1] = (float)(v - (double)out[0]);
  };
  for (int c = 0; c < 3; c++) {
    double a = p.center[c];
    for (int k = 0; k < 3; k++) {
      a += p.R[c][k] * (-p.half[k] + 0.5 * p.dx[k]);
      split(p.R[c][k] * p.dx[k], p.ffb[c][k]);
    }
    split(a, p.ffa[c]);
  }
  split(p.slice, p.ffslice);
  return p;
}

int qj_check_iter(qjg_ctx* ctx, const qjg_iter* it) {
  if (!it) return fail(ctx, QJG_ERR_ARG, "iter is NULL");
  if (it->max_it < 0) return fail(ctx, QJG_ERR_ARG, "max_it = %d < 0", it->max_it);
  if (!(it->escape > 0)) return fail(ctx, QJG_ERR_ARG, "escape radius must be > 0");
  if (it->precision < QJG_FP64 || it->precision > QJG_FP32_REFINE)
    return fail(ctx, QJG_ERR_ARG, "unknown precision %d", it->precision);
  if (it->refine_pow != QJG_REFINE_POW && it->refine_pow != QJG_REFINE_INT)
    return fail(ctx, QJG_ERR_ARG, "unknown refine_pow %d", it->refine_pow);
  if (it->form != QJG_FORM_QUOTIENT && it->form != QJG_FORM_LAGRANGE)
    return fail(ctx, QJG_ERR_ARG, "unknown form %d", it->form);
  if (it->libm != QJG_LIBM_DEVICE && it->libm != QJG_LIBM_CR)
    return fail(ctx, QJG_ERR_ARG, "unknown libm %d", it->libm);
  return QJG_OK;
}

IterParams qj_iter_params(const qjg_iter* it, const qjg_grid* g) {
  IterParams p;
  p.max_it = it->max_it;
  p.want_de = it->want_de ? 1 : 0;
  p.escape = it->escape;
  double h = g->lengths[0] / g->res[0];
  for (int c = 1; c < 3; c++) h = std::fmin(h, g->lengths[c] / g->res[c]);
  p.band = it->band_h * h;
  p.field_tol = it->field_tol;
  // voxels whose tracked error estimate exceeds rel_tol are re-run: the
  // estimate is a first-order bound and overshoots the actual FP32 error
  // (5x or more for 99.9% of voxels on the precision and large workloads)
  p.est_tol = it->rel_tol > 0 ? it->rel_tol : 0.0;
  p.ff_head = 2;
  p.lagrange = it->form == QJG_FORM_LAGRANGE ? 1 : 0;
  p.field_tolf = (float)p.field_tol;
  p.est_tolf = (float)p.est_tol;
  return p;
}

MapParams* qj_lookup(qjg_ctx* ctx, qjg_rootset rs) {
  if (rs < 0 || rs >= (int)ctx->rootsets.size()) return nullptr;
  return ctx->rootsets[rs].get();
}

int qj_fill_map(MapParams* m, int n_top, const double* top_roots, const double* top_powers,
                double sigma_top, int n_bot, const double* bot_roots, const double* bot_powers,
                double sigma_bot, double scale) {
  std::memset(m, 0, sizeof(MapParams));
  m->nt = n_top;
  m->nb = n_bot;
  m->scale = scale;
  m->scalef = (float)scale;
  m->scale_ff[0] = m->scalef;
  m->scale_ff[1] = (float)(scale - (double)m->scalef);
  m->sigma[0] = sigma_top;
  m->sigma[1] = sigma_bot;
  m->all_int = 1;
  for (int i = 0; i < n_top + n_bot; i++) {
    const bool top = i < n_top;
    const double* r = top ? top_roots + 4 * i : bot_roots + 4 * (i - n_top);
    const double pw = top ? top_powers[i] : bot_powers[i - n_top];
    // _powerScalar * _rootPowers[x], POLYNOMIAL_4D.cpp:914, 919
    const double e = (top ? sigma_top : sigma_bot) * pw;
    if (!std::isfinite(e)) return i;
    for (int c = 0; c < 4; c++) {
      if (!std::isfinite(r[c])) return i;
      m->r64[i][c] = r[c];
      m->r32[i][c] = (float)r[c];
      m->rn2[i][c] = make_float2(-m->r32[i][c], -m->r32[i][c]);
      m->rff[i][c][0] = m->r32[i][c];
      m->rff[i][c][1] = (float)(r[c] - (double)m->r32[i][c]);
    }
    m->e64[i] = e;
    m->ep[i] = pw;
    m->e32[i] = (float)e;
    const bool integral = (e == std::floor(e)) && e >= 1 && e <= QJ_MAX_INT_EXP;
    m->ie[i] = integral ? (int)e : 0;
    if (!integral) m->all_int = 0;
    m->x32[i][0] = top ? (float)e : -(float)e;
    m->ex2[i] = make_float2(m->x32[i][0], m->x32[i][0]);
    const int ie_bits = m->ie[i];
    std::memcpy(&m->x32[i][1], &ie_bits, sizeof ie_bits);
  }
  return -1;
}

extern "C" {

int qjg_create(int device, qjg_ctx** out) {
  if (!out) return QJG_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return QJG_ERR_CUDA;
  std::unique_ptr<qjg_ctx> ctx(new qjg_ctx());
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess) return QJG_ERR_CUDA;
  if (cudaMalloc((void**)&ctx->d_stats, sizeof(DevStats)) != cudaSuccess) return QJG_ERR_NOMEM;
  if (cudaMalloc((void**)&ctx->d_mstats, sizeof(DevStats)) != cudaSuccess) return QJG_ERR_NOMEM;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
    return QJG_ERR_CUDA;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  if (cudaMemPoolCreate(&ctx->pool, &props) != cudaSuccess) {
    cudaStreamDestroy(ctx->stream);
    return QJG_ERR_CUDA;
  }
  // Keep freed scratch for the next calls: returning it at every
  // synchronization cost 0.4 ms per energy + gradient call (200k samples,
  // 30 iterations: 2.21 ms against 1.81 ms).
  if (qj_pool_keep(ctx.get(), true) != cudaSuccess) {
    cudaMemPoolDestroy(ctx->pool);
    cudaStreamDestroy(ctx->stream);
    return QJG_ERR_CUDA;
  }
  *out = ctx.release();
  return QJG_OK;
}

int qjg_trim(qjg_ctx* ctx) {
  if (!ctx) return QJG_ERR_ARG;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  QJ_CUDA(ctx, cudaMemPoolTrimTo(ctx->pool, 0));
  return QJG_OK;
}

void qjg_destroy(qjg_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_stats);
  cudaFree(ctx->d_list);
  cudaFree(ctx->d_sorted);
  cudaFree(ctx->d_keys);
  cudaFree(ctx->d_hist);
  cudaFree(ctx->d_ff);
  if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
  for (cudaEvent_t e : ctx->chunk_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  cudaFree(ctx->d_field);
  cudaFree(ctx->d_de);
  cudaFree(ctx->d_mstats);
  cudaFree(ctx->m_field);
  cudaFree(ctx->m_bits);
  cudaFree(ctx->m_sign);
  cudaFree(ctx->m_ucount);
  cudaFree(ctx->m_tot);
  cudaFree(ctx->m_cubes[0]);
  cudaFree(ctx->m_cubes[1]);
  cudaFree(ctx->m_masks);
  cudaFree(ctx->m_vbase);
  cudaFree(ctx->m_list);
  cudaFree(ctx->m_bsum);
  cudaFree(ctx->m_verts);
  cudaFree(ctx->m_tris);
  cudaFree(ctx->m_estate);
  cudaFree(ctx->m_epark);
  cudaFree(ctx->m_ecount);
  cudaFree(ctx->m_run);
  cudaFree(ctx->m_fstats);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
  for (cudaEvent_t e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->mev)
    if (e) cudaEventDestroy(e);
  delete ctx;
}

const char* qjg_last_error(qjg_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int qjg_rootset_upload(qjg_ctx* ctx, int32_t n_top, const double* top_roots,
                       const double* top_powers, double sigma_top, int32_t n_bot,
                       const double* bot_roots, const double* bot_powers, double sigma_bot,
                       double scale, qjg_rootset* out) {
  if (!ctx || !out) return QJG_ERR_ARG;
  if (n_top < 1 || n_bot < 0 || n_top + n_bot > QJG_MAX_ROOTS)
    return fail(ctx, QJG_ERR_ARG, "root counts top=%d bottom=%d (need top >= 1, total <= %d)",
                n_top, n_bot, QJG_MAX_ROOTS);
  if (!top_roots || !top_powers || (n_bot > 0 && (!bot_roots || !bot_powers)))
    return fail(ctx, QJG_ERR_ARG, "root or power array is NULL");
  std::unique_ptr<MapParams> m(new MapParams());
  const int bad = qj_fill_map(m.get(), n_top, top_roots, top_powers, sigma_top, n_bot, bot_roots,
                              bot_powers, sigma_bot, scale);
  if (bad >= 0) return fail(ctx, QJG_ERR_ARG, "root %d or its exponent is not finite", bad);
  ctx->rootsets.push_back(std::move(m));
  *out = (qjg_rootset)(ctx->rootsets.size() - 1);
  return QJG_OK;
}

int qjg_rootset_free(qjg_ctx* ctx, qjg_rootset rs) {
  if (!ctx) return QJG_ERR_ARG;
  if (!qj_lookup(ctx, rs)) return fail(ctx, QJG_ERR_HANDLE, "unknown root set %d", rs);
  ctx->rootsets[rs].reset();
  return QJG_OK;
}

int qjg_field(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
              int32_t z0, int32_t z1, double* d_field, float* d_de, void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  const MapParams* m0 = qj_lookup(ctx, rs);
  // the Lagrange order rides with the launch copy of the map (FP32 and
  // double-float tiers); the resident map keeps the quotient default
  std::unique_ptr<MapParams> mcopy;
  const MapParams* m = m0;
  if (m0 && iter && iter->form == QJG_FORM_LAGRANGE) {
    mcopy.reset(new MapParams(*m0));
    mcopy->lagrange = 1;
    m = mcopy.get();
  }
  if (!m) return fail(ctx, QJG_ERR_HANDLE, "unknown root set %d", rs);
  int rc;
  if ((rc = qj_check_grid(ctx, grid)) || (rc = qj_check_iter(ctx, iter))) return rc;
  if (z0 < 0 || z1 > grid->res[2] || z0 >= z1)
    return fail(ctx, QJG_ERR_ARG, "slice range [%d, %d) outside [0, %d)", z0, z1, grid->res[2]);
  if (!d_field) return fail(ctx, QJG_ERR_ARG, "d_field is NULL");
  const int64_t n = (int64_t)grid->res[0] * grid->res[1] * (z1 - z0);
  const bool refine = iter->precision == QJG_FP32_REFINE;
  if (refine && n > (int64_t)UINT32_MAX)
    return fail(ctx, QJG_ERR_ARG, "%lld voxels in one call; split the slice range below 2^32",
                (long long)n);
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = (cudaStream_t)stream;
  const GridParams g = qj_grid_params(grid, z0, z1);
  IterParams it = qj_iter_params(iter, grid);
  const int pow_mode = qj_pow_mode(iter, m->all_int);
  if (refine && ((rc = ensure(ctx, &ctx->d_list, &ctx->list_cap, (size_t)n)) ||
                 (rc = ensure(ctx, &ctx->d_sorted, &ctx->sorted_cap, (size_t)n)) ||
                 (rc = ensure(ctx, &ctx->d_keys, &ctx->keys_cap, (size_t)n)) ||
                 (rc = ensure(ctx, &ctx->d_hist, &ctx->hist_cap, (size_t)qj::REFINE_KEYS))))
    return rc;
  const bool rerun = refine && it.est_tol > 0.0 && m->all_int;
  if (rerun && (rc = ensure(ctx, &ctx->d_ff, &ctx->ff_cap, (size_t)n))) return rc;
  QJ_CUDA(ctx, cudaMemsetAsync(ctx->d_stats, 0, sizeof(DevStats), s));
  if (ctx->timing) QJ_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
  if (iter->precision == QJG_FP64) {
    QJ_CUDA(ctx, qj::launch_field64(*m, g, it, pow_mode, d_field, d_de, ctx->d_stats, s));
  } else {
    QJ_CUDA(ctx, qj::launch_field32(*m, g, it, refine, d_field, d_de, ctx->d_list, ctx->d_keys,
                                    rerun ? ctx->d_ff : nullptr, ctx->d_stats, s));
  }
  ctx->launches++;
  if (ctx->timing) QJ_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
  if (rerun) {
    QJ_CUDA(ctx, qj::launch_rerun_ff(*m, g, it, ctx->d_ff, d_field, d_de, ctx->d_list, ctx->d_keys,
                                     ctx->d_stats, s));
    ctx->launches++;
  }
  if (refine) {
    QJ_CUDA(ctx, qj::launch_refine64(*m, g, it, pow_mode, ctx->d_list, ctx->d_keys,
                                     ctx->d_sorted, ctx->d_hist, d_field, d_de, ctx->d_stats, s));
    ctx->launches += 4;  // histogram, offsets, scatter, refine
  }
  if (ctx->timing) QJ_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
  ctx->timed_refine = refine;
  ctx->last_voxels = n;
  ctx->last_roots = m->nt + m->nb;
  return QJG_OK;
}

int qjg_field_stats_read(qjg_ctx* ctx, void* stream, qjg_field_stats* out) {
  if (!ctx || !out) return QJG_ERR_ARG;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  QJ_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream));
  DevStats st;
  QJ_CUDA(ctx, cudaMemcpy(&st, ctx->d_stats, sizeof st, cudaMemcpyDeviceToHost));
  out->voxels = ctx->last_voxels;
  out->voxel_iters = (int64_t)st.voxel_iters;
  out->root_terms = (int64_t)st.voxel_iters * ctx->last_roots;
  out->refined = (int64_t)st.refined;
  out->refined_iters = (int64_t)st.aux[0];
  out->nonfinite = (int64_t)st.nonfinite;
  out->lane_iters = (int64_t)st.aux[3];
  out->rerun = (int64_t)st.rerun;
  out->rerun_iters = (int64_t)st.rerun_iters;
  return QJG_OK;
}

int qjg_field_host(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
                   double* host_field, float* host_de, qjg_field_stats* stats) {
  if (!ctx) return QJG_ERR_ARG;
  int rc;
  if ((rc = qj_check_grid(ctx, grid)) || (rc = qj_check_iter(ctx, iter))) return rc;
  if (!host_field) return fail(ctx, QJG_ERR_ARG, "host_field is NULL");
  const int64_t slab = (int64_t)grid->res[0] * grid->res[1];
  // chunks of slices, computed on ctx->stream into two alternating device
  // buffers while the previous chunk copies out on ctx->copy_stream: about
  // eight chunks of at least 2^22 voxels, at most 2^27 voxels each
  const int64_t Z = grid->res[2];
  int64_t chunk = std::max<int64_t>((Z + 7) / 8, ((int64_t)1 << 22) / slab);
  chunk = std::max<int64_t>(1, std::min<int64_t>(chunk, ((int64_t)1 << 27) / slab));
  chunk = std::min<int64_t>(chunk, Z);
  const int64_t n_chunks = (Z + chunk - 1) / chunk;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  // page-locked host buffers are mapped into the device's address space: the
  // kernels then write the field straight into them (over NVLink-C2C on a
  // Grace host) and nothing is staged or copied
  void* df_mapped = mapped_host(host_field);
  void* dd_mapped = host_de ? mapped_host(host_de) : nullptr;
  if (df_mapped && (!host_de || dd_mapped) && slab * Z <= (int64_t)UINT32_MAX) {
    if ((rc = qjg_field(ctx, rs, grid, iter, 0, (int32_t)Z, (double*)df_mapped, (float*)dd_mapped,
                        ctx->stream)))
      return rc;
    return qjg_field_stats_read(ctx, ctx->stream, stats ? stats : &total_sink(ctx));
  }
  if ((rc = ensure(ctx, &ctx->d_field, &ctx->buf_cap, (size_t)(2 * chunk * slab)))) return rc;
  if (host_de && (rc = ensure(ctx, &ctx->d_de, &ctx->de_cap, (size_t)(2 * chunk * slab))))
    return rc;
  if (!ctx->copy_stream)
    QJ_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  for (cudaEvent_t& e : ctx->chunk_ev)
    if (!e) QJ_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  if (ctx->h_stats_cap < (size_t)n_chunks) {
    if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
    ctx->h_stats = nullptr;
    ctx->h_stats_cap = 0;
    QJ_CUDA(ctx, cudaMallocHost((void**)&ctx->h_stats, (size_t)n_chunks * sizeof(DevStats)));
    ctx->h_stats_cap = (size_t)n_chunks;
  }
  cudaStream_t cs = ctx->stream, xs = ctx->copy_stream;
  for (int64_t k = 0; k < n_chunks; k++) {
    const int64_t z0 = k * chunk, z1 = std::min<int64_t>(z0 + chunk, Z);
    const int b = (int)(k & 1);
    double* df = ctx->d_field + (size_t)b * chunk * slab;
    float* dd = host_de ? ctx->d_de + (size_t)b * chunk * slab : nullptr;
    // the buffer's previous chunk must have left the device
    if (k >= 2) QJ_CUDA(ctx, cudaStreamWaitEvent(cs, ctx->chunk_ev[2 + b], 0));
    if ((rc = qjg_field(ctx, rs, grid, iter, (int32_t)z0, (int32_t)z1, df, dd, cs))) return rc;
    QJ_CUDA(ctx, cudaMemcpyAsync(ctx->h_stats + k, ctx->d_stats, sizeof(DevStats),
                                 cudaMemcpyDeviceToHost, cs));
    QJ_CUDA(ctx, cudaEventRecord(ctx->chunk_ev[b], cs));
    QJ_CUDA(ctx, cudaStreamWaitEvent(xs, ctx->chunk_ev[b], 0));
    const size_t nb = (size_t)((z1 - z0) * slab);
    QJ_CUDA(ctx, cudaMemcpyAsync(host_field + z0 * slab, df, nb * sizeof(double),
                                 cudaMemcpyDeviceToHost, xs));
    if (host_de)
      QJ_CUDA(ctx, cudaMemcpyAsync(host_de + z0 * slab, dd, nb * sizeof(float),
                                   cudaMemcpyDeviceToHost, xs));
    QJ_CUDA(ctx, cudaEventRecord(ctx->chunk_ev[2 + b], xs));
  }
  QJ_CUDA(ctx, cudaStreamSynchronize(cs));
  QJ_CUDA(ctx, cudaStreamSynchronize(xs));
  qjg_field_stats total = {};
  const int roots = ctx->last_roots;
  for (int64_t k = 0; k < n_chunks; k++) {
    const DevStats& st = ctx->h_stats[k];
    const int64_t z0 = k * chunk, z1 = std::min<int64_t>(z0 + chunk, Z);
    total.voxels += (z1 - z0) * slab;
    total.voxel_iters += (int64_t)st.voxel_iters;
    total.root_terms += (int64_t)st.voxel_iters * roots;
    total.refined += (int64_t)st.refined;
    total.refined_iters += (int64_t)st.aux[0];
    total.nonfinite += (int64_t)st.nonfinite;
    total.lane_iters += (int64_t)st.aux[3];
    total.rerun += (int64_t)st.rerun;
    total.rerun_iters += (int64_t)st.rerun_iters;
  }
  if (stats) *stats = total;
  return QJG_OK;
}

int qjg_set_timing(qjg_ctx* ctx, int on) {
  if (!ctx) return QJG_ERR_ARG;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  for (cudaEvent_t& e : ctx->ev)
    if (!e) QJ_CUDA(ctx, cudaEventCreate(&e));
  for (cudaEvent_t& e : ctx->mev)
    if (!e) QJ_CUDA(ctx, cudaEventCreate(&e));
  ctx->timing = on != 0;
  return QJG_OK;
}

int qjg_last_timings(qjg_ctx* ctx, float* ms_bulk, float* ms_refine) {
  if (!ctx || !ms_bulk || !ms_refine) return QJG_ERR_ARG;
  if (!ctx->timing) return fail(ctx, QJG_ERR_ARG, "timing is off (qjg_set_timing)");
  QJ_CUDA(ctx, cudaEventSynchronize(ctx->ev[2]));
  QJ_CUDA(ctx, cudaEventElapsedTime(ms_bulk, ctx->ev[0], ctx->ev[1]));
  *ms_refine = 0.f;
  if (ctx->timed_refine) QJ_CUDA(ctx, cudaEventElapsedTime(ms_refine, ctx->ev[1], ctx->ev[2]));
  return QJG_OK;
}

int64_t qjg_launch_count(qjg_ctx* ctx) { return ctx ? ctx->launches : -1; }

int qjg_set_field32_pairs(int on) {
  qj::set_field32_pairs(on);
  return QJG_OK;
}

}  // extern "C"
