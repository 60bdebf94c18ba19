// C ABI of the marching-cubes mesher: slab orchestration on the host.
// The reference's two-slab streaming mesher keeps two FIELD_2D slices alive
// (TRIANGLE_MESH.cpp:4884-4911); here a window of slab_nz cube layers is
// classified, numbered and emitted per pass, with one layer/plane of flags,
// edge masks and vertex ids carried to the next pass (see mesh.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>

#include "../../include/quijibo_gpu_bench.h"
#include "qj_ctx.h"
#include "qj_kernels.h"
#include "qj_mesh.h"

using qj::GridParams;
using qj::IterParams;
using qj::MapParams;

namespace {

// Grow a device buffer to hold n elements, keeping the first `keep`.
template <class T>
int grow_keep(qjg_ctx* ctx, T** buf, size_t* cap, size_t n, size_t keep, cudaStream_t s,
              size_t hint = 0) {
  if (*cap >= n && *buf) return QJG_OK;
  size_t want = std::max(std::max(n, *cap + *cap / 2), hint);
  T* nb = nullptr;
  QJ_CUDA(ctx, cudaMalloc((void**)&nb, want * sizeof(T)));
  if (*buf && keep) QJ_CUDA(ctx, cudaMemcpyAsync(nb, *buf, keep * sizeof(T), cudaMemcpyDeviceToDevice, s));
  QJ_CUDA(ctx, cudaStreamSynchronize(s));
  if (*buf) cudaFree(*buf);
  *buf = nb;
  *cap = want;
  return QJG_OK;
}

// Edge-cache capture of one slab: its vertices' edges (window-encoded list
// entries: window voxel index * 4 + axis, window plane 0 = global c0 - 1)
// and its new cube entries, appended in order.
int capture_slab(qjg_ctx* ctx, const uint32_t* d_list, long long n_new, const qj::McCube* d_cubes,
                 long long nc, int X, int Y, int c0, cudaStream_t s) {
  std::vector<uint32_t> list((size_t)n_new);
  std::vector<qj::McCube> cubes((size_t)nc);
  if (n_new)
    QJ_CUDA(ctx, cudaMemcpyAsync(list.data(), d_list, (size_t)n_new * sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, s));
  if (nc)
    QJ_CUDA(ctx, cudaMemcpyAsync(cubes.data(), d_cubes, (size_t)nc * sizeof(qj::McCube),
                                 cudaMemcpyDeviceToHost, s));
  QJ_CUDA(ctx, cudaStreamSynchronize(s));
  const long long XY = (long long)X * Y;
  for (uint32_t e : list) {
    const long long wv = e >> 2;
    const int a = (int)(e & 3u);
    const int z = c0 - 1 + (int)(wv / XY);
    const int r = (int)(wv % XY);
    const int p[3] = {r % X, r / X, z};
    for (int k = 0; k < 3; k++) ctx->cap_edges.push_back(p[k]);
    for (int k = 0; k < 3; k++) ctx->cap_edges.push_back(p[k] + (k == a));
  }
  for (const qj::McCube& q : cubes) {
    ctx->cap_cubes.push_back((int32_t)(q.gzf >> 24));
    ctx->cap_cubes.push_back((int32_t)(q.r % (uint32_t)X));
    ctx->cap_cubes.push_back((int32_t)(q.r / (uint32_t)X));
    ctx->cap_cubes.push_back((int32_t)(q.gzf & 0xFFFFFFu));
  }
  return QJG_OK;
}

int mesh_core(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
              bool streaming, const double* d_field, int edge_mode, double iso, int slab_nz,
              double* v64, float* v32, int64_t vcap, int32_t* tris, int64_t tcap,
              qjg_mesh_stats* out, cudaStream_t s) {
  int rc;
  if ((rc = qj_check_grid(ctx, grid))) return rc;
  if (edge_mode != QJG_EDGE_LINEAR && edge_mode != QJG_EDGE_BISECT)
    return fail(ctx, QJG_ERR_ARG, "unknown edge_mode %d", edge_mode);
  const bool bisect = edge_mode == QJG_EDGE_BISECT;
  MapParams zero_map;
  std::memset(&zero_map, 0, sizeof zero_map);
  const MapParams* m = &zero_map;
  std::unique_ptr<MapParams> mcopy;  // the Lagrange order rides with a launch copy
  if (bisect || streaming) {
    m = qj_lookup(ctx, rs);
    if (!m) return fail(ctx, QJG_ERR_HANDLE, "unknown root set %d", rs);
    if ((rc = qj_check_iter(ctx, iter))) return rc;
    if (iter->form == QJG_FORM_LAGRANGE) {
      mcopy.reset(new MapParams(*m));
      mcopy->lagrange = 1;
      m = mcopy.get();
    }
  }
  if (!streaming && !d_field) return fail(ctx, QJG_ERR_ARG, "d_field is NULL");
  if (!tris) return fail(ctx, QJG_ERR_ARG, "d_tris is NULL");
  if (vcap < 0 || tcap < 0) return fail(ctx, QJG_ERR_ARG, "negative capacity");
  qjg_mesh_stats st;
  std::memset(&st, 0, sizeof st);
  ctx->cap_edges.clear();
  ctx->cap_cubes.clear();

  const int X = grid->res[0], Y = grid->res[1], Z = grid->res[2];
  const long long XY = (long long)X * Y;
  int nz = slab_nz > 0 ? slab_nz : 64;
  // edge-list entries are window voxel index * 4 + axis in 32 bits
  const long long nz_max = (long long)(UINT32_MAX / 4) / XY - 2;
  if (nz_max < 1) return fail(ctx, QJG_ERR_ARG, "a %d x %d slice is too large", X, Y);
  nz = (int)std::min<long long>(nz, nz_max);
  nz = std::max(1, std::min(nz, std::max(Z - 1, 1)));
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));

  // without a cube (a grid one cell thin) there is no triangle and no vertex
  if (X < 2 || Y < 2) {
    if (out) *out = st;
    return QJG_OK;
  }
  const size_t wplanes = (size_t)(nz + 2) * XY;
  const long long units = qj::mesh_units(X, Y, nz + 1);
  if ((rc = ensure(ctx, &ctx->m_masks, &ctx->m_masks_cap, wplanes)) ||
      (rc = ensure(ctx, &ctx->m_vbase, &ctx->m_vbase_cap, wplanes)) ||
      (rc = ensure(ctx, &ctx->m_sign, &ctx->m_sign_cap, (size_t)units * qj::MESH_UNIT_WORDS)) ||
      (rc = ensure(ctx, &ctx->m_bits, &ctx->m_bits_cap, (size_t)units * qj::MESH_UNIT_WORDS)) ||
      (rc = ensure(ctx, &ctx->m_ucount, &ctx->m_ucount_cap, (size_t)units)) ||
      (rc = ensure(ctx, &ctx->m_tot, &ctx->m_tot_cap, (size_t)1)) ||
      (rc = ensure(ctx, &ctx->m_bsum, &ctx->m_bsum_cap,
                   (size_t)std::max(2 * qj::mesh_scan_blocks(units), (long long)1))))
    return rc;
  if (streaming && (rc = ensure(ctx, &ctx->m_field, &ctx->m_field_cap, (size_t)(nz + 1) * XY)))
    return rc;
  QJ_CUDA(ctx, cudaMemsetAsync(ctx->d_mstats, 0, sizeof(qj::DevStats), s));
  if ((rc = ensure(ctx, &ctx->m_ecount, &ctx->m_ecount_cap, (size_t)3))) return rc;
  QJ_CUDA(ctx, cudaMemsetAsync(ctx->m_ecount, 0, 3 * sizeof(unsigned long long), s));

  qj::MeshWindow w;
  w.X = X;
  w.Y = Y;
  w.masks = ctx->m_masks;
  w.vbase = ctx->m_vbase;
  w.list = ctx->m_list;
  w.bsum = ctx->m_bsum;
  w.bits = ctx->m_bits;
  w.sign = ctx->m_sign;
  w.ucount = ctx->m_ucount;
  w.tot = ctx->m_tot;
  const GridParams g = qj_grid_params(grid, 0, Z);
  IterParams it{};
  if (iter) it = qj_iter_params(iter, grid);
  const int pow_mode = qj_pow_mode(iter, m->all_int);
  const long long S = (X + 63) / 64;  // units per row (qj::mesh_units)

  long long nv = 0, nt = 0;
  long long n_carry = 0, prev_nc = 0;  // cube entries carried into the slab; the last slab's count
  int cur = 0;                         // cube list of this slab (the other takes the carry)
  int prevL = 0;
  // phase timing (qjg_set_timing): events mev[0..4] bracket the phases of a slab
  const bool timed = ctx->timing;
  auto mark = [&](int k) -> cudaError_t {
    return timed ? cudaEventRecord(ctx->mev[k], s) : cudaSuccess;
  };
  auto span = [&](int a, int b, double* acc) -> cudaError_t {
    if (!timed) return cudaSuccess;
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(ctx->mev[b]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ctx->mev[a], ctx->mev[b]);
    *acc += ms;
    return e;
  };
  for (int c0 = 0; c0 < Z - 1;) {
    const int c1 = std::min(c0 + nz, Z - 1);
    const bool last = c1 == Z - 1;
    const int L = c1 - c0;
    // field planes [c0, c1]
    const double* src;
    QJ_CUDA(ctx, mark(0));
    if (streaming) {
      qjg_field_stats fs;
      if (c0 == 0) {
        if ((rc = qjg_field(ctx, rs, grid, iter, 0, c1 + 1, ctx->m_field, nullptr, s))) return rc;
      } else {
        QJ_CUDA(ctx, cudaMemcpyAsync(ctx->m_field, ctx->m_field + (size_t)prevL * XY,
                                     XY * sizeof(double), cudaMemcpyDeviceToDevice, s));
        if ((rc = qjg_field(ctx, rs, grid, iter, c0 + 1, c1 + 1, ctx->m_field + XY, nullptr, s)))
          return rc;
      }
      if ((rc = qjg_field_stats_read(ctx, s, &fs))) return rc;
      if (timed) {
        float ms_bulk = 0.f, ms_rest = 0.f;
        if ((rc = qjg_last_timings(ctx, &ms_bulk, &ms_rest))) return rc;
        st.ms_field_bulk += ms_bulk;
      }
      st.field.voxels += fs.voxels;
      st.field.voxel_iters += fs.voxel_iters;
      st.field.root_terms += fs.root_terms;
      st.field.refined += fs.refined;
      st.field.refined_iters += fs.refined_iters;
      st.field.nonfinite += fs.nonfinite;
      st.field.lane_iters += fs.lane_iters;
      st.field.rerun += fs.rerun;
      st.field.rerun_iters += fs.rerun_iters;
      src = ctx->m_field;
    } else {
      src = d_field + (size_t)c0 * XY;
    }
    // carry the vertex ids and masks of plane c0-1 into window plane 0
    if (c0 > 0) {
      QJ_CUDA(ctx, cudaMemcpyAsync(ctx->m_masks, ctx->m_masks + (size_t)prevL * XY, XY,
                                   cudaMemcpyDeviceToDevice, s));
      QJ_CUDA(ctx, cudaMemcpyAsync(ctx->m_vbase, ctx->m_vbase + (size_t)prevL * XY,
                                   XY * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    }
    // classify voxel planes [c0, c1) (+ Z-1 on the last slab) from field planes [c0, c1]
    QJ_CUDA(ctx, mark(1));
    const int P = L + 1, Pv = L + (last ? 1 : 0);
    QJ_CUDA(ctx, qj::mesh_classify(w, src, P, Pv, c0, s));
    ctx->launches += 4;
    qj::McTotals tot;
    QJ_CUDA(ctx, cudaMemcpyAsync(&tot, ctx->m_tot, sizeof tot, cudaMemcpyDeviceToHost, s));
    QJ_CUDA(ctx, cudaStreamSynchronize(s));
    // the previous slab's last cube layer (its split is still in tot) and
    // the triangles of the previous slab's cubes
    n_carry = c0 > 0 ? prev_nc - tot.split : 0;
    if (c0 > 0) nt += tot.nt;
    const long long n_new = tot.nv, nc = tot.nc;
    if (nv + n_new > INT32_MAX)
      return fail(ctx, QJG_ERR_CAPACITY, "more than 2^31 vertices; int32 indices cannot hold them");
    // the edge list grows by half again at least: the per-slab vertex count rises with the surface
    {
      const size_t want = (size_t)std::max<long long>(n_new, 1);
      if ((rc = ensure(ctx, &ctx->m_list, &ctx->m_list_cap,
                       want > ctx->m_list_cap ? std::max(want, ctx->m_list_cap + ctx->m_list_cap / 2)
                                              : want)))
        return rc;
      w.list = ctx->m_list;
    }
    if ((rc = grow_keep(ctx, &ctx->m_cubes[cur], &ctx->m_cubes_cap[cur],
                        (size_t)std::max<long long>(n_carry + nc, 1), (size_t)n_carry, s)) ||
        (rc = grow_keep(ctx, &ctx->m_cubes[cur ^ 1], &ctx->m_cubes_cap[cur ^ 1],
                        (size_t)std::max<long long>(nc, 1), 0, s)))
      return rc;
    const long long u_split = last ? -1 : (long long)(L - 1) * Y * S;
    QJ_CUDA(ctx, qj::mesh_emit(w, src, P, Pv, c0, u_split, nv, ctx->m_cubes[cur] + n_carry, s));
    if (ctx->m_capture && (rc = capture_slab(ctx, w.list, n_new, ctx->m_cubes[cur] + n_carry, nc,
                                             X, Y, c0, s)))
      return rc;
    // the cube scan's block sums (one per scan block of cubes, and the
    // total) outgrow the unit scan's when a slab has many triangle-bearing
    // cubes per unit; emit has read the unit sums once the stream is synced
    if ((size_t)qj::mesh_scan_blocks(nc) > ctx->m_bsum_cap) {
      if ((rc = grow_keep(ctx, &ctx->m_bsum, &ctx->m_bsum_cap,
                          (size_t)qj::mesh_scan_blocks(nc), 0, s)))
        return rc;
      w.bsum = ctx->m_bsum;
    }
    QJ_CUDA(ctx, qj::mesh_cube_scan(w, ctx->m_cubes[cur] + n_carry, nc, nt, s));
    ctx->launches += nc > 0 ? 4 : 1;
    // per-vertex buffers grow to the vertex count extrapolated from the layers
    // meshed so far (+25%; at most 4x the count so far, and no more than the
    // caller's vertex capacity), so that a large mesh reallocates (cudaMalloc,
    // copy, cudaFree) a few times instead of once per slab
    const double need = (double)(nv + n_new);
    double vh = std::min(need * (Z - 1) / c1 * 1.25, 4.0 * need);
    if (vcap > 0) vh = std::min(vh, std::max((double)vcap, need));
    const size_t vhint = (size_t)vh + 1;
    if ((rc = grow_keep(ctx, &ctx->m_verts, &ctx->m_verts_cap, (size_t)(nv + n_new) * 3,
                        (size_t)nv * 3, s, vhint * 3)))
      return rc;
    QJ_CUDA(ctx, mark(2));
    // FP32-first bisection unless the plain FP64 form is asked for
    const bool hybrid = iter && iter->precision != QJG_FP64;
    qj::EdgeScratch esc{};
    const bool parked = hybrid && bisect && n_new > 0;
    if (parked) {
      // edge states by global vertex id; parked ids accumulate over slabs
      const size_t eb = qj::mesh_edge_state_bytes();
      if ((rc = grow_keep(ctx, &ctx->m_estate, &ctx->m_estate_cap, (size_t)(nv + n_new) * eb,
                          (size_t)nv * eb, s, vhint * eb)) ||
          (rc = grow_keep(ctx, &ctx->m_epark, &ctx->m_epark_cap, (size_t)(nv + n_new),
                          (size_t)nv, s, vhint)))
        return rc;
      esc.state = ctx->m_estate;
      esc.list[0] = ctx->m_epark;
      esc.count = ctx->m_ecount;
    }
    QJ_CUDA(ctx, qj::mesh_vertices(*m, g, it, edge_mode, pow_mode, hybrid, w, n_new, nv, c0, src,
                                   ctx->m_verts, iso, ctx->d_mstats, parked ? &esc : nullptr, s));
    if (n_new) ctx->launches++;
    nv += n_new;
    QJ_CUDA(ctx, mark(3));
    // triangles of cube layers [c0-1, c1-1) (+ c1-1 on the last slab); the
    // entries of layer c1-1 move to the other list for the next slab
    QJ_CUDA(ctx, qj::mesh_triangles(w, ctx->m_cubes[cur], n_carry, nc, last, c0 - 1,
                                    ctx->m_cubes[cur ^ 1], tris, tcap, s));
    ctx->launches += 2;
    QJ_CUDA(ctx, mark(4));
    QJ_CUDA(ctx, span(0, 1, &st.ms_field));
    QJ_CUDA(ctx, span(1, 2, &st.ms_classify));
    QJ_CUDA(ctx, span(2, 3, &st.ms_vertices));
    QJ_CUDA(ctx, span(3, 4, &st.ms_triangles));
    prev_nc = nc;
    prevL = L;
    cur ^= 1;
    st.slabs++;
    c0 = c1;
  }

  // the triangles of the last slab's cubes
  if (st.slabs > 0) {
    long long nt_last = 0;
    QJ_CUDA(ctx, cudaMemcpyAsync(&nt_last, &ctx->m_tot->nt, sizeof nt_last, cudaMemcpyDeviceToHost, s));
    QJ_CUDA(ctx, cudaStreamSynchronize(s));
    nt += nt_last;
  }
  // the parked edges of every slab, resolved together
  const bool any_parked = iter && iter->precision != QJG_FP64 && bisect && nv > 0;
  if (any_parked) {
    QJ_CUDA(ctx, mark(0));
    if ((rc = grow_keep(ctx, &ctx->m_epark, &ctx->m_epark_cap, (size_t)(3 * nv), (size_t)nv, s)))
      return rc;
    qj::EdgeScratch esc{};
    esc.state = ctx->m_estate;
    esc.list[0] = ctx->m_epark;
    esc.list[1] = ctx->m_epark + nv;
    esc.list[2] = ctx->m_epark + 2 * nv;
    esc.count = ctx->m_ecount;
    QJ_CUDA(ctx, qj::mesh_parked_finish(*m, g, it, pow_mode, ctx->m_verts, iso, ctx->d_mstats, esc,
                                        s));
    QJ_CUDA(ctx, mark(1));
    QJ_CUDA(ctx, span(0, 1, &st.ms_vertices));
  }
  st.n_verts = nv;
  st.n_tris = nt;
  qj::DevStats ds;
  QJ_CUDA(ctx, cudaMemcpyAsync(&ds, ctx->d_mstats, sizeof ds, cudaMemcpyDeviceToHost, s));
  QJ_CUDA(ctx, cudaStreamSynchronize(s));
  st.map_evals = (int64_t)ds.aux[1];
  st.n_unbracketed = (int64_t)ds.aux[2];
  st.map_evals_fp32 = (int64_t)ds.aux[3];
  st.map_evals_ff = (int64_t)ds.ff_evals;
  if (nt > tcap || ((v64 || v32) && nv > vcap)) {
    if (out) *out = st;
    return fail(ctx, QJG_ERR_CAPACITY, "mesh needs %lld vertices / %lld triangles (capacity %lld / %lld)",
                nv, nt, (long long)vcap, (long long)tcap);
  }
  // degenerate filter (needs every vertex, so it runs after the last slab)
  if ((rc = ensure(ctx, &ctx->m_tris, &ctx->m_tris_cap, (size_t)std::max<long long>(nt * 3, 1))) ||
      (rc = ensure(ctx, &ctx->m_bsum, &ctx->m_bsum_cap, (size_t)qj::mesh_scan_blocks(nt))))
    return rc;
  long long keep = 0;
  QJ_CUDA(ctx, mark(0));
  QJ_CUDA(ctx, qj::mesh_filter(tris, nt, ctx->m_verts, ctx->m_tris, ctx->m_bsum, &keep, s));
  if (nt) ctx->launches += 3;
  QJ_CUDA(ctx, cudaMemcpyAsync(tris, ctx->m_tris, (size_t)keep * 3 * sizeof(int32_t),
                               cudaMemcpyDeviceToDevice, s));
  st.n_degenerate = nt - keep;
  st.n_tris = keep;
  if (v64)
    QJ_CUDA(ctx, cudaMemcpyAsync(v64, ctx->m_verts, (size_t)nv * 3 * sizeof(double),
                                 cudaMemcpyDeviceToDevice, s));
  if (v32) {
    QJ_CUDA(ctx, qj::mesh_to_float(ctx->m_verts, v32, nv * 3, s));
    if (nv) ctx->launches++;
  }
  QJ_CUDA(ctx, mark(1));
  QJ_CUDA(ctx, cudaStreamSynchronize(s));
  QJ_CUDA(ctx, span(0, 1, &st.ms_filter));
  if (out) *out = st;
  return QJG_OK;
}

// Slab depth of the streaming mesher for a grid (mesh_core's rule).
long long slab_depth(const qjg_grid* grid, int slab_nz) {
  const long long XY = (long long)grid->res[0] * grid->res[1];
  int nz = slab_nz > 0 ? slab_nz : 64;
  const long long nz_max = (long long)(UINT32_MAX / 4) / XY - 2;
  if (nz_max < 1) return 0;
  nz = (int)std::min<long long>(nz, nz_max);
  return std::max(1, std::min(nz, std::max(grid->res[2] - 1, 1)));
}

// Buffer sizes of the fixed launch sequence.
struct RunCaps {
  long long list, cubes, bsum, field_vox;
};
RunCaps run_caps(long long X, long long Y, long long nz, int64_t vcap, int64_t tcap) {
  const long long XY = X * Y;
  RunCaps c;
  c.list = std::max<long long>(1, std::min<long long>(vcap, 3 * XY * (nz + 1)));
  c.cubes = std::max<long long>(1, std::min<long long>(tcap, XY * (nz + 1)));
  const long long units = qj::mesh_units((int)X, (int)Y, (int)nz + 1);
  c.bsum = std::max({2 * qj::mesh_scan_blocks(units), qj::mesh_scan_blocks(c.cubes),
                     qj::mesh_scan_blocks(std::max<long long>(tcap, 1))});
  c.field_vox = (nz + 1) * XY;
  return c;
}

// The streaming mesher as a fixed launch sequence: every count stays on the
// device (McRun), so nothing between the kernels reads the host or waits.
int mesh_core_async(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
                    double iso, int slab_nz, double* v64, float* v32, int64_t vcap,
                    int32_t* tris, int64_t tcap, cudaStream_t s) {
  int rc;
  if ((rc = qj_check_grid(ctx, grid))) return rc;
  const MapParams* m = qj_lookup(ctx, rs);
  if (!m) return fail(ctx, QJG_ERR_HANDLE, "unknown root set %d", rs);
  if ((rc = qj_check_iter(ctx, iter))) return rc;
  std::unique_ptr<MapParams> mcopy;
  if (iter->form == QJG_FORM_LAGRANGE) {
    mcopy.reset(new MapParams(*m));
    mcopy->lagrange = 1;
    m = mcopy.get();
  }
  if (!tris || vcap <= 0 || tcap <= 0)
    return fail(ctx, QJG_ERR_ARG, "the fixed sequence needs d_tris and positive capacities");
  const int X = grid->res[0], Y = grid->res[1], Z = grid->res[2];
  const long long XY = (long long)X * Y;
  const long long nz = slab_depth(grid, slab_nz);
  if (nz < 1) return fail(ctx, QJG_ERR_ARG, "a %d x %d slice is too large", X, Y);
  if (!ctx->m_run || X > ctx->m_prep_X || Y > ctx->m_prep_Y || XY > ctx->m_prep_X * ctx->m_prep_Y ||
      nz > ctx->m_prep_nz || vcap > ctx->m_prep_vcap || tcap > ctx->m_prep_tcap)
    return fail(ctx, QJG_ERR_ARG, "qjg_mesh_prepare has not sized this context for the mesh");
  const RunCaps caps = run_caps(X, Y, nz, vcap, tcap);
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  QJ_CUDA(ctx, qj::mesh_run_init(ctx->m_run, vcap, caps.list, caps.cubes, tcap, s));
  ctx->m_async_slabs = 0;
  if (X < 2 || Y < 2) {  // no cube
    QJ_CUDA(ctx, qj::mesh_run_final(ctx->m_run, ctx->m_tot, false, s));
    return QJG_OK;
  }
  QJ_CUDA(ctx, cudaMemsetAsync(ctx->d_mstats, 0, sizeof(qj::DevStats), s));
  QJ_CUDA(ctx, cudaMemsetAsync(ctx->m_fstats, 0, sizeof(qj::DevStats), s));
  QJ_CUDA(ctx, cudaMemsetAsync(ctx->m_ecount, 0, 3 * sizeof(unsigned long long), s));
  qj::MeshWindow w;
  w.X = X;
  w.Y = Y;
  w.masks = ctx->m_masks;
  w.vbase = ctx->m_vbase;
  w.list = ctx->m_list;
  w.bsum = ctx->m_bsum;
  w.bits = ctx->m_bits;
  w.sign = ctx->m_sign;
  w.ucount = ctx->m_ucount;
  w.tot = ctx->m_tot;
  const GridParams g = qj_grid_params(grid, 0, Z);
  const IterParams it = qj_iter_params(iter, grid);
  const int pow_mode = qj_pow_mode(iter, m->all_int);
  const bool hybrid = iter->precision != QJG_FP64;
  const long long S = (X + 63) / 64;
  qj::EdgeScratch esc{};
  esc.state = ctx->m_estate;
  esc.list[0] = ctx->m_epark;
  esc.list[1] = ctx->m_epark + vcap;
  esc.list[2] = ctx->m_epark + 2 * vcap;
  esc.count = ctx->m_ecount;
  int cur = 0, prevL = 0, slabs = 0;
  for (int c0 = 0; c0 < Z - 1;) {
    const int c1 = (int)std::min<long long>(c0 + nz, Z - 1);
    const bool last = c1 == Z - 1;
    const int L = c1 - c0;
    if (c0 == 0) {
      if ((rc = qjg_field(ctx, rs, grid, iter, 0, c1 + 1, ctx->m_field, nullptr, s))) return rc;
    } else {
      QJ_CUDA(ctx, cudaMemcpyAsync(ctx->m_field, ctx->m_field + (size_t)prevL * XY,
                                   XY * sizeof(double), cudaMemcpyDeviceToDevice, s));
      if ((rc = qjg_field(ctx, rs, grid, iter, c0 + 1, c1 + 1, ctx->m_field + XY, nullptr, s)))
        return rc;
      QJ_CUDA(ctx, cudaMemcpyAsync(ctx->m_masks, ctx->m_masks + (size_t)prevL * XY, XY,
                                   cudaMemcpyDeviceToDevice, s));
      QJ_CUDA(ctx, cudaMemcpyAsync(ctx->m_vbase, ctx->m_vbase + (size_t)prevL * XY,
                                   XY * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    }
    QJ_CUDA(ctx, qj::mesh_stats_add(ctx->m_fstats, ctx->d_stats, s));
    const double* src = ctx->m_field;
    const int P = L + 1, Pv = L + (last ? 1 : 0);
    QJ_CUDA(ctx, qj::mesh_classify(w, src, P, Pv, c0, s));
    QJ_CUDA(ctx, qj::mesh_run_slab(ctx->m_run, w.tot, c0 == 0, s));
    const long long u_split = last ? -1 : (long long)(L - 1) * Y * S;
    QJ_CUDA(ctx, qj::mesh_emit_run(w, src, P, Pv, c0, u_split, ctx->m_cubes[cur], ctx->m_run, s));
    QJ_CUDA(ctx, qj::mesh_cube_scan_run(w, ctx->m_cubes[cur], ctx->m_run, caps.cubes, s));
    QJ_CUDA(ctx, qj::mesh_vertices_run(*m, g, it, QJG_EDGE_BISECT, pow_mode, hybrid, w, c0, src,
                                       ctx->m_verts, iso, ctx->d_mstats, hybrid ? &esc : nullptr,
                                       ctx->m_run, s));
    QJ_CUDA(ctx, qj::mesh_run_next(ctx->m_run, s));
    QJ_CUDA(ctx, qj::mesh_triangles_run(w, ctx->m_cubes[cur], last, c0 - 1, ctx->m_cubes[cur ^ 1],
                                        tris, tcap, ctx->m_run, s));
    ctx->launches += 12;
    prevL = L;
    cur ^= 1;
    slabs++;
    c0 = c1;
  }
  QJ_CUDA(ctx, qj::mesh_run_final(ctx->m_run, w.tot, slabs > 0, s));
  if (hybrid)
    QJ_CUDA(ctx, qj::mesh_parked_finish_fixed(*m, g, it, pow_mode, ctx->m_verts, iso,
                                              ctx->d_mstats, esc, s));
  QJ_CUDA(ctx, qj::mesh_filter_run(tris, ctx->m_verts, ctx->m_tris, ctx->m_bsum, ctx->m_run, tcap, s));
  QJ_CUDA(ctx, qj::mesh_copy_out_run(ctx->m_verts, v64, v32, ctx->m_tris, tris, ctx->m_run, s));
  ctx->launches += hybrid ? 30 : 6;
  ctx->m_async_slabs = slabs;
  ctx->m_async_voxels = slabs > 0 ? (int64_t)Z * XY : 0;  // every plane computed once
  ctx->m_async_roots = m->nt + m->nb;
  return QJG_OK;
}

}  // namespace

extern "C" {

int qjg_mesh_field(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
                   const double* d_field, int32_t edge_mode, double iso, int32_t slab_nz,
                   double* d_verts64, float* d_verts32, int64_t vert_cap, int32_t* d_tris,
                   int64_t tri_cap, qjg_mesh_stats* stats, void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  return mesh_core(ctx, rs, grid, iter, false, d_field, edge_mode, iso, slab_nz, d_verts64,
                   d_verts32, vert_cap, d_tris, tri_cap, stats, (cudaStream_t)stream);
}

int qjg_mesh_stream(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, const qjg_iter* iter,
                    double iso, int32_t slab_nz, double* d_verts64, float* d_verts32,
                    int64_t vert_cap, int32_t* d_tris, int64_t tri_cap, qjg_mesh_stats* stats,
                    void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  return mesh_core(ctx, rs, grid, iter, true, nullptr, QJG_EDGE_BISECT, iso, slab_nz, d_verts64,
                   d_verts32, vert_cap, d_tris, tri_cap, stats, (cudaStream_t)stream);
}

int qjg_mesh_prepare(qjg_ctx* ctx, const qjg_grid* grid, int32_t slab_nz, int64_t vert_cap,
                     int64_t tri_cap) {
  if (!ctx) return QJG_ERR_ARG;
  int rc;
  if ((rc = qj_check_grid(ctx, grid))) return rc;
  if (vert_cap <= 0 || tri_cap <= 0) return fail(ctx, QJG_ERR_ARG, "capacities must be positive");
  const long long X = grid->res[0], Y = grid->res[1], XY = X * Y;
  const long long nz = slab_depth(grid, slab_nz);
  if (nz < 1) return fail(ctx, QJG_ERR_ARG, "a %lld x %lld slice is too large", X, Y);
  const RunCaps caps = run_caps(X, Y, nz, vert_cap, tri_cap);
  const size_t wplanes = (size_t)(nz + 2) * XY;
  const long long units = qj::mesh_units((int)X, (int)Y, (int)nz + 1);
  const size_t fv = (size_t)caps.field_vox;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  if ((rc = ensure(ctx, &ctx->m_masks, &ctx->m_masks_cap, wplanes)) ||
      (rc = ensure(ctx, &ctx->m_vbase, &ctx->m_vbase_cap, wplanes)) ||
      (rc = ensure(ctx, &ctx->m_sign, &ctx->m_sign_cap, (size_t)units * qj::MESH_UNIT_WORDS)) ||
      (rc = ensure(ctx, &ctx->m_bits, &ctx->m_bits_cap, (size_t)units * qj::MESH_UNIT_WORDS)) ||
      (rc = ensure(ctx, &ctx->m_ucount, &ctx->m_ucount_cap, (size_t)units)) ||
      (rc = ensure(ctx, &ctx->m_tot, &ctx->m_tot_cap, (size_t)1)) ||
      (rc = ensure(ctx, &ctx->m_bsum, &ctx->m_bsum_cap, (size_t)caps.bsum)) ||
      (rc = ensure(ctx, &ctx->m_field, &ctx->m_field_cap, fv)) ||
      (rc = ensure(ctx, &ctx->d_list, &ctx->list_cap, fv)) ||
      (rc = ensure(ctx, &ctx->d_sorted, &ctx->sorted_cap, fv)) ||
      (rc = ensure(ctx, &ctx->d_keys, &ctx->keys_cap, fv)) ||
      (rc = ensure(ctx, &ctx->d_hist, &ctx->hist_cap, (size_t)qj::REFINE_KEYS)) ||
      (rc = ensure(ctx, &ctx->d_ff, &ctx->ff_cap, fv)) ||
      (rc = ensure(ctx, &ctx->m_ecount, &ctx->m_ecount_cap, (size_t)3)) ||
      (rc = ensure(ctx, &ctx->m_list, &ctx->m_list_cap, (size_t)caps.list)) ||
      (rc = ensure(ctx, &ctx->m_cubes[0], &ctx->m_cubes_cap[0], (size_t)caps.cubes)) ||
      (rc = ensure(ctx, &ctx->m_cubes[1], &ctx->m_cubes_cap[1], (size_t)caps.cubes)) ||
      (rc = ensure(ctx, &ctx->m_verts, &ctx->m_verts_cap, (size_t)(3 * vert_cap))) ||
      (rc = ensure(ctx, &ctx->m_estate, &ctx->m_estate_cap,
                   (size_t)vert_cap * qj::mesh_edge_state_bytes())) ||
      (rc = ensure(ctx, &ctx->m_epark, &ctx->m_epark_cap, (size_t)(3 * vert_cap))) ||
      (rc = ensure(ctx, &ctx->m_tris, &ctx->m_tris_cap, (size_t)(3 * tri_cap))))
    return rc;
  if (!ctx->m_run) QJ_CUDA(ctx, cudaMalloc((void**)&ctx->m_run, sizeof(qj::McRun)));
  if (!ctx->m_fstats) QJ_CUDA(ctx, cudaMalloc((void**)&ctx->m_fstats, sizeof(qj::DevStats)));
  ctx->m_prep_X = X;
  ctx->m_prep_Y = Y;
  ctx->m_prep_nz = nz;
  ctx->m_prep_vcap = vert_cap;
  ctx->m_prep_tcap = tri_cap;
  return QJG_OK;
}

int qjg_mesh_stream_async(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid,
                          const qjg_iter* iter, double iso, int32_t slab_nz, double* d_verts64,
                          float* d_verts32, int64_t vert_cap, int32_t* d_tris, int64_t tri_cap,
                          void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  ctx->m_async_slabs = -1;
  return mesh_core_async(ctx, rs, grid, iter, iso, slab_nz, d_verts64, d_verts32, vert_cap,
                         d_tris, tri_cap, (cudaStream_t)stream);
}

int qjg_mesh_async_result(qjg_ctx* ctx, qjg_mesh_stats* stats) {
  if (!ctx || !stats) return QJG_ERR_ARG;
  if (ctx->m_async_slabs < 0 || !ctx->m_run)
    return fail(ctx, QJG_ERR_ARG, "no qjg_mesh_stream_async run to read");
  qj::McRun run;
  qj::DevStats ds, fs;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  QJ_CUDA(ctx, cudaMemcpy(&run, ctx->m_run, sizeof run, cudaMemcpyDeviceToHost));
  std::memset(&ds, 0, sizeof ds);
  std::memset(&fs, 0, sizeof fs);
  if (ctx->m_async_slabs > 0) {
    QJ_CUDA(ctx, cudaMemcpy(&ds, ctx->d_mstats, sizeof ds, cudaMemcpyDeviceToHost));
    QJ_CUDA(ctx, cudaMemcpy(&fs, ctx->m_fstats, sizeof fs, cudaMemcpyDeviceToHost));
  }
  qjg_mesh_stats st;
  std::memset(&st, 0, sizeof st);
  st.n_verts = run.nv;
  st.n_tris = run.keep;
  st.n_degenerate = run.overflow ? 0 : run.nt - run.keep;
  st.slabs = ctx->m_async_slabs;
  st.map_evals = (int64_t)ds.aux[1];
  st.n_unbracketed = (int64_t)ds.aux[2];
  st.map_evals_fp32 = (int64_t)ds.aux[3];
  st.map_evals_ff = (int64_t)ds.ff_evals;
  // the slab fields' counters, as qjg_field_stats_read reads them
  st.field.voxels = ctx->m_async_voxels;
  st.field.voxel_iters = (int64_t)fs.voxel_iters;
  st.field.root_terms = (int64_t)fs.voxel_iters * ctx->m_async_roots;
  st.field.refined = (int64_t)fs.refined;
  st.field.refined_iters = (int64_t)fs.aux[0];
  st.field.nonfinite = (int64_t)fs.nonfinite;
  st.field.lane_iters = (int64_t)fs.aux[3];
  st.field.rerun = (int64_t)fs.rerun;
  st.field.rerun_iters = (int64_t)fs.rerun_iters;
  *stats = st;
  if (run.overflow)
    return fail(ctx, QJG_ERR_CAPACITY, "the mesh outgrew the capacities of the fixed sequence");
  return QJG_OK;
}

int qjg_mesh_capture(qjg_ctx* ctx, int32_t on) {
  if (!ctx) return QJG_ERR_ARG;
  ctx->m_capture = on != 0;
  return QJG_OK;
}

int qjg_mesh_edge_cache_write(qjg_ctx* ctx, const char* path) {
  if (!ctx || !path) return QJG_ERR_ARG;
  if (!ctx->m_capture) return fail(ctx, QJG_ERR_ARG, "edge capture is off (qjg_mesh_capture)");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(ctx, QJG_ERR_ARG, "cannot write %s", path);
  const int32_t ne = (int32_t)(ctx->cap_edges.size() / 6), nc = (int32_t)(ctx->cap_cubes.size() / 4);
  bool ok = std::fwrite(&ne, sizeof ne, 1, f) == 1 &&
            std::fwrite(ctx->cap_edges.data(), sizeof(int32_t), ctx->cap_edges.size(), f) ==
                ctx->cap_edges.size() &&
            std::fwrite(&nc, sizeof nc, 1, f) == 1 &&
            std::fwrite(ctx->cap_cubes.data(), sizeof(int32_t), ctx->cap_cubes.size(), f) ==
                ctx->cap_cubes.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? QJG_OK : fail(ctx, QJG_ERR_ARG, "short write to %s", path);
}

int qjg_mesh_edge_cache_read(const char* path, int32_t* edges, int64_t edge_cap, int64_t* n_edges,
                             int32_t* cubes, int64_t cube_cap, int64_t* n_cubes) {
  if (!path || !n_edges || !n_cubes) return QJG_ERR_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return QJG_ERR_ARG;
  int32_t ne = 0, nc = 0;
  int rc = QJG_OK;
  if (std::fread(&ne, sizeof ne, 1, f) != 1 || ne < 0) rc = QJG_ERR_ARG;
  std::vector<int32_t> e(rc ? 0 : (size_t)ne * 6);
  if (!rc && std::fread(e.data(), sizeof(int32_t), e.size(), f) != e.size()) rc = QJG_ERR_ARG;
  if (!rc && (std::fread(&nc, sizeof nc, 1, f) != 1 || nc < 0)) rc = QJG_ERR_ARG;
  std::vector<int32_t> c(rc ? 0 : (size_t)nc * 4);
  if (!rc && std::fread(c.data(), sizeof(int32_t), c.size(), f) != c.size()) rc = QJG_ERR_ARG;
  std::fclose(f);
  if (rc) return rc;
  *n_edges = ne;
  *n_cubes = nc;
  if ((edges && edge_cap < ne) || (cubes && cube_cap < nc)) return QJG_ERR_CAPACITY;
  if (edges) std::memcpy(edges, e.data(), e.size() * sizeof(int32_t));
  if (cubes) std::memcpy(cubes, c.data(), c.size() * sizeof(int32_t));
  return QJG_OK;
}

}  // extern "C"
