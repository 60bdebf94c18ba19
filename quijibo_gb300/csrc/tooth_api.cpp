// C ABI of toothOptimizer's fits: BLMVM (blmvm.cpp) over the tanh score,
// each objective evaluation one GPU pass of the score and its analytic
// gradients (energy.cu, tanh_grad_kernel).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <functional>
#include <vector>

#include "qj_blmvm.h"
#include "qj_conformal.h"
#include "qj_ctx.h"
#include "qj_energy.h"

namespace {

// The solver's variables <-> the map state, in the layouts of
// FormScaledOnlyFunctionGradient ([log s, sigma_t, sigma_b]) and
// FormScaledFunctionGradient ([log s, bottom exps, top exps, sigma_t,
// sigma_b]) (toothOptimizer.cpp:65-130).
struct FitLayout {
  int mode, nt, nb;
  int n() const { return mode == QJG_FIT_SCALED_ONLY ? 3 : 3 + nt + nb; }

  void to_vars(const qjg_map_state& st, double* x) const {
    x[0] = std::log(st.scale);
    if (mode == QJG_FIT_SCALED_ONLY) {
      x[1] = st.sigma_top;
      x[2] = st.sigma_bot;
      return;
    }
    int k = 1;
    for (int i = 0; i < nb; i++) x[k++] = st.bot_powers[i];
    for (int i = 0; i < nt; i++) x[k++] = st.top_powers[i];
    x[k++] = st.sigma_top;
    x[k] = st.sigma_bot;
  }

  // scale = exp(x0) as the callbacks set _expScaling
  void from_vars(const double* x, qjg_map_state& st, double* tp, double* bp) const {
    st.scale = std::exp(x[0]);
    if (mode == QJG_FIT_SCALED_ONLY) {
      st.sigma_top = x[1];
      st.sigma_bot = x[2];
      return;
    }
    int k = 1;
    for (int i = 0; i < nb; i++) bp[i] = x[k++];
    for (int i = 0; i < nt; i++) tp[i] = x[k++];
    st.sigma_top = x[k++];
    st.sigma_bot = x[k];
  }

  // the kernel's gradient [d log s, bottom, top, sigma_t, sigma_b] -> the
  // variables' gradient
  void grad(const double* full, double* g) const {
    if (mode == QJG_FIT_SCALED_ONLY) {
      g[0] = full[0];
      g[1] = full[1 + nb + nt];
      g[2] = full[2 + nb + nt];
      return;
    }
    for (int i = 0; i < 3 + nt + nb; i++) g[i] = full[i];
  }
};

}  // namespace

extern "C" {

int qjg_tanh_fit(qjg_ctx* ctx, int32_t mode, qjg_map_state* state, const qjg_grid* grid,
                 int32_t max_it, const qjg_grid* weight_grid, const double* d_weights, double alpha,
                 double threshold, const qjg_blmvm_settings* settings, qjg_monitor_fn monitor,
                 void* monitor_user, double* d_field, qjg_blmvm_stats* stats, void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  if (mode != QJG_FIT_SCALED_ONLY && mode != QJG_FIT_SCALED)
    return fail(ctx, QJG_ERR_ARG, "unknown fit mode %d", mode);
  if (!state || !d_weights) return fail(ctx, QJG_ERR_ARG, "NULL state or weights");
  const int nt = state->n_top, nb = state->n_bot;
  if (nt < 1 || nb < 0 || nt + nb > QJG_MAX_ROOTS)
    return fail(ctx, QJG_ERR_ARG, "root counts top=%d bottom=%d", nt, nb);
  if (!state->top_roots || !state->top_powers || (nb > 0 && (!state->bot_roots || !state->bot_powers)))
    return fail(ctx, QJG_ERR_ARG, "NULL roots or powers");
  if (!(state->scale > 0)) return fail(ctx, QJG_ERR_ARG, "scale %g is not > 0", state->scale);
  int rc;
  if ((rc = qj_check_grid(ctx, grid)) || (rc = qj_check_grid(ctx, weight_grid))) return rc;
  if (max_it < 0) return fail(ctx, QJG_ERR_ARG, "max_it = %d < 0", max_it);
  qj::blmvm::Settings st;
  if (settings) st = qj::blmvm::settings_from(*settings);
  if (st.max_it < 0 || st.ls_max_funcs < 1) return fail(ctx, QJG_ERR_ARG, "bad solver settings");
  cudaStream_t s = (cudaStream_t)stream;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));

  const FitLayout lay{mode, nt, nb};
  const int n = lay.n();
  const qj::GridParams g = qj_grid_params(grid, 0, grid->res[2]);
  const qj::WeightGrid wg = qj_weight_grid(weight_grid);
  const int nblocks = qj::tanh_blocks();
  const int slots = qj::tanh_slots(nt, nb);
  double* d_part = nullptr;
  QJ_CUDA(ctx, qj_malloc_async(ctx, &d_part, sizeof(double) * ((size_t)nblocks + 1) * slots, s));
  double* d_out = d_part + (size_t)nblocks * slots;
  double* h_out = nullptr;
  if (cudaMallocHost((void**)&h_out, sizeof(double) * slots) != cudaSuccess) {
    cudaFreeAsync(d_part, s);
    return fail(ctx, QJG_ERR_NOMEM, "no pinned memory for the fit");
  }

  // working copies of the exponents: the state is written back at the end
  std::vector<double> tp(state->top_powers, state->top_powers + nt);
  std::vector<double> bp(state->bot_powers, state->bot_powers + nb);
  qjg_map_state cur = *state;
  qj::MapParams m;
  std::vector<double> x(n), lo(n, 0.0), hi(n, (double)FLT_MAX);
  lo[0] = -(double)FLT_MAX;
  lay.to_vars(*state, x.data());

  int cuda_failed = 0;
  qj::MapParams m_last;  // the last evaluation's map, whose field d_field gets
  bool evaluated = false;
  qj::blmvm::Objective obj = [&](const double* xv, double* f, double* gv) -> int {
    lay.from_vars(xv, cur, tp.data(), bp.data());
    if (qj_fill_map(&m, nt, cur.top_roots, tp.data(), cur.sigma_top, nb, cur.bot_roots, bp.data(),
                    cur.sigma_bot, cur.scale) >= 0) {
      // an exponent overflowed: the reference's score is then not finite
      *f = NAN;
      for (int i = 0; i < n; i++) gv[i] = NAN;
      return 0;
    }
    // no field during the solve; d_field is filled once at the end
    cudaError_t e = qj::launch_tanh_grad(m, g, wg, d_weights, max_it, alpha, threshold, true,
                                         nullptr, d_part, nblocks, d_out, s);
    m_last = m;
    evaluated = true;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_out, d_out, sizeof(double) * slots, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cuda_failed = 1;
      fail(ctx, QJG_ERR_CUDA, "tanh fit: %s", cudaGetErrorString(e));
      return QJG_ERR_CUDA;
    }
    ctx->launches += 3;
    *f = h_out[3 + nt + nb];
    lay.grad(h_out, gv);
    return 0;
  };
  qj::blmvm::Monitor mon;
  if (monitor)
    mon = [&](int it, double f, double gn, const double* xv) {
      return monitor(monitor_user, it, f, gn, xv);
    };
  qj::blmvm::Stats bs;
  rc = qj::blmvm::minimize(n, x.data(), lo.data(), hi.data(), obj, mon, st, bs);
  if (!rc && d_field && evaluated) {
    // OPTIMIZE_3D::_fractal: the field of the last evaluation
    cudaError_t e = qj::launch_tanh_grad(m_last, g, wg, d_weights, max_it, alpha, threshold, true,
                                         d_field, d_part, nblocks, d_out, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cuda_failed = 1;
      rc = fail(ctx, QJG_ERR_CUDA, "tanh fit field: %s", cudaGetErrorString(e));
    }
    ctx->launches += 3;
  }
  cudaFreeAsync(d_part, s);
  cudaStreamSynchronize(s);
  cudaFreeHost(h_out);
  if (stats) qj::blmvm::stats_to(bs, stats);
  if (rc) return cuda_failed ? QJG_ERR_CUDA : rc;
  // the callers' copy-back (toothOptimizer.cpp:162-164, 213-222)
  lay.from_vars(x.data(), *state, tp.data(), bp.data());
  for (int i = 0; i < nt; i++) state->top_powers[i] = tp[i];
  for (int i = 0; i < nb; i++) state->bot_powers[i] = bp[i];
  return QJG_OK;
}

int qjg_tanh_max_score(qjg_ctx* ctx, const qjg_grid* grid, const qjg_grid* weight_grid,
                       const double* d_weights, double* out, void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  int rc;
  if ((rc = qj_check_grid(ctx, grid)) || (rc = qj_check_grid(ctx, weight_grid))) return rc;
  if (!d_weights || !out) return fail(ctx, QJG_ERR_ARG, "NULL weights or output");
  cudaStream_t s = (cudaStream_t)stream;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  const long long n = (long long)grid->res[0] * grid->res[1] * grid->res[2];
  const int nb = qj::conformal_blocks(n);
  double* d_w = nullptr;
  QJ_CUDA(ctx, qj_malloc_async(ctx, &d_w, sizeof(double) * ((size_t)n + 3 * (size_t)nb + 3), s));
  double* part = d_w + n;
  double* sums = part + 3 * (size_t)nb;
  double h[3];
  cudaError_t e = qj::launch_lookup(qj_grid_params(grid, 0, grid->res[2]),
                                    qj_weight_grid(weight_grid), d_weights, d_w, s);
  if (e == cudaSuccess) e = qj::launch_side_sums(d_w, d_w, n, 1.0, part, sums, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, sums, sizeof h, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d_w, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(ctx, QJG_ERR_CUDA, "max score: %s", cudaGetErrorString(e));
  ctx->launches += 3;
  *out = h[0];
  return QJG_OK;
}

}  // extern "C"

// ---- toothOptimizer's run ---------------------------------------------------
namespace {

// device buffer released at scope exit
struct DevBuf {
  double* p = nullptr;
  size_t n = 0;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  bool reserve(size_t want) {
    if (want <= n) return true;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (cudaMalloc((void**)&p, want * sizeof(double)) != cudaSuccess) return false;
    n = want;
    return true;
  }
};

qjg_grid cube_grid(int res, const double* center, const double* lengths) {
  qjg_grid g = {};
  for (int c = 0; c < 3; c++) {
    g.res[c] = res;
    g.center[c] = center[c];
    g.lengths[c] = lengths[c];
  }
  g.rot[0] = 1.0;
  return g;
}

struct ToothRun {
  qjg_ctx* ctx;
  cudaStream_t s;
  const qjg_tooth_config* cfg;
  qjg_o3d_info info;  // header of the input; rewritten for every state file
  std::vector<double> troots, tpow, broots, bpow;
  double sig_t = 1, sig_b = 1, scale = 1;
  std::vector<double> h_dist, h_curv;  // distance (fractal frame), curvature (as read)
  qjg_grid dgrid;                      // the distance / weight field's grid
  double fcenter[3], flengths[3];      // the fractal grid's box
  DevBuf d_dist, d_w, d_w2, d_field, d_fd, d_mesh;
  int monitor_calls = 0;
  int level_checkpoints = 0;
  int cur_res = 0;
  int fit_mode = 0;
  qjg_grid cur_grid;               // the running fit's grid and weights
  const double* cur_w = nullptr;

  qjg_map_state state() {
    qjg_map_state m;
    m.n_top = (int)tpow.size();
    m.n_bot = (int)bpow.size();
    m.top_roots = troots.data();
    m.bot_roots = broots.empty() ? nullptr : broots.data();
    m.top_powers = tpow.data();
    m.bot_powers = bpow.empty() ? nullptr : bpow.data();
    m.sigma_top = sig_t;
    m.sigma_bot = sig_b;
    m.scale = scale;
    return m;
  }
  void take(const qjg_map_state& m) {
    sig_t = m.sigma_top;
    sig_b = m.sigma_bot;
    scale = m.scale;
  }

  int with_rootset(const std::function<int(qjg_rootset)>& f) {
    qjg_rootset rs = -1;
    int rc = qjg_rootset_upload(ctx, (int)tpow.size(), troots.data(), tpow.data(), sig_t,
                                (int)bpow.size(), broots.empty() ? nullptr : broots.data(),
                                bpow.empty() ? nullptr : bpow.data(), sig_b, scale, &rs);
    if (rc) return rc;
    rc = f(rs);
    qjg_rootset_free(ctx, rs);
    return rc;
  }

  // OPTIMIZE_3D::write of the current map (OPTIMIZE_3D.cpp:3254-3297): the
  // fractal is the field of the last score evaluation on the level's grid
  int write_state(const char* path, int res) {
    const size_t nf = (size_t)res * res * res;
    std::vector<double> h_field(nf);
    QJ_CUDA(ctx, cudaMemcpyAsync(h_field.data(), d_field.p, nf * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
    QJ_CUDA(ctx, cudaStreamSynchronize(s));
    qjg_o3d_info o = info;
    o.n_top = (int)tpow.size();
    o.n_bot = (int)bpow.size();
    o.sigma_top = sig_t;
    o.sigma_bot = sig_b;
    o.exp_scaling = scale;
    for (int c = 0; c < 3; c++) {
      o.field_res[0][c] = res;
      o.field_center[0][c] = fcenter[c];
      o.field_lengths[0][c] = flengths[c];
      o.field_res[1][c] = o.field_res[2][c] = dgrid.res[c];
      o.field_center[1][c] = o.field_center[2][c] = dgrid.center[c];
      o.field_lengths[1][c] = o.field_lengths[2][c] = dgrid.lengths[c];
      // setScoreFields made the optimizer's resolution and box the distance field's
      o.res[c] = dgrid.res[c];
      o.center[c] = dgrid.center[c];
      o.lengths[c] = dgrid.lengths[c];
    }
    const int rc = qjg_o3d_write(path, &o, troots.data(), tpow.data(),
                                 broots.empty() ? nullptr : broots.data(),
                                 bpow.empty() ? nullptr : bpow.data(), h_field.data(),
                                 h_dist.data(), h_curv.data());
    if (rc) return fail(ctx, QJG_ERR_ARG, "cannot write the state file %s", path);
    return QJG_OK;
  }
};

// the monitor (toothOptimizer.cpp:48-61): a state file on every 10th call of
// the run
int tooth_monitor(void* user, int32_t, double, double, const double* x) {
  ToothRun& r = *static_cast<ToothRun*>(user);
  if (r.monitor_calls++ % 10 != 0 || !r.cfg->checkpoint_path) return 0;
  const FitLayout lay{r.fit_mode, (int)r.tpow.size(), (int)r.bpow.size()};
  qjg_map_state m = r.state();
  std::vector<double> tp(r.tpow), bp(r.bpow);
  lay.from_vars(x, m, tp.data(), bp.data());
  // write the iterate's map, then restore the run's own copy (element-wise:
  // the running fit holds pointers into these arrays)
  std::vector<double> keep_t(r.tpow), keep_b(r.bpow);
  const double ks[3] = {r.sig_t, r.sig_b, r.scale};
  std::copy(tp.begin(), tp.end(), r.tpow.begin());
  std::copy(bp.begin(), bp.end(), r.bpow.begin());
  r.take(m);
  // the fractal of the iterate, as the reference's last evaluation left it
  std::vector<double> g(3 + tp.size() + bp.size());
  double sc = 0;
  int rc = r.with_rootset([&](qjg_rootset rs) {
    return qjg_tanh_score_grad(r.ctx, rs, &r.cur_grid, 1, &r.dgrid, r.cur_w, 10.0, 0.0, &sc,
                               g.data(), r.d_field.p, nullptr, r.s);
  });
  if (!rc) rc = r.write_state(r.cfg->checkpoint_path, r.cur_res);
  std::copy(keep_t.begin(), keep_t.end(), r.tpow.begin());
  std::copy(keep_b.begin(), keep_b.end(), r.bpow.begin());
  r.sig_t = ks[0];
  r.sig_b = ks[1];
  r.scale = ks[2];
  r.level_checkpoints++;
  return rc ? 1 : 0;
}

// computeFractal (toothOptimizer.cpp:240-273): the field at maxIterations 1,
// infinities clamped to the mean, borders set to the cell count, linear
// marching cubes; the mesh goes to the caller's sdf on the distance grid.
int fractal_distance(ToothRun& r, const qjg_grid& fg, int64_t* n_tris) {
  qjg_ctx* ctx = r.ctx;
  const long long n = (long long)fg.res[0] * fg.res[1] * fg.res[2];
  qjg_iter it = {};
  it.max_it = 1;
  it.precision = QJG_FP64;
  it.refine_pow = QJG_REFINE_POW;
  it.escape = 2000.0;
  int rc = r.with_rootset([&](qjg_rootset rs) {
    return qjg_field(ctx, rs, &fg, &it, 0, fg.res[2], r.d_field.p, nullptr, r.s);
  });
  if (rc) return rc;
  // clampInfsToMean (FIELD_3D.cpp:5182-5206)
  const int nb = qj::conformal_blocks(n);
  if (!r.d_mesh.reserve(4 * (size_t)nb)) return fail(ctx, QJG_ERR_NOMEM, "no memory for stats");
  int nblk = 0;
  QJ_CUDA(ctx, qj::launch_field_stats(r.d_field.p, n, r.d_mesh.p, &nblk, r.s));
  std::vector<double> st(4 * (size_t)nblk);
  QJ_CUDA(ctx, cudaMemcpyAsync(st.data(), r.d_mesh.p, st.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, r.s));
  QJ_CUDA(ctx, cudaStreamSynchronize(r.s));
  double sum = 0, cnt = 0;
  for (int b = 0; b < nblk; b++) {
    sum += st[4 * b];
    cnt += st[4 * b + 1];
  }
  QJ_CUDA(ctx, qj::launch_clamp_infs(r.d_field.p, n, sum / cnt, r.s));
  QJ_CUDA(ctx, qj::launch_borders(r.d_field.p, fg.res[0], fg.res[1], fg.res[2], (double)n, r.s));
  // TRIANGLE_MESH(const FIELD_3D&): capacities grown until they suffice
  int64_t vcap = 4 * n + 16, tcap = 8 * n + 16;
  qjg_mesh_stats ms;
  DevBuf verts, tris;
  for (;;) {
    if (!verts.reserve(3 * (size_t)vcap) || !tris.reserve((3 * (size_t)tcap + 1) / 2))
      return fail(ctx, QJG_ERR_NOMEM, "no memory for the fractal's mesh");
    rc = r.with_rootset([&](qjg_rootset rs) {
      return qjg_mesh_field(ctx, rs, &fg, &it, r.d_field.p, QJG_EDGE_LINEAR, 0.0, 0, verts.p,
                            nullptr, vcap, (int32_t*)tris.p, tcap, &ms, r.s);
    });
    if (rc != QJG_ERR_CAPACITY) break;
    vcap = ms.n_verts + 16;
    tcap = ms.n_tris + 16;
  }
  if (rc) return rc;
  std::vector<double> hv(3 * (size_t)ms.n_verts);
  std::vector<int32_t> ht(3 * (size_t)ms.n_tris);
  QJ_CUDA(ctx, cudaMemcpyAsync(hv.data(), verts.p, hv.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, r.s));
  QJ_CUDA(ctx, cudaMemcpyAsync(ht.data(), tris.p, ht.size() * sizeof(int32_t),
                               cudaMemcpyDeviceToHost, r.s));
  QJ_CUDA(ctx, cudaStreamSynchronize(r.s));
  *n_tris = ms.n_tris;
  const size_t nd = (size_t)r.dgrid.res[0] * r.dgrid.res[1] * r.dgrid.res[2];
  std::vector<double> fd(nd);
  if (r.cfg->sdf(r.cfg->sdf_user, hv.data(), ms.n_verts, ht.data(), ms.n_tris, &r.dgrid,
                 fd.data()))
    return fail(ctx, QJG_ERR_ARG, "the signed-distance callback failed");
  if (!r.d_fd.reserve(nd)) return fail(ctx, QJG_ERR_NOMEM, "no memory for the shape's distance");
  QJ_CUDA(ctx, cudaMemcpyAsync(r.d_fd.p, fd.data(), nd * sizeof(double), cudaMemcpyHostToDevice,
                               r.s));
  QJ_CUDA(ctx, cudaStreamSynchronize(r.s));
  return QJG_OK;
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

}  // namespace

extern "C" {

int qjg_reweight_inside(qjg_ctx* ctx, int64_t n, const double* d_md, const double* d_fd,
                        const double* d_w, double* d_out, double* poor_sum, double* well_sum,
                        void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  if (n < 1 || !d_md || !d_fd || !d_w || !d_out)
    return fail(ctx, QJG_ERR_ARG, "bad size or NULL field");
  cudaStream_t s = (cudaStream_t)stream;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  const int nb = qj::conformal_blocks(n);
  double* d_part = nullptr;
  QJ_CUDA(ctx, qj_malloc_async(ctx, &d_part, sizeof(double) * (3 * (size_t)nb + 3), s));
  double h[3];
  cudaError_t e = qj::launch_region_sums(d_md, d_fd, d_w, n, d_part, d_part + 3 * nb, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h, d_part + 3 * nb, sizeof h, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) {
    // toothOptimizer.cpp:336-366: a quarter of the score to each inside
    // region, half spread flat over the outside
    const double poor = std::fabs(h[0]), well = std::fabs(h[1]);
    const double total_worth = 0.5, outside_worth = 0.5, poor_fraction = 0.5;
    const double outside = ((outside_worth * total_worth) / (1.0 - outside_worth)) / h[2];
    const double k_poor = total_worth * poor_fraction / poor;
    const double k_well = total_worth * (1.0 - poor_fraction) / well;
    e = qj::launch_reweight(d_md, d_fd, d_w, n, k_poor, k_well, outside, d_out, s);
  }
  cudaFreeAsync(d_part, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(ctx, QJG_ERR_CUDA, "reweight: %s", cudaGetErrorString(e));
  ctx->launches += 3;
  if (poor_sum) *poor_sum = h[0];
  if (well_sum) *well_sum = h[1];
  return QJG_OK;
}

int qjg_tooth_optimize(qjg_ctx* ctx, const qjg_tooth_config* cfg, qjg_tooth_level* levels_out,
                       void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  if (!cfg || !cfg->input_path || !levels_out) return fail(ctx, QJG_ERR_ARG, "NULL argument");
  if (cfg->n_levels < 1 || cfg->n_levels > 8)
    return fail(ctx, QJG_ERR_ARG, "n_levels = %d outside [1, 8]", cfg->n_levels);
  for (int l = 0; l < cfg->n_levels; l++)
    if (cfg->levels[l] < 2 || cfg->levels[l] > 1024)
      return fail(ctx, QJG_ERR_ARG, "level resolution %d outside [2, 1024]", cfg->levels[l]);
  if (!(cfg->fractal_radius > 0)) return fail(ctx, QJG_ERR_ARG, "fractal radius must be > 0");
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  ToothRun r;
  r.ctx = ctx;
  r.s = (cudaStream_t)stream;
  r.cfg = cfg;

  // OPTIMIZE_3D::read (OPTIMIZE_3D.cpp:3302-3391)
  if (qjg_o3d_read_info(cfg->input_path, &r.info))
    return fail(ctx, QJG_ERR_ARG, "cannot read the state file %s", cfg->input_path);
  const qjg_o3d_info& in = r.info;
  if (in.n_top < 1 || in.n_bot < 0 || in.n_top + in.n_bot > QJG_MAX_ROOTS)
    return fail(ctx, QJG_ERR_ARG, "state file root counts top=%d bottom=%d", in.n_top, in.n_bot);
  const size_t nd = (size_t)in.field_res[1][0] * in.field_res[1][1] * in.field_res[1][2];
  if (nd == 0) return fail(ctx, QJG_ERR_ARG, "the state file has no distance field");
  r.troots.resize(4 * (size_t)in.n_top);
  r.tpow.resize(in.n_top);
  r.broots.resize(4 * (size_t)in.n_bot);
  r.bpow.resize(in.n_bot);
  const size_t nf = (size_t)in.field_res[0][0] * in.field_res[0][1] * in.field_res[0][2];
  const size_t nc = (size_t)in.field_res[2][0] * in.field_res[2][1] * in.field_res[2][2];
  std::vector<double> h_fractal(nf), h_curv_in(nc);
  r.h_dist.resize(nd);
  if (qjg_o3d_read(cfg->input_path, r.troots.data(), r.tpow.data(), r.broots.data(),
                   r.bpow.data(), h_fractal.data(), r.h_dist.data(), h_curv_in.data()))
    return fail(ctx, QJG_ERR_ARG, "cannot read the state file %s", cfg->input_path);
  r.sig_t = in.sigma_top;
  r.sig_b = in.sigma_bot;
  r.scale = in.exp_scaling;
  // setScoreFields(distance, distance) (:3442-3472): every grid is the
  // distance field's, the curvature a copy of the distance
  r.dgrid = cube_grid(1, in.field_center[1], in.field_lengths[1]);
  for (int c = 0; c < 3; c++) r.dgrid.res[c] = in.field_res[1][c];
  r.h_curv = r.h_dist;
  // the weights: invertedDistanceNormalized of the distance (:3366-3378, 10840)
  if (!r.d_dist.reserve(nd) || !r.d_w.reserve(nd) || !r.d_w2.reserve(nd))
    return fail(ctx, QJG_ERR_NOMEM, "no memory for the distance and weight fields");
  QJ_CUDA(ctx, cudaMemcpyAsync(r.d_dist.p, r.h_dist.data(), nd * sizeof(double),
                               cudaMemcpyHostToDevice, r.s));
  int rc = qjg_inverted_distance(ctx, r.dgrid.res, r.d_dist.p, 1, r.d_w.p, r.s);
  if (rc) return rc;
  // toothOptimizer.cpp:497-507: a unit-cube problem moves to the fractal's
  // frame (translateEverythingExceptFirst, scaleEverything; OPTIMIZE_3D.cpp:
  // 4338-4393)
  const double R = cfg->fractal_radius;
  if (r.dgrid.lengths[0] < 0.95 * R) {
    for (int c = 0; c < 3; c++) r.dgrid.center[c] += -0.5;
    for (int i = 1; i < in.n_top; i++)
      for (int c = 0; c < 3; c++) r.troots[4 * i + c] += -0.5;
    for (int i = 1; i < in.n_bot; i++)
      for (int c = 0; c < 3; c++) r.broots[4 * i + c] += -0.5;
    for (int c = 0; c < 3; c++) {
      r.dgrid.lengths[c] *= R;
      r.dgrid.center[c] *= R;
    }
    for (double& v : r.h_dist) v *= R;
    for (double& v : r.troots) v *= R;
    for (double& v : r.broots) v *= R;
    QJ_CUDA(ctx, cudaMemcpyAsync(r.d_dist.p, r.h_dist.data(), nd * sizeof(double),
                                 cudaMemcpyHostToDevice, r.s));
  }
  for (int c = 0; c < 3; c++) {
    r.fcenter[c] = r.dgrid.center[c];
    r.flengths[c] = r.dgrid.lengths[c];
  }
  // :509-522: every exponent but the first scaled by amp, power scalars 1
  for (int i = 1; i < in.n_top; i++) r.tpow[i] *= cfg->amp;
  for (int i = 1; i < in.n_bot; i++) r.bpow[i] *= cfg->amp;
  r.sig_t = r.sig_b = 1.0;

  int maxres = 0;
  for (int l = 0; l < cfg->n_levels; l++) maxres = std::max(maxres, cfg->levels[l]);
  if (!r.d_field.reserve((size_t)maxres * maxres * maxres))
    return fail(ctx, QJG_ERR_NOMEM, "no memory for the fractal field");
  const int np = 3 + in.n_top + in.n_bot;
  std::vector<double> grad(np);

  for (int l = 0; l < cfg->n_levels; l++) {
    const double t0 = now_ms();
    qjg_tooth_level& L = levels_out[l];
    L = qjg_tooth_level{};
    const int res = cfg->levels[l];
    L.res = res;
    r.cur_res = res;
    r.level_checkpoints = 0;
    const qjg_grid fg = cube_grid(res, r.fcenter, r.flengths);
    auto score_now = [&](double* out) {
      return r.with_rootset([&](qjg_rootset rs) {
        return qjg_tanh_score_grad(ctx, rs, &fg, 1, &r.dgrid, r.d_w.p, 10.0, 0.0, out,
                                   grad.data(), r.d_field.p, nullptr, r.s);
      });
    };
    auto fit = [&](int mode, const double* d_weights, qjg_blmvm_stats* st) {
      r.fit_mode = mode;
      r.cur_grid = fg;
      r.cur_w = d_weights;
      qjg_map_state m = r.state();
      const int frc = qjg_tanh_fit(ctx, mode, &m, &fg, 1, &r.dgrid, d_weights, 10.0, 0.0,
                                   cfg->settings, tooth_monitor, &r, r.d_field.p, st, r.s);
      if (!frc) r.take(m);
      return frc;
    };
    // the conformal-radius scan sets the scale (:403-409, at the first level)
    if (l == 0) {
      double thr = 0, es = 0;
      rc = r.with_rootset([&](qjg_rootset rs) {
        return qjg_conformal_radius(ctx, rs, &fg, &r.dgrid, r.d_dist.p, 10.0, &L.conformal_score,
                                    &thr, &es, r.s);
      });
      if (rc) return rc;
      r.scale = es;
    }
    if ((rc = score_now(&L.initial_score))) return rc;
    if ((rc = qjg_tanh_max_score(ctx, &fg, &r.dgrid, r.d_w.p, &L.max_score, r.s))) return rc;
    if ((rc = fit(QJG_FIT_SCALED_ONLY, r.d_w.p, &L.solve[0]))) return rc;
    if ((rc = fit(QJG_FIT_SCALED, r.d_w.p, &L.solve[1]))) return rc;
    if (cfg->sdf) {
      // buildReweightedInsideField (:277-382), then the reweighted solve
      if ((rc = fractal_distance(r, fg, &L.mesh_tris))) return rc;
      if ((rc = qjg_reweight_inside(ctx, (int64_t)nd, r.d_dist.p, r.d_fd.p, r.d_w.p, r.d_w2.p,
                                    &L.poor_sum, &L.well_sum, r.s)))
        return rc;
      if ((rc = fit(QJG_FIT_SCALED, r.d_w2.p, &L.solve[2]))) return rc;
      L.reweighted = 1;
    }
    if ((rc = fit(QJG_FIT_SCALED, r.d_w.p, &L.solve[3]))) return rc;
    if ((rc = score_now(&L.final_score))) return rc;
    if (cfg->output_prefix) {
      char path[4096];
      std::snprintf(path, sizeof path, "%s_res_%i.o3d", cfg->output_prefix, res);
      if ((rc = r.write_state(path, res))) return rc;
    }
    L.checkpoints = r.level_checkpoints;
    L.ms = now_ms() - t0;
  }
  return QJG_OK;
}

}  // extern "C"
