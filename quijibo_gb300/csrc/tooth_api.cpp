// C ABI of toothOptimizer's fits: BLMVM (blmvm.cpp) over the tanh score,
// each objective evaluation one GPU pass of the score and its analytic
// gradients (energy.cu, tanh_grad_kernel).
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
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
  const int slots = 6 + nt + nb;
  double* d_part = nullptr;
  QJ_CUDA(ctx, cudaMallocAsync((void**)&d_part, sizeof(double) * ((size_t)nblocks + 1) * slots, s));
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
  qj::blmvm::Objective obj = [&](const double* xv, double* f, double* gv) -> int {
    lay.from_vars(xv, cur, tp.data(), bp.data());
    if (qj_fill_map(&m, nt, cur.top_roots, tp.data(), cur.sigma_top, nb, cur.bot_roots, bp.data(),
                    cur.sigma_bot, cur.scale) >= 0) {
      // an exponent overflowed: the reference's score is then not finite
      *f = NAN;
      for (int i = 0; i < n; i++) gv[i] = NAN;
      return 0;
    }
    cudaError_t e = qj::launch_tanh_grad(m, g, wg, d_weights, max_it, alpha, threshold, true,
                                         d_field, d_part, nblocks, d_out, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_out, d_out, sizeof(double) * slots, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cuda_failed = 1;
      fail(ctx, QJG_ERR_CUDA, "tanh fit: %s", cudaGetErrorString(e));
      return QJG_ERR_CUDA;
    }
    ctx->launches += 2;
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
  QJ_CUDA(ctx, cudaMallocAsync((void**)&d_w, sizeof(double) * ((size_t)n + 3 * (size_t)nb + 3), s));
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
