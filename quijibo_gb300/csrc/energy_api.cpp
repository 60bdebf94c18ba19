// C ABI of the fitting energies and their gradients.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/quijibo_gpu_bench.h"
#include "qj_ctx.h"
#include "qj_energy.h"
#include "qj_lbfgs.h"

qj::WeightGrid qj_weight_grid(const qjg_grid* g) {
  qj::WeightGrid wg;
  wg.X = g->res[0];
  wg.Y = g->res[1];
  wg.Z = g->res[2];
  for (int c = 0; c < 3; c++) {
    // FIELD_3D.cpp:971-980: corner = center - 0.5 lengths; corner += 0.5 dxs; 1/dx
    const double dx = g->lengths[c] / g->res[c];
    double corner = g->center[c] - g->lengths[c] * 0.5;
    corner += dx * 0.5;
    wg.corner[c] = corner;
    wg.inv[c] = 1.0 / dx;
  }
  return wg;
}

extern "C" {

int qjg_energy_backward_batch(qjg_ctx* ctx, int32_t n_items, qjg_energy_item* items,
                              void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  if (n_items < 0 || (n_items > 0 && !items)) return fail(ctx, QJG_ERR_ARG, "no items");
  if (n_items == 0) return QJG_OK;
  std::vector<qj::SqBatchReq> req((size_t)n_items);
  for (int i = 0; i < n_items; i++) {
    const qjg_energy_item& it = items[i];
    if (it.n_top < 1 || it.n_bot < 0 || it.n_top + it.n_bot > QJG_MAX_ROOTS)
      return fail(ctx, QJG_ERR_ARG, "item %d: root counts top=%d bottom=%d", i, it.n_top, it.n_bot);
    if (it.n < 0 || it.n > INT32_MAX || !it.d_params || !it.d_grad ||
        (it.n > 0 && (!it.d_xyz || !it.d_target)))
      return fail(ctx, QJG_ERR_ARG, "item %d: NULL or out-of-range arguments", i);
    if (it.max_it < 0 || it.max_it > qj::sq_max_iterations())
      return fail(ctx, QJG_ERR_ARG, "item %d: max_it = %d", i, it.max_it);
    if (!(it.escape > 0)) return fail(ctx, QJG_ERR_ARG, "item %d: escape radius must be > 0", i);
    req[(size_t)i] = qj::SqBatchReq{it.d_params, it.n_top, it.n_bot, it.n, it.d_xyz, it.d_target,
                                    it.slice, it.max_it, it.escape, it.d_sat};
  }
  cudaStream_t s = (cudaStream_t)stream;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  void* d_scr = nullptr;
  QJ_CUDA(ctx, qj_malloc_async(ctx, &d_scr, qj::sq_batch_scratch_bytes(req.data(), n_items), s));
  std::vector<double*> outs((size_t)n_items);
  std::vector<double> energies((size_t)n_items);
  int launched = 0;
  cudaError_t e = qj::launch_sq_energy_batch(req.data(), n_items, d_scr, outs.data(), s, &launched);
  for (int i = 0; i < n_items && e == cudaSuccess; i++) {
    const int P = 5 * (items[i].n_top + items[i].n_bot) + 1;
    e = cudaMemcpyAsync(items[i].d_grad, outs[(size_t)i] + 1, sizeof(double) * P,
                        cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&energies[(size_t)i], outs[(size_t)i], sizeof(double),
                          cudaMemcpyDeviceToHost, s);
  }
  cudaFreeAsync(d_scr, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(ctx, QJG_ERR_CUDA, "energy batch: %s", cudaGetErrorString(e));
  for (int i = 0; i < n_items; i++) items[i].energy = energies[(size_t)i];
  ctx->launches += launched;
  return QJG_OK;
}

int qjg_set_energy_pairs(int on) {
  qj::set_energy_pairs(on);
  return QJG_OK;
}

int qjg_set_energy_adjoint_roots(int on) {
  qj::set_energy_adjoint_roots(on);
  return QJG_OK;
}

int qjg_set_energy_forward_blocks(int per_sm) {
  if (per_sm < 0) return QJG_ERR_ARG;
  qj::set_energy_forward_blocks(per_sm);
  return QJG_OK;
}

int qjg_set_energy_fast(int on) {
  return qj::set_energy_fast(on) == cudaSuccess ? QJG_OK : QJG_ERR_CUDA;
}

int qjg_energy_last_work(qjg_ctx* ctx, int64_t* applications, int64_t* steps) {
  if (!ctx || !applications || !steps) return QJG_ERR_ARG;
  *applications = ctx->sq_applications;
  *steps = ctx->sq_steps;
  return QJG_OK;
}

int qjg_tanh_score_grad(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid, int32_t max_it,
                        const qjg_grid* weight_grid, const double* d_weights, double alpha,
                        double threshold, double* score, double* grad, double* d_field,
                        qjg_tanh_stats* stats, void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  const qj::MapParams* m = qj_lookup(ctx, rs);
  if (!m) return fail(ctx, QJG_ERR_HANDLE, "unknown root set %d", rs);
  int rc;
  if ((rc = qj_check_grid(ctx, grid)) || (rc = qj_check_grid(ctx, weight_grid))) return rc;
  if (max_it < 0) return fail(ctx, QJG_ERR_ARG, "max_it = %d < 0", max_it);
  if (!d_weights || !score || !grad) return fail(ctx, QJG_ERR_ARG, "NULL weights/score/grad");
  cudaStream_t s = (cudaStream_t)stream;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  const qj::GridParams g = qj_grid_params(grid, 0, grid->res[2]);
  const qj::WeightGrid wg = qj_weight_grid(weight_grid);
  const int nblocks = qj::tanh_blocks();
  const int slots = qj::tanh_slots(m->nt, m->nb);
  double* d_part = nullptr;
  QJ_CUDA(ctx, qj_malloc_async(ctx, &d_part, sizeof(double) * ((size_t)nblocks + 1) * slots, s));
  double* d_out = d_part + (size_t)nblocks * slots;
  cudaError_t e = qj::launch_tanh_grad(*m, g, wg, d_weights, max_it, alpha, threshold, true,
                                       d_field, d_part, nblocks, d_out, s);
  std::vector<double> out(slots);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out.data(), d_out, sizeof(double) * slots, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d_part, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(ctx, QJG_ERR_CUDA, "tanh score: %s", cudaGetErrorString(e));
  ctx->launches += 3;
  const int nt = m->nt, nb = m->nb;
  for (int k = 0; k < 3 + nt + nb; k++) grad[k] = out[k];
  *score = out[3 + nt + nb];
  if (stats) {
    stats->voxels = (int64_t)grid->res[0] * grid->res[1] * grid->res[2];
    stats->overflowed = (int64_t)out[4 + nt + nb];
    stats->bad_terms = (int64_t)out[5 + nt + nb];
    stats->band_voxels = (int64_t)out[7 + nt + nb];
  }
  return QJG_OK;
}

static int sq_energy(qjg_ctx* ctx, const double* d_params, int32_t nt, int32_t nb, int64_t n,
                     const double* d_xyz, const double* d_target, double slice, int32_t max_it,
                     double escape, double d_sat, int32_t precision, double* energy,
                     double* d_grad, int32_t* d_iters, void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  if (nt < 1 || nb < 0 || nt + nb > QJG_MAX_ROOTS)
    return fail(ctx, QJG_ERR_ARG, "root counts top=%d bottom=%d", nt, nb);
  if (n < 0 || !d_params || !energy || (n > 0 && (!d_xyz || !d_target)))
    return fail(ctx, QJG_ERR_ARG, "NULL or negative energy arguments");
  if (max_it < 0 || max_it > qj::sq_max_iterations())
    return fail(ctx, QJG_ERR_ARG, "max_it = %d outside [0, %d]", max_it, qj::sq_max_iterations());
  if (!(escape > 0)) return fail(ctx, QJG_ERR_ARG, "escape radius must be > 0");
  if (precision != QJG_FP32 && precision != QJG_FP64)
    return fail(ctx, QJG_ERR_ARG, "energy precision must be QJG_FP32 or QJG_FP64");
  cudaStream_t s = (cudaStream_t)stream;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  if (n > INT32_MAX) return fail(ctx, QJG_ERR_ARG, "energy: %lld samples (at most 2^31 - 1)", (long long)n);
  const bool fp64 = precision == QJG_FP64, grad = d_grad != nullptr;
  const int P = 5 * (nt + nb) + 1;
  void* d_scr = nullptr;
  QJ_CUDA(ctx, qj_malloc_async(ctx, &d_scr, qj::sq_scratch_bytes(fp64, grad, n, max_it, nt, nb), s));
  double* d_out = nullptr;
  unsigned long long* d_work = nullptr;
  int launched = 0;
  // the previous call's work sizes the forward grid when it ran on as many
  // samples with the same iteration cap (the optimizer's repeated calls)
  const long long hint =
      (ctx->sq_last_n == n && ctx->sq_last_max_it == max_it) ? ctx->sq_applications : 0;
  cudaError_t e = qj::launch_sq_energy(fp64, grad, d_params, nt, nb, d_xyz, d_target, n, slice,
                                       max_it, escape, d_sat, d_scr, &d_out, d_iters, s, &launched,
                                       &d_work, hint);
  unsigned long long work[2] = {0, 0};
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(work, d_work, sizeof work, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && d_grad)
    e = cudaMemcpyAsync(d_grad, d_out + 1, sizeof(double) * P, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(energy, d_out, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d_scr, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(ctx, QJG_ERR_CUDA, "energy: %s", cudaGetErrorString(e));
  ctx->launches += launched;
  ctx->sq_applications = (int64_t)work[0];
  ctx->sq_steps = (int64_t)work[1];
  ctx->sq_last_n = n;
  ctx->sq_last_max_it = max_it;
  return QJG_OK;
}

int qjg_energy_forward(qjg_ctx* ctx, const double* d_params, int32_t n_top, int32_t n_bot,
                       int64_t n, const double* d_xyz, const double* d_target, double slice,
                       int32_t max_it, double escape, double d_sat, int32_t precision,
                       double* energy, int32_t* d_iters, void* stream) {
  return sq_energy(ctx, d_params, n_top, n_bot, n, d_xyz, d_target, slice, max_it, escape, d_sat,
                   precision, energy, nullptr, d_iters, stream);
}

int qjg_energy_backward(qjg_ctx* ctx, const double* d_params, int32_t n_top, int32_t n_bot,
                        int64_t n, const double* d_xyz, const double* d_target, double slice,
                        int32_t max_it, double escape, double d_sat, int32_t precision,
                        double* energy, double* d_grad, void* stream) {
  if (!d_grad) return fail(ctx, QJG_ERR_ARG, "d_grad is NULL");
  return sq_energy(ctx, d_params, n_top, n_bot, n, d_xyz, d_target, slice, max_it, escape, d_sat,
                   precision, energy, d_grad, nullptr, stream);
}

int qjg_fit_lbfgs(qjg_ctx* ctx, double* d_params, int32_t nt, int32_t nb, int64_t n,
                  const double* d_xyz, const double* d_target, double slice, int32_t max_it,
                  double escape, double d_sat, int32_t precision, int32_t steps, int32_t history,
                  double* energies, qjg_fit_stats* stats, void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  if (!d_params || steps < 0 || history < 1 || history > 64)
    return fail(ctx, QJG_ERR_ARG, "fit: NULL params, steps < 0 or history outside [1, 64]");
  if (nt < 1 || nb < 0 || nt + nb > QJG_MAX_ROOTS)
    return fail(ctx, QJG_ERR_ARG, "root counts top=%d bottom=%d", nt, nb);
  cudaStream_t s = (cudaStream_t)stream;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  const int P = 5 * (nt + nb) + 1, m = history;
  // x1 g0 g1 d | S Y (m x P) | rho alpha (m) | gd
  const size_t total = (size_t)P * 4 + (size_t)2 * m * P + 2 * (size_t)m + 1;
  double* buf = nullptr;
  QJ_CUDA(ctx, qj_malloc_async(ctx, &buf, total * sizeof(double), s));
  double *x = d_params, *x1 = buf, *g0 = x1 + P, *g1 = g0 + P, *d = g1 + P;
  double *S = d + P, *Y = S + (size_t)m * P, *rho = Y + (size_t)m * P, *alpha = rho + m;
  double* gd_dev = alpha + m;
  qjg_fit_stats st = {};
  int rc = QJG_OK;
  auto energy = [&](const double* params, double* e, double* grad) {
    return grad ? qjg_energy_backward(ctx, params, nt, nb, n, d_xyz, d_target, slice, max_it,
                                      escape, d_sat, precision, e, grad, stream)
                : qjg_energy_forward(ctx, params, nt, nb, n, d_xyz, d_target, slice, max_it,
                                     escape, d_sat, precision, e, nullptr, stream);
  };
  double E = 0;
  int k = 0, head = -1;
  if ((rc = energy(x, &E, g0))) goto done;
  st.gradient_evals++;
  st.energy0 = E;
  if (energies) energies[0] = E;
  for (int it = 0; it < steps; it++) {
    double gd = 0, gg = 0;
    cudaError_t e = qj::lbfgs_direction(g0, S, Y, rho, P, m, k, head < 0 ? 0 : head, alpha, d,
                                        gd_dev, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&gd, gd_dev, sizeof gd, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      rc = fail(ctx, QJG_ERR_CUDA, "lbfgs: %s", cudaGetErrorString(e));
      goto done;
    }
    ctx->launches++;
    if (!(gd < 0)) {  // not a descent direction: restart from steepest descent
      k = 0;
      head = -1;
      e = qj::lbfgs_direction(g0, S, Y, rho, P, m, 0, 0, alpha, d, gd_dev, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&gd, gd_dev, sizeof gd, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) {
        rc = fail(ctx, QJG_ERR_CUDA, "lbfgs: %s", cudaGetErrorString(e));
        goto done;
      }
      ctx->launches++;
    }
    gg = -gd;  // |g|^2 when d = -g
    double a = (k == 0) ? 1.0 / std::max(1.0, std::sqrt(std::max(gg, 0.0))) : 1.0;
    double Et = 0;
    bool accepted = false;
    for (int ls = 0; ls < 30; ls++) {
      if ((e = qj::lbfgs_axpy(x, d, a, P, x1, s)) != cudaSuccess) {
        rc = fail(ctx, QJG_ERR_CUDA, "lbfgs: %s", cudaGetErrorString(e));
        goto done;
      }
      ctx->launches++;
      if ((rc = energy(x1, &Et, nullptr))) goto done;
      st.energy_evals++;
      if (std::isfinite(Et) && Et <= E + 1e-4 * a * gd) {
        accepted = true;
        break;
      }
      a *= 0.5;
    }
    if (!accepted) break;  // no decrease along d: converged to noise level
    if ((rc = energy(x1, &Et, g1))) goto done;
    st.gradient_evals++;
    head = (head + 1) % m;
    if ((e = qj::lbfgs_update(x, x1, g0, g1, P, head, S, Y, rho, s)) != cudaSuccess) {
      rc = fail(ctx, QJG_ERR_CUDA, "lbfgs: %s", cudaGetErrorString(e));
      goto done;
    }
    ctx->launches++;
    k = std::min(k + 1, m);
    cudaMemcpyAsync(x, x1, P * sizeof(double), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(g0, g1, P * sizeof(double), cudaMemcpyDeviceToDevice, s);
    E = Et;
    st.steps++;
    if (energies) energies[st.steps] = E;
  }
  st.energy = E;
done:
  cudaFreeAsync(buf, s);
  cudaStreamSynchronize(s);
  if (stats) *stats = st;
  return rc;
}

}  // extern "C"
