// C ABI of the optimizer's set-up passes (conformal.cu): the inverted
// distance weight field and the conformal-radius scan.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/quijibo_gpu.h"
#include "qj_conformal.h"
#include "qj_ctx.h"
#include "qj_kernels.h"

namespace {

// Scratch freed on every exit path.
struct Scratch {
  qjg_ctx* ctx;
  cudaStream_t s;
  std::vector<void*> ptrs;
  Scratch(qjg_ctx* c, cudaStream_t st) : ctx(c), s(st) {}
  template <class T>
  T* get(size_t n) {
    void* p = nullptr;
    if (qj_malloc_async(ctx, &p, (n ? n : 1) * sizeof(T), s) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  ~Scratch() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
  }
};

// FIELD_3D::invertedDistance[Normalized] of d_dist into d_out.
int inverted_distance(qjg_ctx* ctx, const int32_t res[3], const double* d_dist, bool normalized,
                      double* d_out, cudaStream_t s, Scratch& sc) {
  const int X = res[0], Y = res[1], Z = res[2];
  const long long n = (long long)X * Y * Z;
  double* tmp = sc.get<double>((size_t)n);
  unsigned long long* left = sc.get<unsigned long long>(1);
  double* part = sc.get<double>(3 * (size_t)qj::conformal_blocks(n) + 3);
  if (!tmp || !left || !part) return fail(ctx, QJG_ERR_NOMEM, "no memory for the weight field");
  QJ_CUDA(ctx, qj::launch_shells(d_dist, X, Y, Z, d_out, s));
  // one breadth-first layer per sweep, until no zero cell is left; a sweep
  // that numbers nothing means cells no shell can reach (no sign change)
  double* cur = d_out;
  double* next = tmp;
  unsigned long long prev_left = ~0ull;
  for (long long sweep = 0;; sweep++) {
    QJ_CUDA(ctx, cudaMemsetAsync(left, 0, sizeof *left, s));
    QJ_CUDA(ctx, qj::launch_layer(cur, next, X, Y, Z, left, s));
    unsigned long long h = 0;
    QJ_CUDA(ctx, cudaMemcpyAsync(&h, left, sizeof h, cudaMemcpyDeviceToHost, s));
    QJ_CUDA(ctx, cudaStreamSynchronize(s));
    std::swap(cur, next);
    if (h == 0) break;
    if (h == prev_left || sweep > (long long)X + Y + Z)
      return fail(ctx, QJG_ERR_ARG,
                  "the distance field has no sign change reaching %llu cells", h);
    prev_left = h;
  }
  if (cur != d_out)
    QJ_CUDA(ctx, cudaMemcpyAsync(d_out, cur, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice,
                                 s));
  QJ_CUDA(ctx, qj::launch_invert(d_dist, d_out, n, s));
  if (!normalized) return QJG_OK;
  // FIELD_3D.cpp:5316-5352: scale by 1 / sum|w|, then each side to 0.5
  double sums[3];
  QJ_CUDA(ctx, qj::launch_side_sums(d_dist, d_out, n, 1.0, part, part + 3 * qj::conformal_blocks(n),
                                    s));
  QJ_CUDA(ctx, cudaMemcpyAsync(sums, part + 3 * qj::conformal_blocks(n), sizeof sums,
                               cudaMemcpyDeviceToHost, s));
  QJ_CUDA(ctx, cudaStreamSynchronize(s));
  const double scale = 1.0 / sums[0];
  QJ_CUDA(ctx, qj::launch_side_sums(d_dist, d_out, n, scale, part,
                                    part + 3 * qj::conformal_blocks(n), s));
  QJ_CUDA(ctx, cudaMemcpyAsync(sums, part + 3 * qj::conformal_blocks(n), sizeof sums,
                               cudaMemcpyDeviceToHost, s));
  QJ_CUDA(ctx, cudaStreamSynchronize(s));
  const double k_in = 0.5 / std::fabs(sums[1]), k_out = 0.5 / std::fabs(sums[2]);
  QJ_CUDA(ctx, qj::launch_scale_sides(d_dist, d_out, n, scale, k_in, k_out, s));
  return QJG_OK;
}

bool valid_res(const int32_t r[3]) { return r && r[0] > 0 && r[1] > 0 && r[2] > 0; }

}  // namespace

extern "C" {

int qjg_inverted_distance(qjg_ctx* ctx, const int32_t res[3], const double* d_dist,
                          int32_t normalized, double* d_out, void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  if (!valid_res(res) || !d_dist || !d_out)
    return fail(ctx, QJG_ERR_ARG, "bad resolution or NULL buffer");
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = (cudaStream_t)stream;
  Scratch sc(ctx, s);
  return inverted_distance(ctx, res, d_dist, normalized != 0, d_out, s, sc);
}

int qjg_conformal_radius(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid,
                         const qjg_grid* dist_grid, const double* d_dist, double alpha,
                         double* min_score, double* threshold, double* exp_scaling, void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  const qj::MapParams* m0 = qj_lookup(ctx, rs);
  if (!m0) return fail(ctx, QJG_ERR_HANDLE, "unknown root set %d", rs);
  int rc;
  if ((rc = qj_check_grid(ctx, grid)) || (rc = qj_check_grid(ctx, dist_grid))) return rc;
  if (!d_dist || !min_score || !threshold || !exp_scaling)
    return fail(ctx, QJG_ERR_ARG, "NULL distance field or output");
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = (cudaStream_t)stream;
  Scratch sc(ctx, s);
  const long long n = (long long)grid->res[0] * grid->res[1] * grid->res[2];
  const long long nd = (long long)dist_grid->res[0] * dist_grid->res[1] * dist_grid->res[2];

  // the scan's field: one application of T/B with the roots' own exponents
  // (evaluatePowerFactored, no power scalar), s = 1, escape 20
  // (estimateConformalRadius, OPTIMIZE_3D.cpp:4704-4714; the map
  // computeLogPowerRationalMapCached, :1165-1265)
  qj::MapParams m;
  std::memcpy(&m, m0, sizeof m);
  for (int i = 0; i < m.nt + m.nb; i++) m.e64[i] = m.ep[i];
  m.sigma[0] = m.sigma[1] = 1.0;
  m.scale = 1.0;
  m.scalef = 1.0f;
  qjg_iter it = {};
  it.max_it = 1;
  it.precision = QJG_FP64;
  it.refine_pow = QJG_REFINE_POW;
  it.escape = 20.0;
  double* f = sc.get<double>((size_t)n);
  double* wf = sc.get<double>((size_t)nd);
  double* wl = sc.get<double>((size_t)n);
  const int nb = qj::conformal_blocks(n);
  double* part = sc.get<double>((size_t)nb * 4096 + 4 * (size_t)nb);
  double* thr = sc.get<double>(4096);
  double* scores = sc.get<double>(4096);
  if (!f || !wf || !wl || !part || !thr || !scores)
    return fail(ctx, QJG_ERR_NOMEM, "no memory for the conformal scan");
  // the field kernel takes its tiles from the context's counter block
  QJ_CUDA(ctx, cudaMemsetAsync(ctx->d_stats, 0, sizeof(qj::DevStats), s));
  QJ_CUDA(ctx, qj::launch_field64(m, qj_grid_params(grid, 0, grid->res[2]),
                                  qj_iter_params(&it, grid), true, f, nullptr, ctx->d_stats, s));
  // clampInfsToMean (FIELD_3D.cpp:5182-5203), then the field's range
  int nblk = 0;
  QJ_CUDA(ctx, qj::launch_field_stats(f, n, part, &nblk, s));
  std::vector<double> st((size_t)4 * nblk);
  QJ_CUDA(ctx, cudaMemcpyAsync(st.data(), part, st.size() * sizeof(double), cudaMemcpyDeviceToHost,
                               s));
  QJ_CUDA(ctx, cudaStreamSynchronize(s));
  double sum = 0, cnt = 0, lo = INFINITY, hi = -INFINITY;
  for (int b = 0; b < nblk; b++) {
    sum += st[4 * b];
    cnt += st[4 * b + 1];
    lo = std::fmin(lo, st[4 * b + 2]);
    hi = std::fmax(hi, st[4 * b + 3]);
  }
  const double mean = sum / cnt;
  if (std::isinf(lo) || std::isinf(hi)) {
    QJ_CUDA(ctx, qj::launch_clamp_infs(f, n, mean, s));
    QJ_CUDA(ctx, qj::launch_field_stats(f, n, part, &nblk, s));
    QJ_CUDA(ctx, cudaMemcpyAsync(st.data(), part, st.size() * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
    QJ_CUDA(ctx, cudaStreamSynchronize(s));
    lo = INFINITY;
    hi = -INFINITY;
    for (int b = 0; b < nblk; b++) {
      lo = std::fmin(lo, st[4 * b + 2]);
      hi = std::fmax(hi, st[4 * b + 3]);
    }
  }
  // the inverted distance field, looked up at the fractal's cell centres
  if ((rc = inverted_distance(ctx, dist_grid->res, d_dist, false, wf, s, sc))) return rc;
  QJ_CUDA(ctx, qj::launch_lookup(qj_grid_params(grid, 0, grid->res[2]), qj_weight_grid(dist_grid),
                                 wf, wl, s));
  // four passes of ~100 thresholds, each around the previous minimum
  double min_t = lo, found = FLT_MAX;
  double a = lo, b = hi;
  std::vector<double> xs, sv;
  for (int pass = 0; pass < 4; pass++) {
    const double inc = (b - a) / 100;
    if (!(inc > 0) || !std::isfinite(inc))
      return fail(ctx, QJG_ERR_ARG, "the scan range [%g, %g] is empty", a, b);
    xs.clear();
    for (double x = a; x < b && xs.size() < 4096; x += inc) xs.push_back(x);
    QJ_CUDA(ctx, cudaMemcpyAsync(thr, xs.data(), xs.size() * sizeof(double),
                                 cudaMemcpyHostToDevice, s));
    QJ_CUDA(ctx, qj::launch_scan(f, wl, n, thr, (int)xs.size(), alpha, part, scores, s));
    sv.resize(xs.size());
    QJ_CUDA(ctx, cudaMemcpyAsync(sv.data(), scores, sv.size() * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
    QJ_CUDA(ctx, cudaStreamSynchronize(s));
    found = FLT_MAX;
    for (size_t k = 0; k < xs.size(); k++)
      if (sv[k] < found) {
        found = sv[k];
        min_t = xs[k];
      }
    a = min_t - 5 * inc;
    b = min_t + 5 * inc;
  }
  *min_score = found;
  *threshold = min_t;
  *exp_scaling = std::exp(-min_t);
  return QJG_OK;
}

}  // extern "C"
