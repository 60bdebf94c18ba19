// Central-difference root gradients of OPTIMIZE_3D's binary-score objectives,
// every perturbed map in one pass (qjg_centered_gradient):
//
//   computeLogRationalCenteredGradient (OPTIMIZE_3D.cpp:2872-2951) and
//   computeLogRationalBottomCenteredGradient (:2956-3008): the binary score
//   (computeBinaryScore, :2275-2297) of computeLogRationalMap (:1907-1985);
//   computeCenteredGradient (:2761-2812): half the binary plus the curvature
//   score (computeCurvatureScore, :2497-2537) of computeMap (:853-980).
//
// The reference evaluates the grid twice per root component (root moved by
// +eps and by -eps), one component after the other.  Here a variant index
// selects the moved root, the component and the side, and one launch
// evaluates every variant on every voxel: the grid's blocks are the
// variants' voxel words.  Each warp writes one 32-voxel word of the variant's
// sign bits (fractal > 0); the binary score is then N - 2 popcount(P xor D)
// over N voxels (D: distance < 0), an integer, exactly the reference's sum of
// +-1 terms; the curvature score repeats the reference's sequential Kahan
// sum, one thread per variant.  Every map evaluation is FP64 in the
// reference's operation order (quaternion products only, no
// transcendentals but the final log), so signs, scores and gradients are the
// reference's bits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/quijibo_gpu.h"
#include "qj_ctx.h"
#include "qj_device.cuh"

namespace {

using namespace qj;

constexpr int FD_WARPS = 8;  // words (32 voxels) per block

struct FdSetup {
  int kind;      // QJG_FD_*
  int k0, nk;    // perturbed roots: MapParams indices [k0, k0 + nk)
  int variants;  // 8 nk + 1 (the last is the unperturbed map)
  int max_it;
  double eps;
  long long n;      // voxels
  long long words;  // ceil(n / 32)
};

// evaluateFactored (POLYNOMIAL_4D.cpp:1080-1088): (q - r_lo)(q - r_lo+1)...,
// left to right; root `pk` (if in range) replaced by `rp`.
__device__ __forceinline__ q64::Q factored(const MapParams& m, const q64::Q& q, int lo, int hi,
                                           int pk, const q64::Q& rp) {
  using namespace q64;
  Q r = {1.0, 0.0, 0.0, 0.0};
#pragma unroll 1
  for (int i = lo; i < hi; i++) {
    Q d;
    if (i == pk) {
      d.w = sub(q.w, rp.w);
      d.x = sub(q.x, rp.x);
      d.y = sub(q.y, rp.y);
      d.z = sub(q.z, rp.z);
    } else {
      d.w = sub(q.w, m.r64[i][0]);
      d.x = sub(q.x, m.r64[i][1]);
      d.y = sub(q.y, m.r64[i][2]);
      d.z = sub(q.z, m.r64[i][3]);
    }
    r = (i == lo) ? d : qmul(r, d);
  }
  return r;
}

// fractal > 0 at start point p for variant v
__device__ __forceinline__ bool fd_positive(const MapParams& m, const FdSetup& f, int v,
                                            const double p[3], double slice) {
  using namespace q64;
  int pk = -1;
  Q rp = {0.0, 0.0, 0.0, 0.0};
  if (v < f.variants - 1) {
    pk = f.k0 + v / 8;
    const int c = (v >> 1) & 3;
    const double delta = (v & 1) ? -f.eps : f.eps;
    double r[4] = {m.r64[pk][0], m.r64[pk][1], m.r64[pk][2], m.r64[pk][3]};
    r[c] = add(r[c], delta);  // newRoot[y] += eps, or -= eps
    rp = Q{r[0], r[1], r[2], r[3]};
  }
  Q q = {p[0], p[1], p[2], slice};
  double mg = mag(q);
  int n = 0;
  if (f.kind == QJG_FD_POLYNOMIAL) {
    // computeMap: iterate = top.evaluateFactored(iterate), escape 10,
    // fractal = -1 if the orbit stayed (max_it) or |q| < 10, else +1
    while (mg < 10.0 && n < f.max_it) {
      q = factored(m, q, 0, m.nt, pk, rp);
      mg = mag(q);
      n++;
    }
    return !(n == f.max_it || mg < 10.0);
  }
  // computeLogRationalMap: q T(q) / (q B(q)) times s, escape 20, log|q|
  while (mg < 20.0 && n < f.max_it) {
    const Q top = qmul(q, factored(m, q, 0, m.nt, pk, rp));
    Q o = top;
    if (m.nb > 0) o = qdiv(top, qmul(q, factored(m, q, m.nt, m.nt + m.nb, pk, rp)));
    q = Q{mul(m.scale, o.w), mul(m.scale, o.x), mul(m.scale, o.y), mul(m.scale, o.z)};
    mg = mag(q);
    n++;
  }
  return log(mg) > 0.0;
}

// bits[v * words + w]: bit j = fractal > 0 at voxel 32 w + j of variant v
__global__ void __launch_bounds__(32 * FD_WARPS) fd_sign_kernel(const __grid_constant__ MapParams m,
                                                                const GridParams g, const FdSetup f,
                                                                uint32_t* __restrict__ bits) {
  const int v = blockIdx.y;
  const long long w = (long long)blockIdx.x * FD_WARPS + (threadIdx.x >> 5);
  if (w >= f.words) return;  // whole warps leave together
  const long long i = w * 32 + (threadIdx.x & 31);
  bool pos = false;
  if (i < f.n) {
    const int x = (int)(i % g.X);
    const int y = (int)((i / g.X) % g.Y);
    const int z = (int)(i / ((long long)g.X * g.Y));
    double p[3];
    cell_center(g, x, y, z, p);
    pos = fd_positive(m, f, v, p, g.slice);
  }
  const uint32_t word = __ballot_sync(0xffffffffu, pos);
  if ((threadIdx.x & 31) == 0) bits[(long long)v * f.words + w] = word;
}

// D bits (distance at the cell centre < 0, computeBinaryScore's lookup) and
// the curvature score's per-voxel term sign * curvature (sign = +1 where
// _distanceField[x] < 0, else -1).
__global__ void __launch_bounds__(256) fd_dist_kernel(const GridParams g, const WeightGrid wg,
                                                      const double* __restrict__ dist,
                                                      const double* __restrict__ curv, long long n,
                                                      long long words, uint32_t* __restrict__ dbits,
                                                      double* __restrict__ adding) {
  const long long w = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (w >= words) return;
  const long long i = w * 32 + (threadIdx.x & 31);
  bool neg = false;
  if (i < n) {
    const int x = (int)(i % g.X);
    const int y = (int)((i / g.X) % g.Y);
    const int z = (int)(i / ((long long)g.X * g.Y));
    double p[3];
    cell_center(g, x, y, z, p);
    neg = trilinear(wg, dist, p) < 0.0;
    if (curv) adding[i] = q64::mul(dist[i] < 0.0 ? 1.0 : -1.0, curv[i]);
  }
  const uint32_t word = __ballot_sync(0xffffffffu, neg);
  if ((threadIdx.x & 31) == 0) dbits[w] = word;
}

// mismatches[v] = popcount(P_v xor D) over the grid
__global__ void __launch_bounds__(256) fd_count_kernel(const uint32_t* __restrict__ bits,
                                                       const uint32_t* __restrict__ dbits,
                                                       long long words, long long n,
                                                       unsigned long long* mism) {
  const int v = blockIdx.y;
  unsigned long long c = 0;
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (long long)gridDim.x * blockDim.x) {
    uint32_t x = bits[(long long)v * words + w] ^ dbits[w];
    if (w == words - 1 && (n & 31)) x &= (1u << (n & 31)) - 1u;
    c += __popc(x);
  }
  for (int o = 16; o; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(mism + v, c);
}

// computeCurvatureScore's numerator for each variant: the sequential Kahan
// sum (OPTIMIZE_3D.cpp:2486-2492) of adding[x] * fractal[x], fractal = +-1
__global__ void __launch_bounds__(128) fd_kahan_kernel(const uint32_t* __restrict__ bits,
                                                       const double* __restrict__ adding,
                                                       long long words, long long n, int variants,
                                                       double* __restrict__ out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= variants) return;
  using namespace q64;
  double score = 0.0, err = 0.0;
  const uint32_t* row = bits + (long long)v * words;
  for (long long w = 0; w < words; w++) {
    const uint32_t word = row[w];
    const int m = (int)((n - w * 32) < 32 ? (n - w * 32) : 32);
    for (int j = 0; j < m; j++) {
      const double a = adding[w * 32 + j];
      const double term = ((word >> j) & 1u) ? a : -a;  // adding * fractal[x], exact
      const double y = sub(term, err);
      const double t = add(score, y);
      err = sub(sub(t, score), y);
      score = t;
    }
  }
  out[v] = score;
}

}  // namespace

extern "C" int qjg_centered_gradient(qjg_ctx* ctx, qjg_rootset rs, const qjg_grid* grid,
                                     int32_t max_it, int32_t kind, const double* d_dist,
                                     const double* d_curv, double* grad, double* score,
                                     void* stream) {
  if (!ctx) return QJG_ERR_ARG;
  const MapParams* m = qj_lookup(ctx, rs);
  if (!m) return fail(ctx, QJG_ERR_HANDLE, "unknown root set %d", rs);
  int rc;
  if ((rc = qj_check_grid(ctx, grid))) return rc;
  if (max_it < 0) return fail(ctx, QJG_ERR_ARG, "max_it = %d < 0", max_it);
  if (kind != QJG_FD_LOG_RATIONAL && kind != QJG_FD_LOG_RATIONAL_BOTTOM &&
      kind != QJG_FD_POLYNOMIAL)
    return fail(ctx, QJG_ERR_ARG, "unknown kind %d", kind);
  if (!d_dist || !grad || (kind == QJG_FD_POLYNOMIAL && !d_curv))
    return fail(ctx, QJG_ERR_ARG, "NULL distance / curvature field or gradient");
  FdSetup f;
  f.kind = kind;
  f.max_it = max_it;
  f.k0 = kind == QJG_FD_LOG_RATIONAL_BOTTOM ? m->nt : 0;
  f.nk = kind == QJG_FD_LOG_RATIONAL ? m->nt + m->nb
         : kind == QJG_FD_POLYNOMIAL ? m->nt
                                     : m->nb;
  f.variants = 8 * f.nk + 1;
  // const Real dx = _lengths[0] / _xRes; eps = dx
  f.eps = grid->lengths[0] / grid->res[0];
  f.n = (long long)grid->res[0] * grid->res[1] * grid->res[2];
  f.words = (f.n + 31) / 32;
  if (f.variants > 65535) return fail(ctx, QJG_ERR_ARG, "too many roots (%d)", f.nk);
  cudaStream_t s = (cudaStream_t)stream;
  QJ_CUDA(ctx, cudaSetDevice(ctx->device));
  const GridParams g = qj_grid_params(grid, 0, grid->res[2]);
  const WeightGrid wg = qj_weight_grid(grid);
  const bool curv = kind == QJG_FD_POLYNOMIAL;
  const size_t bits_bytes = sizeof(uint32_t) * (size_t)f.words * (size_t)(f.variants + 1);
  const size_t add_bytes = curv ? sizeof(double) * (size_t)f.n : 0;
  const size_t out_bytes = sizeof(unsigned long long) * f.variants + sizeof(double) * f.variants;
  unsigned char* scratch = nullptr;
  QJ_CUDA(ctx, qj_malloc_async(ctx, &scratch, bits_bytes + add_bytes + out_bytes, s));
  uint32_t* bits = reinterpret_cast<uint32_t*>(scratch);
  uint32_t* dbits = bits + (size_t)f.words * f.variants;
  double* adding = curv ? reinterpret_cast<double*>(scratch + bits_bytes) : nullptr;
  unsigned long long* mism = reinterpret_cast<unsigned long long*>(scratch + bits_bytes + add_bytes);
  double* kahan = reinterpret_cast<double*>(mism + f.variants);
  cudaError_t e = cudaMemsetAsync(mism, 0, sizeof(unsigned long long) * f.variants, s);
  const unsigned wblocks = (unsigned)((f.words + FD_WARPS - 1) / FD_WARPS);
  if (e == cudaSuccess) {
    fd_dist_kernel<<<(unsigned)((f.words + 7) / 8), 256, 0, s>>>(g, wg, d_dist, curv ? d_curv : nullptr,
                                                                  f.n, f.words, dbits, adding);
    fd_sign_kernel<<<dim3(wblocks, (unsigned)f.variants), 32 * FD_WARPS, 0, s>>>(*m, g, f, bits);
    const unsigned cblocks = (unsigned)std::min<long long>((f.words + 255) / 256, 64);
    fd_count_kernel<<<dim3(cblocks, (unsigned)f.variants), 256, 0, s>>>(bits, dbits, f.words, f.n,
                                                                          mism);
    if (curv)
      fd_kahan_kernel<<<(f.variants + 127) / 128, 128, 0, s>>>(bits, adding, f.words, f.n,
                                                                f.variants, kahan);
    e = cudaGetLastError();
  }
  std::vector<unsigned long long> h_mism((size_t)f.variants);
  std::vector<double> h_kahan(curv ? (size_t)f.variants : 0);
  std::vector<double> h_add(curv ? (size_t)f.n : 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h_mism.data(), mism, sizeof(unsigned long long) * f.variants,
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && curv)
    e = cudaMemcpyAsync(h_kahan.data(), kahan, sizeof(double) * f.variants, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && curv)
    e = cudaMemcpyAsync(h_add.data(), adding, sizeof(double) * f.n, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(scratch, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(ctx, QJG_ERR_CUDA, "centered gradient: %s", cudaGetErrorString(e));
  ctx->launches += curv ? 4 : 3;
  // computeCurvatureScore's denominator: the sequential Kahan sum of |adding|
  double den = 0.0, den_err = 0.0;
  for (long long i = 0; i < (curv ? f.n : 0); i++) {
    const double y = std::fabs(h_add[(size_t)i]) - den_err;
    const double t = den + y;
    den_err = (t - den) - y;
    den = t;
  }
  const double N = (double)f.n;  // score / fractal.totalCells()
  auto score_of = [&](int v) {
    const double binary = (N - 2.0 * (double)h_mism[(size_t)v]) / N;
    if (!curv) return binary;
    return (binary + h_kahan[(size_t)v] / den) * 0.5;
  };
  for (int k = 0; k < f.nk; k++)
    for (int c = 0; c < 4; c++) {
      const int v = 8 * k + 2 * c;
      grad[4 * k + c] = (score_of(v) - score_of(v + 1)) / (2.0 * f.eps);
    }
  if (score) *score = score_of(f.variants - 1);
  return QJG_OK;
}
