// The optimizer's set-up passes on the device:
//
//  * inverted distance weight field (FIELD_3D::invertedDistance and
//    invertedDistanceNormalized, src/geometry/FIELD_3D.cpp:5241-5352): the
//    26-neighbour shells on both sides of the signed distance field's sign
//    change get 1, then every other cell the 6-neighbour breadth-first layer
//    number (a Jacobi sweep per layer, as the reference's loop), inverted,
//    negated inside and quartered outside; optionally normalised to |sum| 1
//    and 0.5 per side.
//  * the conformal-radius scan (OPTIMIZE_3D::estimateConformalRadius,
//    src/solvers/OPTIMIZE_3D.cpp:4693-4772): scores
//      S(x) = sum_i -tanh(alpha (F_i - x)) W(c_i)
//    of a one-application field F (computeLogPowerRationalMapCached,
//    :1165-1265) for every threshold x of a pass in one launch; the reference
//    evaluates each threshold with a serial sweep over the grid.
//
// Layer numbers are small integers and the other operations are single
// roundings, so the weight field is exact; sums use fixed-order trees.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "qj_conformal.h"
#include "qj_device.cuh"

namespace qj {

namespace {

constexpr int CT = 256;  // threads per block

__global__ void __launch_bounds__(CT) shell_kernel(const double* __restrict__ dist, int X, int Y,
                                                   int Z, double* __restrict__ out) {
  const long long n = (long long)X * Y * Z;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((long long)X * Y));
    const double c = dist[i];
    bool flip = false;
    for (int k = -1; k <= 1; k++)
      for (int j = -1; j <= 1; j++)
        for (int h = -1; h <= 1; h++) {
          if (!h && !j && !k) continue;
          const int xn = x + h, yn = y + j, zn = z + k;
          if (xn < 0 || xn > X - 1 || yn < 0 || yn > Y - 1 || zn < 0 || zn > Z - 1) continue;
          if (dist[xn + (long long)yn * X + (long long)zn * X * Y] * c < 0) flip = true;
        }
    // outerShell (centre >= 0) + innerShell (centre <= 0); a zero centre never flips
    out[i] = flip ? 1.0 : 0.0;
  }
}

// One layer: zero cells next to a numbered cell take the smallest
// neighbour number + 1 (reads `cur`, writes `next`).
__global__ void __launch_bounds__(CT) layer_kernel(const double* __restrict__ cur,
                                                   double* __restrict__ next, int X, int Y, int Z,
                                                   unsigned long long* zeros_left) {
  const long long n = (long long)X * Y * Z;
  const double big = (double)n + 1.0;
  unsigned long long left = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = cur[i];
    if (v > 1e-5) {
      next[i] = v;
      continue;
    }
    const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((long long)X * Y));
    const long long XY = (long long)X * Y;
    const double nb[6] = {x != 0 ? cur[i - 1] : 0.0,       x != X - 1 ? cur[i + 1] : 0.0,
                          y != 0 ? cur[i - X] : 0.0,       y != Y - 1 ? cur[i + X] : 0.0,
                          z != 0 ? cur[i - XY] : 0.0,      z != Z - 1 ? cur[i + XY] : 0.0};
    double smallest = big;
    for (int k = 0; k < 6; k++)
      if (nb[k] > 1e-5 && nb[k] < smallest) smallest = nb[k];
    if (smallest < (double)n) {
      next[i] = smallest + 1.0;
    } else {
      next[i] = v;
      left++;
    }
  }
  for (int o = 16; o; o >>= 1) left += __shfl_xor_sync(0xffffffffu, left, o);
  if ((threadIdx.x & 31) == 0 && left) atomicAdd(zeros_left, left);
}

// 1 / layer, negated inside, quartered outside.
__global__ void __launch_bounds__(CT) invert_kernel(const double* __restrict__ dist,
                                                    double* __restrict__ w, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double v = __ddiv_rn(1.0, w[i]);
    v = dist[i] < 0 ? -v : __dmul_rn(v, 0.25);
    w[i] = v;
  }
}

// Block sums of up to three masked quantities of w: |w|, w where dist < 0,
// w where dist >= 0 (fixed-order tree within the block).
__device__ __forceinline__ double block_sum(double v, double* sh) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < nw; k++) s += sh[k];
  return s;  // valid in thread 0
}

__global__ void __launch_bounds__(CT) sums_kernel(const double* __restrict__ dist,
                                                  const double* __restrict__ w, long long n,
                                                  double scale, double* __restrict__ part) {
  __shared__ double sh[CT / 32];
  double a = 0.0, in = 0.0, out = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = __dmul_rn(w[i], scale);
    a += fabs(w[i]);
    if (dist[i] < 0) in += v;
    else out += v;
  }
  a = block_sum(a, sh);
  in = block_sum(in, sh);
  out = block_sum(out, sh);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = a;
    part[3 * blockIdx.x + 1] = in;
    part[3 * blockIdx.x + 2] = out;
  }
}

__global__ void scale_sides_kernel(const double* __restrict__ dist, double* __restrict__ w,
                                   long long n, double scale, double k_in, double k_out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = __dmul_rn(w[i], scale);
    w[i] = __dmul_rn(v, dist[i] < 0 ? k_in : k_out);
  }
}

// Field statistics for clampInfsToMean and the scan range: sum and count of
// the finite-or-NaN (non-infinite) values, min and max.
__global__ void __launch_bounds__(CT) field_stats_kernel(const double* __restrict__ f, long long n,
                                                         double* __restrict__ part) {
  __shared__ double sh[CT / 32];
  __shared__ double shm[2][CT / 32];
  double s = 0.0, cnt = 0.0, lo = INFINITY, hi = -INFINITY;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = f[i];
    if (!isinf(v)) {
      s += v;
      cnt += 1.0;
    }
    if (v < lo) lo = v;
    if (v > hi) hi = v;
  }
  s = block_sum(s, sh);
  cnt = block_sum(cnt, sh);
  for (int o = 16; o; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    shm[0][warp] = lo;
    shm[1][warp] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      lo = fmin(lo, shm[0][k]);
      hi = fmax(hi, shm[1][k]);
    }
    part[4 * blockIdx.x] = s;
    part[4 * blockIdx.x + 1] = cnt;
    part[4 * blockIdx.x + 2] = lo;
    part[4 * blockIdx.x + 3] = hi;
  }
}

__global__ void clamp_infs_kernel(double* __restrict__ f, long long n, double mean) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    if (isinf(f[i])) f[i] = mean;
}

// W at every fractal cell centre (FIELD_3D::operator()(VEC3F), float weights).
__global__ void __launch_bounds__(CT) lookup_kernel(const GridParams g, const WeightGrid wg,
                                                    const double* __restrict__ w,
                                                    double* __restrict__ out) {
  const long long n = (long long)g.X * g.Y * g.Z;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % g.X), y = (int)((i / g.X) % g.Y), z = (int)(i / ((long long)g.X * g.Y));
    double p[3];
    cell_center(g, x, y, z, p);
    out[i] = trilinear(wg, w, p);
  }
}

// part[block][t] = sum over the block's voxels of -tanh(alpha (F - thr[t])) w.
__global__ void __launch_bounds__(CT) scan_kernel(const double* __restrict__ f,
                                                  const double* __restrict__ w, long long n,
                                                  const double* __restrict__ thr, int nthr,
                                                  double alpha, double* __restrict__ part) {
  __shared__ double sh[CT / 32];
  const long long per = (n + gridDim.x - 1) / gridDim.x;
  const long long lo = blockIdx.x * per, hi = lo + per < n ? lo + per : n;
  for (int t = 0; t < nthr; t++) {
    const double x = thr[t];
    double acc = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x)
      acc += __dmul_rn(-tanh(__dmul_rn(alpha, __dsub_rn(f[i], x))), w[i]);
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) part[(long long)blockIdx.x * nthr + t] = acc;
  }
}

// buildReweightedInsideField's region sums (toothOptimizer.cpp:318-340):
// per block {w over target-inside cells the fractal misses (fd > 0), w over
// target-inside cells it covers (fd < 0), count of target-outside cells}.
__global__ void __launch_bounds__(CT) region_sums_kernel(const double* __restrict__ md,
                                                         const double* __restrict__ fd,
                                                         const double* __restrict__ w, long long n,
                                                         double* __restrict__ part) {
  __shared__ double sh[CT / 32];
  double poor = 0.0, well = 0.0, outside = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (md[i] < 0) {
      if (fd[i] > 0) poor += w[i];
      if (fd[i] < 0) well += w[i];
    }
    if (md[i] > 0) outside += 1.0;
  }
  poor = block_sum(poor, sh);
  well = block_sum(well, sh);
  outside = block_sum(outside, sh);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = poor;
    part[3 * blockIdx.x + 1] = well;
    part[3 * blockIdx.x + 2] = outside;
  }
}

// The reweighted field (toothOptimizer.cpp:368-381): inside cells scaled by
// their region's factor, every other cell the flat outside value.
__global__ void reweight_kernel(const double* __restrict__ md, const double* __restrict__ fd,
                                const double* __restrict__ w, long long n, double k_poor,
                                double k_well, double outside, double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double v = w[i];
    if (md[i] < 0) {
      if (fd[i] > 0) v = __dmul_rn(v, k_poor);
      if (fd[i] < 0) v = __dmul_rn(v, k_well);
    } else {
      v = outside;
    }
    out[i] = v;
  }
}

// FIELD_3D::setBorders (FIELD_3D.cpp:5357-5379): every boundary cell = value.
__global__ void borders_kernel(double* __restrict__ f, int X, int Y, int Z, double value) {
  const long long n = (long long)X * Y * Z;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((long long)X * Y));
    if (x == 0 || y == 0 || z == 0 || x == X - 1 || y == Y - 1 || z == Z - 1) f[i] = value;
  }
}

// Block partials summed in block order (Neumaier compensation); the loads of
// 16 rows are issued before their additions.
__global__ void reduce_cols_kernel(const double* __restrict__ part, int nblk, int ncol,
                                   double* __restrict__ out) {
  constexpr int U = 16;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  double s = 0.0, comp = 0.0;
  for (int b0 = 0; b0 < nblk; b0 += U) {
    double v[U];
#pragma unroll
    for (int u = 0; u < U; u++) v[u] = b0 + u < nblk ? part[(long long)(b0 + u) * ncol + c] : 0.0;
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (b0 + u >= nblk) break;
      const double t = s + v[u];
      comp += fabs(s) >= fabs(v[u]) ? (s - t) + v[u] : (v[u] - t) + s;
      s = t;
    }
  }
  out[c] = s + comp;
}

int blocks_for(long long n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (n + CT - 1) / CT;
  return (int)(want < 4ll * sms ? (want > 0 ? want : 1) : 4ll * sms);
}

}  // namespace

int conformal_blocks(long long n) { return blocks_for(n); }

cudaError_t launch_shells(const double* dist, int X, int Y, int Z, double* w, cudaStream_t s) {
  shell_kernel<<<blocks_for((long long)X * Y * Z), CT, 0, s>>>(dist, X, Y, Z, w);
  return cudaGetLastError();
}

cudaError_t launch_layer(const double* cur, double* next, int X, int Y, int Z,
                         unsigned long long* zeros_left, cudaStream_t s) {
  layer_kernel<<<blocks_for((long long)X * Y * Z), CT, 0, s>>>(cur, next, X, Y, Z, zeros_left);
  return cudaGetLastError();
}

cudaError_t launch_invert(const double* dist, double* w, long long n, cudaStream_t s) {
  invert_kernel<<<blocks_for(n), CT, 0, s>>>(dist, w, n);
  return cudaGetLastError();
}

cudaError_t launch_side_sums(const double* dist, const double* w, long long n, double scale,
                             double* part, double* out3, cudaStream_t s) {
  const int nb = blocks_for(n);
  sums_kernel<<<nb, CT, 0, s>>>(dist, w, n, scale, part);
  reduce_cols_kernel<<<1, 32, 0, s>>>(part, nb, 3, out3);
  return cudaGetLastError();
}

cudaError_t launch_region_sums(const double* md, const double* fd, const double* w, long long n,
                               double* part, double* out3, cudaStream_t s) {
  const int nb = blocks_for(n);
  region_sums_kernel<<<nb, CT, 0, s>>>(md, fd, w, n, part);
  reduce_cols_kernel<<<1, 32, 0, s>>>(part, nb, 3, out3);
  return cudaGetLastError();
}

cudaError_t launch_reweight(const double* md, const double* fd, const double* w, long long n,
                            double k_poor, double k_well, double outside, double* out,
                            cudaStream_t s) {
  reweight_kernel<<<blocks_for(n), CT, 0, s>>>(md, fd, w, n, k_poor, k_well, outside, out);
  return cudaGetLastError();
}

cudaError_t launch_borders(double* f, int X, int Y, int Z, double value, cudaStream_t s) {
  borders_kernel<<<blocks_for((long long)X * Y * Z), CT, 0, s>>>(f, X, Y, Z, value);
  return cudaGetLastError();
}

cudaError_t launch_scale_sides(const double* dist, double* w, long long n, double scale,
                               double k_in, double k_out, cudaStream_t s) {
  scale_sides_kernel<<<blocks_for(n), CT, 0, s>>>(dist, w, n, scale, k_in, k_out);
  return cudaGetLastError();
}

cudaError_t launch_field_stats(const double* f, long long n, double* part, int* nblk,
                               cudaStream_t s) {
  *nblk = blocks_for(n);
  field_stats_kernel<<<*nblk, CT, 0, s>>>(f, n, part);
  return cudaGetLastError();
}

cudaError_t launch_clamp_infs(double* f, long long n, double mean, cudaStream_t s) {
  clamp_infs_kernel<<<blocks_for(n), CT, 0, s>>>(f, n, mean);
  return cudaGetLastError();
}

cudaError_t launch_lookup(const GridParams& g, const WeightGrid& wg, const double* w, double* out,
                          cudaStream_t s) {
  lookup_kernel<<<blocks_for((long long)g.X * g.Y * g.Z), CT, 0, s>>>(g, wg, w, out);
  return cudaGetLastError();
}

cudaError_t launch_scan(const double* f, const double* w, long long n, const double* thr,
                        int nthr, double alpha, double* part, double* scores, cudaStream_t s) {
  const int nb = blocks_for(n);
  scan_kernel<<<nb, CT, 0, s>>>(f, w, n, thr, nthr, alpha, part);
  reduce_cols_kernel<<<(nthr + 127) / 128, 128, 0, s>>>(part, nb, nthr, scores);
  return cudaGetLastError();
}

}  // namespace qj
