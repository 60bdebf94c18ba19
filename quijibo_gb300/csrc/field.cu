// Escape-time field kernels.
//
// Work unit: a warp tile of 8 (x) by 4 (y) voxels of one z-slice.  Warps
// take tiles from a global counter, so tiles whose voxels iterate long (the
// inside of the set) and tiles that escape at once spread evenly over the
// SMs; the 8x4 footprint keeps the voxels of a warp close, which keeps their
// iteration counts close (a warp runs until its slowest lane escapes).
//
// Kernels:
//   field64_kernel  -- the plain FP64 form: the reference's escape loop
//                      (OPTIMIZE_3D.cpp:1317-1362) with QUATERNION::pow per
//                      root term, reference-exact rounding.
//   field32_kernel  -- the FP32 bulk form: integer exponents by repeated
//                      products, the distance estimate, and a refine list of
//                      voxels that must be recomputed in FP64.
//   refine64_kernel -- FP64 recomputation of the listed voxels.
#include <cuda_runtime.h>
#include <stdint.h>

#include "qj_device.cuh"
#include "qj_kernels.h"

namespace qj {

static constexpr int TILE_X = 8, TILE_Y = 4;

struct TileMap {
  int tx_n, ty_n;  // tiles per row / column of a slice
  long long per_slice, total;
};

__device__ __forceinline__ TileMap tile_map(const GridParams& g) {
  TileMap t;
  t.tx_n = (g.X + TILE_X - 1) / TILE_X;
  t.ty_n = (g.Y + TILE_Y - 1) / TILE_Y;
  t.per_slice = (long long)t.tx_n * t.ty_n;
  t.total = t.per_slice * (g.z1 - g.z0);
  return t;
}

// Next tile for this warp (lane 0 takes it, all lanes get it).
__device__ __forceinline__ long long next_tile(unsigned long long* counter) {
  unsigned long long t = 0;
  if ((threadIdx.x & 31) == 0) t = atomicAdd(counter, 1ull);
  return (long long)__shfl_sync(0xffffffffu, t, 0);
}

__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

// ------------------------------------------------------------------ FP64

// One application of the map in reference order (OPTIMIZE_3D.cpp:1331-1350),
// plus |grad log|R|| for the distance estimate when DE is set.
template <bool POW_REF, bool DE>
__global__ void __launch_bounds__(128) field64_kernel(const __grid_constant__ MapParams m,
                                                      const GridParams g, const IterParams it, double* __restrict__ field,
                                                      float* __restrict__ de, DevStats* st) {
  const TileMap tm = tile_map(g);
  const int lane = threadIdx.x & 31;
  unsigned long long iters_acc = 0;
  for (;;) {
    const long long t = next_tile(&st->tiles_done);
    if (t >= tm.total) break;
    const int zl = (int)(t / tm.per_slice);
    const long long r = t - (long long)zl * tm.per_slice;
    const int x = (int)(r % tm.tx_n) * TILE_X + (lane & 7);
    const int y = (int)(r / tm.tx_n) * TILE_Y + (lane >> 3);
    if (x >= g.X || y >= g.Y) continue;
    const int z = g.z0 + zl;
    double p[3];
    cell_center(g, x, y, z, p);
    int n;
    double d = 0.0;
    const double f = escape64<POW_REF, DE>(m, it, p, g.slice, &n, &d);
    const long long i = ((long long)zl * g.Y + y) * g.X + x;
    field[i] = f;
    if (DE && de) de[i] = (float)d;
    iters_acc += n;
  }
  warp_add(&st->voxel_iters, iters_acc);
}

// FP64 recomputation of the voxels in `list` (local linear indices).
template <bool POW_REF>
__global__ void __launch_bounds__(128) refine64_kernel(const __grid_constant__ MapParams m,
                                                       const GridParams g,
                                                       const IterParams it, const uint32_t* list,
                                                       const DevStats* counts,
                                                       double* __restrict__ field,
                                                       float* __restrict__ de, DevStats* st) {
  const unsigned long long n_list = counts->refined;
  unsigned long long iters_acc = 0;
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n_list;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const uint32_t i = list[k];
    const int x = (int)(i % (uint32_t)g.X);
    const int y = (int)((i / (uint32_t)g.X) % (uint32_t)g.Y);
    const int zl = (int)(i / ((uint32_t)g.X * (uint32_t)g.Y));
    double p[3];
    cell_center(g, x, y, g.z0 + zl, p);
    int n;
    double d = 0.0;
    const double f = escape64<POW_REF, true>(m, it, p, g.slice, &n, &d);
    field[i] = f;
    if (de) de[i] = (float)d;
    iters_acc += n;
  }
  warp_add(&st->aux[0], iters_acc);
}

// ------------------------------------------------------------------ FP32

template <bool DE>
__global__ void __launch_bounds__(128) field32_kernel(const __grid_constant__ MapParams m,
                                                      const GridParams g, const IterParams it, double* __restrict__ field,
                                                      float* __restrict__ de, uint32_t* refine_list,
                                                      int refine, DevStats* st) {
  using namespace q32;
  const TileMap tm = tile_map(g);
  const int lane = threadIdx.x & 31;
  const float esc2 = (float)(it.escape * it.escape);
  const float l2band = log2f((float)it.band), ftol = (float)it.field_tol;
  const float esc_tol = 2e-3f;  // relative, on |q|^2
  unsigned long long iters_acc = 0, nonfinite_acc = 0, lane_iters_acc = 0;
  for (;;) {
    const long long t = next_tile(&st->tiles_done);
    if (t >= tm.total) break;
    const int zl = (int)(t / tm.per_slice);
    const long long r = t - (long long)zl * tm.per_slice;
    const int x = (int)(r % tm.tx_n) * TILE_X + (lane & 7);
    const int y = (int)(r / tm.tx_n) * TILE_Y + (lane >> 3);
    const bool valid = (x < g.X && y < g.Y);
    bool need = false;
    long long i = 0;
    int n_exec = 0;
    if (valid) {
      double p[3];
      cell_center(g, x, y, g.z0 + zl, p);
      Q q = {(float)p[0], (float)p[1], (float)p[2], (float)g.slice};
      float m2 = norm2(q), m2_prev = m2;
      float l2d = 0.f;  // log2 |q_n'|
      int n = 0;
      bool bad = false;
      while (m2 < esc2 && n < it.max_it) {
        float gg = 0.f;
        q = apply32<DE>(m, q, &gg);
        m2_prev = m2;
        m2 = norm2(q);
        if (DE) l2d += 0.5f * (__log2f(gg) + __log2f(m2));
        n++;
        // |q| below 1e-18: |q|^2 nears the bottom of the FP32 range, where
        // FP32 cannot follow the reference's 10*FLT_MIN exit; hand to FP64
        if (m2 < 1e-36f) {
          bad = true;
          break;
        }
      }
      iters_acc += n;
      n_exec = n;
      const float f = 0.5f * logf(m2);
      // d = |q| log|q| / |q'| kept as log2|d|: contracting orbits drive |q'|
      // below the FP32 range long before d itself matters
      float l2abs_d = 0.f, d = 0.f;
      if (DE) {
        l2abs_d = __log2f(fabsf(f)) + 0.5f * __log2f(m2) - l2d;
        d = copysignf(exp2f(l2abs_d), f);
      }
      bad = bad || !isfinite(f) || (DE && isnan(l2abs_d));
      nonfinite_acc += bad;
      // the escape test is a discontinuity: an orbit whose escaping iterate
      // (or the one before it) lies within FP32 error of the escape radius
      // may escape one iteration earlier or later in FP64
      const bool near_escape = n > 0 && m2 >= esc2 &&
                               (fabsf(m2 - esc2) < esc_tol * esc2 || fabsf(m2_prev - esc2) < esc_tol * esc2);
      need = refine && (bad || near_escape || l2abs_d < l2band || fabsf(f) < ftol);
      i = ((long long)zl * g.Y + y) * g.X + x;
      if (!need) {
        field[i] = (double)f;
        if (DE && de) de[i] = d;
      }
    }
    // lane slots the warp spent: 32 x its longest orbit
    const unsigned wmax = __reduce_max_sync(0xffffffffu, (unsigned)n_exec);
    if (lane == 0) lane_iters_acc += 32ull * wmax;
    // warp-aggregated append to the refine list
    const unsigned mask = __ballot_sync(0xffffffffu, need);
    if (mask) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&st->refined, (unsigned long long)__popc(mask));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (need) refine_list[base + __popc(mask & ((1u << lane) - 1u))] = (uint32_t)i;
    }
  }
  warp_add(&st->voxel_iters, iters_acc);
  warp_add(&st->nonfinite, nonfinite_acc);
  warp_add(&st->aux[3], lane_iters_acc);
}

// ------------------------------------------------------------- launchers

static int grid_blocks(const void* fn, int threads) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

cudaError_t launch_field64(const MapParams& m, const GridParams& g, const IterParams& it,
                           bool pow_ref, double* field, float* de, DevStats* st,
                           cudaStream_t s) {
  const void* fn;
  if (pow_ref)
    fn = it.want_de ? (const void*)field64_kernel<true, true> : (const void*)field64_kernel<true, false>;
  else
    fn = it.want_de ? (const void*)field64_kernel<false, true> : (const void*)field64_kernel<false, false>;
  const int blocks = grid_blocks(fn, 128);
  if (pow_ref) {
    if (it.want_de)
      field64_kernel<true, true><<<blocks, 128, 0, s>>>(m, g, it, field, de, st);
    else
      field64_kernel<true, false><<<blocks, 128, 0, s>>>(m, g, it, field, de, st);
  } else {
    if (it.want_de)
      field64_kernel<false, true><<<blocks, 128, 0, s>>>(m, g, it, field, de, st);
    else
      field64_kernel<false, false><<<blocks, 128, 0, s>>>(m, g, it, field, de, st);
  }
  return cudaGetLastError();
}

cudaError_t launch_field32(const MapParams& m, const GridParams& g, const IterParams& it,
                           bool refine, double* field, float* de, uint32_t* list, DevStats* st,
                           cudaStream_t s) {
  const bool want = it.want_de || refine;
  const void* fn = want ? (const void*)field32_kernel<true> : (const void*)field32_kernel<false>;
  const int blocks = grid_blocks(fn, 128);
  if (want)
    field32_kernel<true><<<blocks, 128, 0, s>>>(m, g, it, field, de, list, refine ? 1 : 0, st);
  else
    field32_kernel<false><<<blocks, 128, 0, s>>>(m, g, it, field, de, list, 0, st);
  return cudaGetLastError();
}

cudaError_t launch_refine64(const MapParams& m, const GridParams& g, const IterParams& it,
                            bool pow_ref, const uint32_t* list, double* field, float* de,
                            DevStats* st, cudaStream_t s) {
  const void* fn = pow_ref ? (const void*)refine64_kernel<true> : (const void*)refine64_kernel<false>;
  const int blocks = grid_blocks(fn, 128);
  if (pow_ref)
    refine64_kernel<true><<<blocks, 128, 0, s>>>(m, g, it, list, st, field, de, st);
  else
    refine64_kernel<false><<<blocks, 128, 0, s>>>(m, g, it, list, st, field, de, st);
  return cudaGetLastError();
}

}  // namespace qj
