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
#include "qj_ff.cuh"
#include "qj_kernels.h"

namespace qj {

static constexpr int TILE_X = 8, TILE_Y = 4;

struct TileMap {
  int tx_n, ty_n;  // tiles per row / column of a slice
  long long per_slice, total;
};

__device__ __forceinline__ TileMap tile_map(const GridParams& g, int tile_x = TILE_X) {
  TileMap t;
  t.tx_n = (g.X + tile_x - 1) / tile_x;
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
template <int POW_REF, bool DE>
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
template <int POW_REF>
__global__ void __launch_bounds__(128) refine64_kernel(const __grid_constant__ MapParams m,
                                                       const GridParams g,
                                                       const IterParams it, const uint32_t* list,
                                                       const DevStats* counts,
                                                       double* __restrict__ field,
                                                       float* __restrict__ de, DevStats* st) {
  const unsigned long long n_list = counts->refined;
  unsigned long long iters_acc = 0;
  // the list is sorted by FP32 orbit length: warps take 32-entry chunks
  // (similar orbits, coherent warps) dealt round-robin over the blocks, so
  // every SM gets short and long orbits alike
  const unsigned long long slot = (threadIdx.x >> 5) * (unsigned long long)gridDim.x + blockIdx.x;
  const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
  for (unsigned long long c = slot; c * 32 < n_list; c += warps) {
    const unsigned long long k = c * 32 + (threadIdx.x & 31);
    if (k >= n_list) continue;
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

// Sort key of a refine-list entry: the FP32 orbit length, which predicts the
// FP64 one.
__device__ __forceinline__ uint8_t refine_key(int n) { return (uint8_t)min(n, 255); }

// Escape state of one voxel's FP32 orbit.
struct Orbit32 {
  float m2;           // |q_n|^2
  float l2d;          // log2 |q_n'|
  int n;
  bool live, bad;     // still iterating; FP32 lost the orbit (|q| below 1e-18)
  bool near;          // an iterate before the last lay within FP32 error of the escape radius
  float err;          // first-order relative FP32 error of q_n (with DE)
};

__device__ __forceinline__ Orbit32 orbit_start(bool valid, float m2, float esc2, int max_it) {
  return Orbit32{m2, 0.f, 0, valid && m2 < esc2 && max_it > 0, false, false, q32::EPS32};
}

// One map application's bookkeeping, the loop test of the reference escape
// loop (OPTIMIZE_3D.cpp:1317-1362) included.
template <bool DE>
__device__ __forceinline__ void orbit_step(Orbit32& o, float m2, float gg, float esc2,
                                           int max_it) {
  if (!o.live) return;
  if (DE) {
    o.near = o.near || q32::near_radius(o.m2, esc2, o.err);
    o.err = q32::propagate_err(o.err, gg, o.m2);
    o.l2d += 0.5f * (__log2f(gg) + __log2f(m2));
  }
  o.m2 = m2;
  o.n++;
  // |q| below 1e-18: |q|^2 nears the bottom of the FP32 range, where FP32
  // cannot follow the reference's 10*FLT_MIN exit; hand to FP64
  if (m2 < 1e-36f) {
    o.bad = true;
    o.live = false;
  } else {
    o.live = m2 < esc2 && o.n < max_it;
  }
}

// Where a finished orbit goes.
enum Route : int { WRITTEN = 0, TO_FP64 = 1, TO_FF = 2 };

// Field value, distance estimate and the refine decision of a finished
// orbit; writes the voxel when it stays (WRITTEN).  allow_ff: the voxel may
// go to the double-float re-run (not for re-runs themselves).
template <bool DE>
__device__ __forceinline__ int orbit_finish(const Orbit32& o, const IterParams& it, float esc2,
                                            float l2band, int refine, bool allow_ff, long long i,
                                            double* __restrict__ field, float* __restrict__ de,
                                            unsigned long long& nonfinite_acc) {
  const float f = 0.5f * logf(o.m2);
  // d = |q| log|q| / |q'| kept as log2|d|: contracting orbits drive |q'|
  // below the FP32 range long before d itself matters
  float l2abs_d = 0.f, d = 0.f;
  if (DE) {
    l2abs_d = __log2f(fabsf(f)) + 0.5f * __log2f(o.m2) - o.l2d;
    d = copysignf(exp2f(l2abs_d), f);
  }
  const bool bad = o.bad || !isfinite(f) || (DE && isnan(l2abs_d));
  nonfinite_acc += bad;
  int route = WRITTEN;
  if (refine) {
    // the escape test is a discontinuity: where an iterate lies within FP32
    // error of the escape radius, FP64 may stop the orbit at a different
    // iterate.  The last iterate of an orbit cut by max_it is the same
    // iterate on either side of the radius.
    const bool near_escape =
        DE && (o.near || (o.m2 >= esc2 && o.n < it.max_it && q32::near_radius(o.m2, esc2, o.err)));
    if (bad || near_escape || l2abs_d < l2band || fabsf(f) < it.field_tolf)
      route = TO_FP64;
    else if (it.est_tolf > 0.f && !(o.err <= it.est_tolf * fabsf(f)))
      route = (allow_ff && it.ff_head > 0) ? TO_FF : TO_FP64;
  }
  if (route == WRITTEN) {
    field[i] = (double)f;
    if (DE && de) de[i] = d;
  }
  return route;
}

// Warp-aggregated append of up to two entries per lane (lane order, the a
// entries first) to a list whose length counter is *count.
__device__ __forceinline__ void warp_append(bool a, uint32_t ia, int na, bool b, uint32_t ib,
                                            int nb, unsigned long long* count, uint32_t* list,
                                            uint8_t* keys) {
  const int lane = threadIdx.x & 31;
  const unsigned ma = __ballot_sync(0xffffffffu, a);
  const unsigned mb = __ballot_sync(0xffffffffu, b);
  if (!(ma | mb)) return;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(count, (unsigned long long)(__popc(ma) + __popc(mb)));
  base = __shfl_sync(0xffffffffu, base, 0);
  const unsigned below = (1u << lane) - 1u;
  if (a) {
    const unsigned long long slot = base + __popc(ma & below);
    list[slot] = ia;
    if (keys) keys[slot] = refine_key(na);
  }
  if (b) {
    const unsigned long long slot = base + __popc(ma) + __popc(mb & below);
    list[slot] = ib;
    if (keys) keys[slot] = refine_key(nb);
  }
}

// One voxel per lane: the form the mesher's bisection shares (escape32).
template <bool DE>
__global__ void __launch_bounds__(128) field32_kernel(const __grid_constant__ MapParams m,
                                                      const GridParams g, const IterParams it,
                                                      double* __restrict__ field,
                                                      float* __restrict__ de, RefineLists rl,
                                                      int refine, DevStats* st) {
  using namespace q32;
  const TileMap tm = tile_map(g);
  const int lane = threadIdx.x & 31;
  const float esc2 = (float)(it.escape * it.escape);
  const float l2band = log2f((float)it.band);
  const bool allow_ff = rl.ff != nullptr;
  unsigned long long iters_acc = 0, nonfinite_acc = 0, lane_iters_acc = 0;
  for (;;) {
    const long long t = next_tile(&st->tiles_done);
    if (t >= tm.total) break;
    const int zl = (int)(t / tm.per_slice);
    const long long r = t - (long long)zl * tm.per_slice;
    const int x = (int)(r % tm.tx_n) * TILE_X + (lane & 7);
    const int y = (int)(r / tm.tx_n) * TILE_Y + (lane >> 3);
    const bool valid = (x < g.X && y < g.Y);
    Q q = qff::cell_center_f32(g, x, y, g.z0 + zl);
    Orbit32 o = orbit_start(valid, norm2(q), esc2, it.max_it);
    while (o.live) {
      float gg = 0.f;
      q = apply32<DE>(m, q, &gg);
      orbit_step<DE>(o, norm2(q), gg, esc2, it.max_it);
    }
    iters_acc += o.n;
    const long long i = ((long long)zl * g.Y + y) * g.X + x;
    const int route = valid ? orbit_finish<DE>(o, it, esc2, l2band, refine, allow_ff, i, field,
                                               de, nonfinite_acc)
                            : WRITTEN;
    // lane slots the warp spent: 32 x its longest orbit
    const unsigned wmax = __reduce_max_sync(0xffffffffu, (unsigned)o.n);
    if (lane == 0) lane_iters_acc += 32ull * wmax;
    warp_append(route == TO_FP64, (uint32_t)i, o.n, false, 0, 0, &st->refined, rl.list, rl.keys);
    warp_append(route == TO_FF, (uint32_t)i, 0, false, 0, 0, &st->rerun, rl.ff, nullptr);
  }
  warp_add(&st->voxel_iters, iters_acc);
  warp_add(&st->nonfinite, nonfinite_acc);
  warp_add(&st->aux[3], lane_iters_acc);
}

// Two voxels per lane, (x, y) and (x + 1, y), on the packed f32x2 pipe
// forms: one issue slot does the arithmetic of both orbits, and each orbit
// rounds exactly as in field32_kernel.  Warp tile 16 x 4.  A lane runs until
// both of its orbits stop; the one that stopped first keeps iterating
// unobserved (its state is frozen in its Orbit32).
static constexpr int TILE2_X = 16;

// Per-warp tallies of a bulk pass.
struct BulkAcc {
  unsigned long long iters = 0, nonfinite = 0, lane_iters = 0;
};

// One 16 x 4 tile (tile index t of the launch's z-range) of the two-voxel
// bulk pass; list entries are `tag | local voxel index`.  Returns the
// executed map applications of the warp's voxels (summed over the warp).
template <bool DE, int NT = 0, int NB = 0>
__device__ __forceinline__ unsigned long long tile2(const MapParams& m, const GridParams& g,
                                                    const IterParams& it, long long t,
                                                    double* __restrict__ field,
                                                    float* __restrict__ de, const RefineLists& rl,
                                                    int refine, bool allow_ff, uint32_t tag,
                                                    DevStats* st, BulkAcc& acc, float esc2,
                                                    float l2band) {
  using namespace q32x2;
  const TileMap tm = tile_map(g, TILE2_X);
  const int lane = threadIdx.x & 31;
  const int zl = (int)(t / tm.per_slice);
  const long long r = t - (long long)zl * tm.per_slice;
  const int x = (int)(r % tm.tx_n) * TILE2_X + 2 * (lane & 7);
  const int y = (int)(r / tm.tx_n) * TILE_Y + (lane >> 3);
  const bool va = (x < g.X && y < g.Y), vb = (x + 1 < g.X && y < g.Y);
  // start points from the double-float cell centre: no FP64 at the tile start
  const q32::Q pa = qff::cell_center_f32(g, x, y, g.z0 + zl);
  const q32::Q pb = qff::cell_center_f32(g, x + 1, y, g.z0 + zl);
  Q2 q = join(pa, pb);
  const float2 m20 = norm2(q);
  Orbit32 a = orbit_start(va, m20.x, esc2, it.max_it);
  Orbit32 b = orbit_start(vb, m20.y, esc2, it.max_it);
  while (a.live || b.live) {
    float2 gg = pair(0.f);
    q = apply32x2<DE, NT, NB>(m, q, &gg);
    const float2 m2 = norm2(q);
    orbit_step<DE>(a, m2.x, gg.x, esc2, it.max_it);
    orbit_step<DE>(b, m2.y, gg.y, esc2, it.max_it);
  }
  acc.iters += a.n + b.n;
  const long long i = ((long long)zl * g.Y + y) * g.X + x;
  const int ra = va ? orbit_finish<DE>(a, it, esc2, l2band, refine, allow_ff, i, field, de,
                                       acc.nonfinite)
                    : WRITTEN;
  const int rb = vb ? orbit_finish<DE>(b, it, esc2, l2band, refine, allow_ff, i + 1, field, de,
                                       acc.nonfinite)
                    : WRITTEN;
  // voxel slots the warp spent: 64 x its longest orbit
  const unsigned wmax = __reduce_max_sync(0xffffffffu, (unsigned)max(a.n, b.n));
  if (lane == 0) acc.lane_iters += 64ull * wmax;
  warp_append(ra == TO_FP64, tag | (uint32_t)i, a.n, rb == TO_FP64, tag | (uint32_t)(i + 1), b.n,
              &st->refined, rl.list, rl.keys);
  warp_append(ra == TO_FF, tag | (uint32_t)i, 0, rb == TO_FF, tag | (uint32_t)(i + 1), 0,
              &st->rerun, rl.ff, nullptr);
  return __reduce_add_sync(0xffffffffu, (unsigned)(a.n + b.n));
}

// The unrolled forms (NT > 0) ask for 4 resident blocks per SM: ptxas then
// keeps them at ~110 registers without spills, 3.7% faster at 16 / 8 roots
// (the looped form is unchanged by it).
template <bool DE, int NT = 0, int NB = 0>
__global__ void __launch_bounds__(128, NT > 0 ? 4 : 0) field32x2_kernel(const __grid_constant__ MapParams m,
                                                        const GridParams g, const IterParams it,
                                                        double* __restrict__ field,
                                                        float* __restrict__ de, RefineLists rl,
                                                        int refine, DevStats* st) {
  const TileMap tm = tile_map(g, TILE2_X);
  const bool allow_ff = rl.ff != nullptr;
  const float esc2 = (float)(it.escape * it.escape), l2band = log2f((float)it.band);
  BulkAcc acc;
  for (;;) {
    const long long t = next_tile(&st->tiles_done);
    if (t >= tm.total) break;
    tile2<DE, NT, NB>(m, g, it, t, field, de, rl, refine, allow_ff, 0u, st, acc, esc2, l2band);
  }
  warp_add(&st->voxel_iters, acc.iters);
  warp_add(&st->nonfinite, acc.nonfinite);
  warp_add(&st->aux[3], acc.lane_iters);
}

// The double-float re-run of the listed voxels: it.ff_head map applications
// in double-float, then FP32 to the end, one voxel per lane.  The tracked
// error restarts at the rounding of the head's result to FP32, so voxels
// whose error came from the first iterations now pass; the others (and the
// band, escape-radius and overflow cases) go to the FP64 list.
// One re-run voxel (local index i); returns its route (WRITTEN or TO_FP64)
// and leaves its orbit in *o.
__device__ __forceinline__ int rerun_voxel(const MapParams& m, const GridParams& g,
                                           const IterParams& it, float esc2, float l2band,
                                           uint32_t i, double* __restrict__ field,
                                           float* __restrict__ de, Orbit32* o,
                                           unsigned long long& nonfinite_acc) {
  const int x = (int)(i % (uint32_t)g.X);
  const int y = (int)((i / (uint32_t)g.X) % (uint32_t)g.Y);
  const int zl = (int)(i / ((uint32_t)g.X * (uint32_t)g.Y));
  qff::Q q = qff::cell_center_ff(g, x, y, g.z0 + zl);
  *o = orbit_start(true, qff::norm2(q).hi, esc2, it.max_it);
  for (int h = 0; h < it.ff_head && o->live; h++) {
    float gg = 0.f;
    q = apply_ff<true>(m, q, &gg);
    o->err = q32::EPS32;  // double-float iterates: only their FP32 rounding counts
    orbit_step<true>(*o, qff::norm2(q).hi, gg, esc2, it.max_it);
  }
  o->err = q32::EPS32;
  q32::Q qf = qff::hi(q);
  while (o->live) {
    float gg = 0.f;
    qf = apply32<true>(m, qf, &gg);
    orbit_step<true>(*o, q32::norm2(qf), gg, esc2, it.max_it);
  }
  return orbit_finish<true>(*o, it, esc2, l2band, 1, false, i, field, de, nonfinite_acc);
}

// rerun_voxel for two listed voxels on one lane (b may be absent), on packed
// f32x2 operands: each voxel gets the bits of rerun_voxel.
__device__ __forceinline__ void rerun_pair(const MapParams& m, const GridParams& g,
                                           const IterParams& it, float esc2, float l2band,
                                           uint32_t ia, bool vb, uint32_t ib,
                                           double* __restrict__ field, float* __restrict__ de,
                                           Orbit32* oa, Orbit32* ob, int* ra, int* rb,
                                           unsigned long long& nonfinite_acc) {
  auto centre = [&](uint32_t i) {
    const int x = (int)(i % (uint32_t)g.X);
    const int y = (int)((i / (uint32_t)g.X) % (uint32_t)g.Y);
    const int zl = (int)(i / ((uint32_t)g.X * (uint32_t)g.Y));
    return qff::cell_center_ff(g, x, y, g.z0 + zl);
  };
  const qff::Q qa = centre(ia);
  qff2::Q q = qff2::join(qa, vb ? centre(ib) : qa);
  qff2::F2 n2 = qff2::norm2(q);
  *oa = orbit_start(true, n2.hi.x, esc2, it.max_it);
  *ob = orbit_start(vb, n2.hi.y, esc2, it.max_it);
  for (int h = 0; h < it.ff_head && (oa->live || ob->live); h++) {
    float2 gg = q32x2::pair(0.f);
    q = apply_ff2<true>(m, q, &gg);
    oa->err = q32::EPS32;  // double-float iterates: only their FP32 rounding counts
    ob->err = q32::EPS32;
    n2 = qff2::norm2(q);
    orbit_step<true>(*oa, n2.hi.x, gg.x, esc2, it.max_it);
    orbit_step<true>(*ob, n2.hi.y, gg.y, esc2, it.max_it);
  }
  oa->err = q32::EPS32;
  ob->err = q32::EPS32;
  q32x2::Q2 qf = qff2::hi(q);
  while (oa->live || ob->live) {
    float2 gg = q32x2::pair(0.f);
    qf = apply32x2<true>(m, qf, &gg);
    const float2 m2 = q32x2::norm2(qf);
    orbit_step<true>(*oa, m2.x, gg.x, esc2, it.max_it);
    orbit_step<true>(*ob, m2.y, gg.y, esc2, it.max_it);
  }
  *ra = orbit_finish<true>(*oa, it, esc2, l2band, 1, false, ia, field, de, nonfinite_acc);
  *rb = vb ? orbit_finish<true>(*ob, it, esc2, l2band, 1, false, ib, field, de, nonfinite_acc)
           : WRITTEN;
}

// Two consecutive list entries per lane.
__global__ void __launch_bounds__(128) rerun_ff_kernel(const __grid_constant__ MapParams m,
                                                       const GridParams g, const IterParams it,
                                                       const uint32_t* __restrict__ ff_list,
                                                       double* __restrict__ field,
                                                       float* __restrict__ de, uint32_t* list,
                                                       uint8_t* keys, DevStats* st) {
  const unsigned long long n_list = st->rerun;
  const int lane = threadIdx.x & 31;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x * 2;
  unsigned long long iters_acc = 0, nonfinite_acc = 0;
  const float esc2 = (float)(it.escape * it.escape), l2band = log2f((float)it.band);
  // warp-uniform trips: the append below is a warp collective
  for (unsigned long long base =
           ((blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) & ~31ull) * 2;
       base < n_list; base += stride) {
    const unsigned long long k = base + 2 * lane;
    uint32_t ia = 0, ib = 0;
    int ra = WRITTEN, rb = WRITTEN;
    Orbit32 oa = orbit_start(false, 0.f, 0.f, 0), ob = oa;
    if (k < n_list) {
      ia = ff_list[k];
      const bool vb = k + 1 < n_list;
      if (vb) ib = ff_list[k + 1];
      rerun_pair(m, g, it, esc2, l2band, ia, vb, ib, field, de, &oa, &ob, &ra, &rb,
                 nonfinite_acc);
      iters_acc += oa.n + ob.n;
    }
    warp_append(ra == TO_FP64, ia, oa.n, rb == TO_FP64, ib, ob.n, &st->refined, list, keys);
  }
  warp_add(&st->rerun_iters, iters_acc);
  warp_add(&st->nonfinite, nonfinite_acc);
}

// ------------------------------------------------------------- batches
// Several field requests (different grids and maps) in one pass: the tiles
// of all items form one work queue, list entries carry the item in their top
// bits (BATCH_SHIFT), and each kernel reads the item's map and grid from the
// batch table in global memory.  Per voxel, the arithmetic is that of the
// single-request kernels, so each item's field has the same bits as its own
// qjg_field call.

// the item owning tile t (largest k with tile0[k] <= t)
__device__ __forceinline__ int batch_item(const long long* tile0, int n, long long t) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tile0[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <bool DE>
__global__ void __launch_bounds__(128) field32x2_batch_kernel(const BatchTable* __restrict__ tab,
                                                              const MapParams* __restrict__ maps,
                                                              RefineLists rl,
                                                              BatchCounts* __restrict__ counts,
                                                              DevStats* st) {
  __shared__ long long tile0[BATCH_MAX];
  const int n = tab->n;
  for (int k = threadIdx.x; k < n; k += blockDim.x) tile0[k] = tab->items[k].tile0;
  __syncthreads();
  const long long total = tab->total_tiles;
  BulkAcc acc;
  for (;;) {
    const long long t = next_tile(&st->tiles_done);
    if (t >= total) break;
    const int k = batch_item(tile0, n, t);
    const BatchItem& b = tab->items[k];
    const MapParams& m = maps[k];
    const bool allow_ff = rl.ff != nullptr && b.refine && m.all_int && b.it.est_tol > 0.0;
    const unsigned long long it_sum =
        tile2<DE>(m, b.g, b.it, t - tile0[k], b.field, b.de, rl, b.refine, allow_ff,
                  (uint32_t)k << BATCH_SHIFT, st, acc, (float)(b.it.escape * b.it.escape),
                  log2f((float)b.it.band));
    if ((threadIdx.x & 31) == 0) atomicAdd(&counts[k].voxel_iters, it_sum);
  }
  warp_add(&st->voxel_iters, acc.iters);
  warp_add(&st->nonfinite, acc.nonfinite);
  warp_add(&st->aux[3], acc.lane_iters);
}

__global__ void __launch_bounds__(128) rerun_ff_batch_kernel(const BatchTable* __restrict__ tab,
                                                             const MapParams* __restrict__ maps,
                                                             const uint32_t* __restrict__ ff_list,
                                                             uint32_t* list, uint8_t* keys,
                                                             DevStats* st) {
  const unsigned long long n_list = st->rerun;
  const int lane = threadIdx.x & 31;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long iters_acc = 0, nonfinite_acc = 0;
  for (unsigned long long base = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) & ~31ull;
       base < n_list; base += stride) {
    const unsigned long long j = base + lane;
    uint32_t e = 0;
    int route = WRITTEN;
    Orbit32 o = orbit_start(false, 0.f, 0.f, 0);
    if (j < n_list) {
      e = ff_list[j];
      const int k = (int)(e >> BATCH_SHIFT);
      const BatchItem& b = tab->items[k];
      route = rerun_voxel(maps[k], b.g, b.it, (float)(b.it.escape * b.it.escape),
                          log2f((float)b.it.band), e & BATCH_MASK, b.field, b.de, &o,
                          nonfinite_acc);
      iters_acc += o.n;
    }
    warp_append(route == TO_FP64, e, o.n, false, 0, 0, &st->refined, list, keys);
  }
  warp_add(&st->rerun_iters, iters_acc);
  warp_add(&st->nonfinite, nonfinite_acc);
}

// FP64 re-evaluation of batch entries (integer exponents by products: the
// batch admits only maps whose effective exponents are integers).
__global__ void __launch_bounds__(128) refine64_batch_kernel(const BatchTable* __restrict__ tab,
                                                             const MapParams* __restrict__ maps,
                                                             const uint32_t* list,
                                                             DevStats* st) {
  const unsigned long long n_list = st->refined;
  unsigned long long iters_acc = 0;
  // sorted list: 32-entry chunks dealt round-robin over the blocks (as refine64_kernel)
  const unsigned long long slot = (threadIdx.x >> 5) * (unsigned long long)gridDim.x + blockIdx.x;
  const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x >> 5);
  for (unsigned long long c = slot; c * 32 < n_list; c += warps) {
    const unsigned long long j = c * 32 + (threadIdx.x & 31);
    if (j >= n_list) continue;
    const uint32_t e = list[j];
    const int k = (int)(e >> BATCH_SHIFT);
    const uint32_t i = e & BATCH_MASK;
    const BatchItem& b = tab->items[k];
    const GridParams& g = b.g;
    const int x = (int)(i % (uint32_t)g.X);
    const int y = (int)((i / (uint32_t)g.X) % (uint32_t)g.Y);
    const int zl = (int)(i / ((uint32_t)g.X * (uint32_t)g.Y));
    double p[3];
    cell_center(g, x, y, g.z0 + zl, p);
    int n;
    double d = 0.0;
    const double f = escape64<false, true>(maps[k], b.it, p, g.slice, &n, &d);
    b.field[i] = f;
    if (b.de) b.de[i] = (float)d;
    iters_acc += n;
  }
  warp_add(&st->aux[0], iters_acc);
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
                           int pow_mode, double* field, float* de, DevStats* st,
                           cudaStream_t s) {
#define QJ_F64(P)                                                                              \
  do {                                                                                         \
    const void* fn = it.want_de ? (const void*)field64_kernel<P, true>                          \
                                : (const void*)field64_kernel<P, false>;                       \
    const int blocks = grid_blocks(fn, 128);                                                   \
    if (it.want_de)                                                                            \
      field64_kernel<P, true><<<blocks, 128, 0, s>>>(m, g, it, field, de, st);                 \
    else                                                                                       \
      field64_kernel<P, false><<<blocks, 128, 0, s>>>(m, g, it, field, de, st);                \
  } while (0)
  if (pow_mode == 2)
    QJ_F64(2);
  else if (pow_mode == 1)
    QJ_F64(1);
  else
    QJ_F64(0);
#undef QJ_F64
  return cudaGetLastError();
}

// 1: field32x2_kernel (the default), 0: field32_kernel
static int g_field32_pairs = 1;

void set_field32_pairs(int on) { g_field32_pairs = on ? 1 : 0; }

cudaError_t launch_field32(const MapParams& m, const GridParams& g, const IterParams& it,
                           bool refine, double* field, float* de, uint32_t* list, uint8_t* keys,
                           uint32_t* ff_list, DevStats* st, cudaStream_t s) {
  const bool want = it.want_de || refine;
  const int r = refine ? 1 : 0;
  // the double-float head needs integer exponents and an error target
  const RefineLists rl = {list, keys, (refine && m.all_int && it.est_tol > 0.0) ? ff_list : nullptr};
  if (g_field32_pairs) {
    // root counts of the benchmark maps compiled in: the precision form's
    // 16 / 8 and the plain form's 8 / 0 fully unrolled (5% faster at 16 / 8),
    // the large form's 48 / 24 two pairs per trip (8% faster; fully unrolled
    // it ran 38% slower, instruction fetch); other maps read their counts
#define QJ_F32X2(NT, NB)                                                                   \
  do {                                                                                     \
    const void* fn = want ? (const void*)field32x2_kernel<true, NT, NB>                   \
                          : (const void*)field32x2_kernel<false, NT, NB>;                 \
    const int blocks = grid_blocks(fn, 128);                                               \
    if (want)                                                                              \
      field32x2_kernel<true, NT, NB><<<blocks, 128, 0, s>>>(m, g, it, field, de, rl, r, st); \
    else                                                                                   \
      field32x2_kernel<false, NT, NB><<<blocks, 128, 0, s>>>(m, g, it, field, de, rl, 0, st); \
  } while (0)
    if (m.lagrange)
      QJ_F32X2(0, 0);
    else if (m.nt == 16 && m.nb == 8)
      QJ_F32X2(16, 8);
    else if (m.nt == 8 && m.nb == 0)
      QJ_F32X2(8, 0);
    else if (m.nt == 48 && m.nb == 24)
      QJ_F32X2(48, 24);
    else
      QJ_F32X2(0, 0);
#undef QJ_F32X2
    return cudaGetLastError();
  }
  const void* fn = want ? (const void*)field32_kernel<true> : (const void*)field32_kernel<false>;
  const int blocks = grid_blocks(fn, 128);
  if (want)
    field32_kernel<true><<<blocks, 128, 0, s>>>(m, g, it, field, de, rl, r, st);
  else
    field32_kernel<false><<<blocks, 128, 0, s>>>(m, g, it, field, de, rl, 0, st);
  return cudaGetLastError();
}

cudaError_t launch_rerun_ff(const MapParams& m, const GridParams& g, const IterParams& it,
                            const uint32_t* ff_list, double* field, float* de, uint32_t* list,
                            uint8_t* keys, DevStats* st, cudaStream_t s) {
  const int blocks = grid_blocks((const void*)rerun_ff_kernel, 128);
  rerun_ff_kernel<<<blocks, 128, 0, s>>>(m, g, it, ff_list, field, de, list, keys, st);
  return cudaGetLastError();
}

// ------------------------------------------------------ refine-list order
// A refine warp runs until its longest orbit ends, and the list comes out of
// the FP32 pass in tile order, where 1-iteration and 40-iteration orbits
// share warps.  A counting sort by the FP32 orbit length (longest first)
// gives each refine warp orbits of one length.

__global__ void __launch_bounds__(256) refine_hist_kernel(const uint8_t* __restrict__ keys,
                                                          const DevStats* counts,
                                                          unsigned* __restrict__ hist) {
  __shared__ unsigned sh[REFINE_KEYS];
  for (int k = threadIdx.x; k < REFINE_KEYS; k += blockDim.x) sh[k] = 0;
  __syncthreads();
  const unsigned long long n = counts->refined;
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x)
    atomicAdd(&sh[keys[k]], 1u);
  __syncthreads();
  for (int k = threadIdx.x; k < REFINE_KEYS; k += blockDim.x)
    if (sh[k]) atomicAdd(&hist[k], sh[k]);
}

// Counts -> first output slot of each key, largest key first (one block of
// REFINE_KEYS threads; Hillis-Steele scan in shared memory).
__global__ void __launch_bounds__(REFINE_KEYS) refine_offsets_kernel(unsigned* hist) {
  __shared__ unsigned sh[REFINE_KEYS];
  const int t = threadIdx.x;
  const int key = REFINE_KEYS - 1 - t;
  const unsigned c = hist[key];
  sh[t] = c;
  __syncthreads();
  for (int o = 1; o < REFINE_KEYS; o <<= 1) {
    const unsigned v = t >= o ? sh[t - o] : 0u;
    __syncthreads();
    sh[t] += v;
    __syncthreads();
  }
  hist[key] = sh[t] - c;
}

// Scatter into key order; lanes with equal keys share one cursor update.
__global__ void __launch_bounds__(256) refine_scatter_kernel(const uint32_t* __restrict__ list,
                                                             const uint8_t* __restrict__ keys,
                                                             const DevStats* counts,
                                                             unsigned* __restrict__ cursor,
                                                             uint32_t* __restrict__ out) {
  const unsigned long long n = counts->refined;
  const int lane = threadIdx.x & 31;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long base = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) & ~31ull;
       base < n; base += stride) {
    const unsigned long long k = base + lane;
    const bool v = k < n;
    const int key = v ? (int)keys[k] : REFINE_KEYS;  // idle lanes group apart
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    unsigned pos = 0;
    if (v && lane == leader) pos = atomicAdd(&cursor[key], (unsigned)__popc(peers));
    pos = __shfl_sync(0xffffffffu, pos, leader);
    if (v) out[pos + __popc(peers & ((1u << lane) - 1u))] = list[k];
  }
}

static int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

cudaError_t launch_refine64(const MapParams& m, const GridParams& g, const IterParams& it,
                            int pow_mode, const uint32_t* list, const uint8_t* keys,
                            uint32_t* sorted, unsigned* hist, double* field, float* de,
                            DevStats* st, cudaStream_t s) {
  if (keys) {
    cudaError_t e = cudaMemsetAsync(hist, 0, REFINE_KEYS * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    const int blocks = 2 * sm_count();
    refine_hist_kernel<<<blocks, 256, 0, s>>>(keys, st, hist);
    refine_offsets_kernel<<<1, REFINE_KEYS, 0, s>>>(hist);
    refine_scatter_kernel<<<blocks, 256, 0, s>>>(list, keys, st, hist, sorted);
    list = sorted;
  }
#define QJ_R64(P)                                                                    \
  do {                                                                               \
    const int blocks = grid_blocks((const void*)refine64_kernel<P>, 128);            \
    refine64_kernel<P><<<blocks, 128, 0, s>>>(m, g, it, list, st, field, de, st);    \
  } while (0)
  if (pow_mode == 2)
    QJ_R64(2);
  else if (pow_mode == 1)
    QJ_R64(1);
  else
    QJ_R64(0);
#undef QJ_R64
  return cudaGetLastError();
}

BatchShapes batch_shapes() {
  BatchShapes sh;
  sh.bulk = grid_blocks((const void*)field32x2_batch_kernel<true>, 128);
  sh.rerun = grid_blocks((const void*)rerun_ff_batch_kernel, 128);
  sh.sort = 2 * sm_count();
  sh.refine = grid_blocks((const void*)refine64_batch_kernel, 128);
  return sh;
}

long long batch_item_tiles(int X, int Y, int Z) {
  return (long long)((X + TILE2_X - 1) / TILE2_X) * ((Y + TILE_Y - 1) / TILE_Y) * Z;
}

cudaError_t launch_field_batch(const BatchBuffers& b, const BatchShapes& sh, cudaStream_t s) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(b.st, 0, sizeof(DevStats), s))) return e;
  if ((e = cudaMemsetAsync(b.counts, 0, BATCH_MAX * sizeof(BatchCounts), s))) return e;
  field32x2_batch_kernel<true><<<sh.bulk, 128, 0, s>>>(b.tab, b.maps, b.rl, b.counts, b.st);
  rerun_ff_batch_kernel<<<sh.rerun, 128, 0, s>>>(b.tab, b.maps, b.rl.ff, b.rl.list, b.rl.keys,
                                                 b.st);
  if ((e = cudaMemsetAsync(b.hist, 0, REFINE_KEYS * sizeof(unsigned), s))) return e;
  refine_hist_kernel<<<sh.sort, 256, 0, s>>>(b.rl.keys, b.st, b.hist);
  refine_offsets_kernel<<<1, REFINE_KEYS, 0, s>>>(b.hist);
  refine_scatter_kernel<<<sh.sort, 256, 0, s>>>(b.rl.list, b.rl.keys, b.st, b.hist, b.sorted);
  refine64_batch_kernel<<<sh.refine, 128, 0, s>>>(b.tab, b.maps, b.sorted, b.st);
  return cudaGetLastError();
}

}  // namespace qj
