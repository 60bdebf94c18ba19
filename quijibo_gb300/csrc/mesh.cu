// Marching cubes as a classify / scan-compact / emit pipeline over z-slabs.
//
// Reference: TRIANGLE_MESH's three mesher families
//   computeNonlinearMarchingCubesLowMemoryHuge (TRIANGLE_MESH.cpp:681-768,
//     slices from computeAllLowMemorySlicesHuge :4884-4948),
//   computeNonlinearMarchingCubes (:152-275) and
//   computeStagedMarchingCubes (:989-1114).
// All three classify a cube by the signs (> 0) of its eight corner values,
// place one vertex on every edge that some cube's case uses, number the
// vertices in ascending (z, y, x, axis) order of the edge's lower endpoint
// (the iteration order of the reference's std::map of (VEC3I, VEC3I) or
// (int, int) edge keys), emit each cube's triangles in scan order, and drop
// triangles with an edge shorter than 1e-7.  Vertices come from linear
// interpolation of stored values (computeEdgeInterpolations :2373-2425) or
// from the bisection of TRIANGLE_MESH::midpointSearch (:2232-2271) on the map.
//
// Slab window (cube layers [c0, c1) per slab; "window index" j <-> global
// index c0 - 1 + j): flags of layers c0-1 .. c1-1, edge masks and vertex ids
// of planes c0-1 .. c1 (plane/layer c0-1 is carried over from the previous
// slab).  Each slab numbers the vertices of planes [c0, c1) (the last slab
// also plane Z-1) and emits the triangles of layers [c0-1, c1-1) (the last
// slab also layer c1-1), whose vertices all have ids by then.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#define QJ_MC_STORAGE static __constant__
#include "mc_cases.h"
#include "qj_device.cuh"
#include "qj_ff.cuh"
#include "qj_mesh.h"

namespace qj {

namespace {

constexpr int SCAN_T = 256;              // threads per scan block
constexpr int SCAN_V = 8;                // items per thread
constexpr int SCAN_B = SCAN_T * SCAN_V;  // items per scan block

// Edge id (1..12) -> lower-endpoint corner offset and axis (0=x, 1=y, 2=z),
// TRIANGLE_MESH::getVertexTriplets, TRIANGLE_MESH.cpp:1569-1665.
__constant__ signed char c_edge_off[13][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 1}, {0, 1, 0},
                                              {1, 0, 0}, {1, 0, 0}, {1, 0, 1}, {1, 1, 0}, {0, 1, 0},
                                              {0, 0, 0}, {0, 0, 1}, {0, 1, 1}};
__constant__ signed char c_edge_axis[13] = {0, 1, 2, 1, 2, 1, 2, 1, 2, 0, 0, 0, 0};

__device__ __forceinline__ int ntri_of(int flag) {
  int n = 0;
#pragma unroll
  for (int t = 0; t < QJ_MC_MAX_TRIS; t++) n += QJ_MC_CASES[flag][3 * t] != 0;
  return n;
}

// Exclusive scan across a block of SCAN_T threads; returns the thread's
// exclusive prefix and writes the block total to *total.
__device__ __forceinline__ long long block_exclusive_scan(long long v, long long* total) {
  __shared__ long long warp_sums[SCAN_T / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long n = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += n;
  }
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    long long w = lane < SCAN_T / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long n = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += n;
    }
    if (lane < SCAN_T / 32) warp_sums[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  const long long warp_base = warp ? warp_sums[warp - 1] : 0;
  *total = warp_sums[SCAN_T / 32 - 1];
  __syncthreads();
  return warp_base + inc - v;
}

// Generic pass 1: per-block sums of op.count(i) over items [0, n).
template <class Op>
__global__ void __launch_bounds__(SCAN_T) count_kernel(Op op, long long n, long long* bsum) {
  const long long base = (long long)blockIdx.x * SCAN_B + (long long)threadIdx.x * SCAN_V;
  long long c = 0;
#pragma unroll
  for (int k = 0; k < SCAN_V; k++)
    if (base + k < n) c += op.count(base + k);
  long long total;
  block_exclusive_scan(c, &total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// Pass 2: exclusive scan of the nb block sums in place; bsum[nb] = total.
__global__ void __launch_bounds__(1024) scan_bsum_kernel(long long* bsum, long long nb) {
  __shared__ long long sh[32];
  __shared__ long long carry_sh;
  if (threadIdx.x == 0) carry_sh = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long c0 = 0; c0 < nb; c0 += 1024) {
    const long long i = c0 + threadIdx.x;
    const long long v = i < nb ? bsum[i] : 0;
    long long inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) sh[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      long long w = sh[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      sh[lane] = w;
    }
    __syncthreads();
    const long long carry = carry_sh;
    const long long excl = carry + (warp ? sh[warp - 1] : 0) + inc - v;
    if (i < nb) bsum[i] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry_sh = carry + sh[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[nb] = carry_sh;
}

// Generic pass 3: op.emit(i, k) with k = running + exclusive prefix of
// op.count over items [0, n).
template <class Op>
__global__ void __launch_bounds__(SCAN_T) emit_kernel(Op op, long long n, const long long* bsum,
                                                      long long running) {
  const long long base = (long long)blockIdx.x * SCAN_B + (long long)threadIdx.x * SCAN_V;
  int c[SCAN_V];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_V; k++) {
    c[k] = base + k < n ? op.count(base + k) : 0;
    s += c[k];
  }
  long long total;
  long long k0 = running + bsum[blockIdx.x] + block_exclusive_scan(s, &total);
#pragma unroll
  for (int k = 0; k < SCAN_V; k++) {
    if (c[k]) op.emit(base + k, k0);
    k0 += c[k];
  }
}

// ------------------------------------------------------------ classify

// flags[l * XY + y * X + x] for layers l of `src` planes l and l+1.  One
// thread per (x, y) walks the layers: the four corners of plane l+1 are
// loaded once and reused as the lower corners of the next layer (4 loads per
// cube instead of 8, of which the x+1 pair hits L1 behind the neighbouring
// lane; rows are read coalesced across the warp).
__device__ __forceinline__ int plane_bits(const double* u, int X) {
  // corner weights NNN=1 NNP=2 NPN=4 NPP=8 PNN=16 PNP=32 PPN=64 PPP=128
  // (TRIANGLE_MESH.cpp:4929-4931; letters x, y, z): the z-lower corners
  return (u[0] > 0) | ((u[X] > 0) << 2) | ((u[1] > 0) << 4) | ((u[1 + X] > 0) << 6);
}

__global__ void __launch_bounds__(128) flags_kernel(const double* __restrict__ src, int X, int Y,
                                                    long long n_layers,
                                                    uint8_t* __restrict__ flags) {
  const long long XY = (long long)X * Y;
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= XY) return;
  const int y = (int)(p / X), x = (int)(p - (long long)y * X);
  if (x >= X - 1 || y >= Y - 1) {
    for (long long l = 0; l < n_layers; l++) flags[l * XY + p] = 0;
    return;
  }
  int lo = plane_bits(src + p, X);
#pragma unroll 4
  for (long long l = 0; l < n_layers; l++) {
    const int hi = plane_bits(src + (l + 1) * XY + p, X);
    flags[l * XY + p] = (uint8_t)(lo | (hi << 1));
    lo = hi;
  }
}

// Edge masks of window planes [j0, j0 + n/XY): bit a set when the edge from
// the voxel along axis a carries a vertex.  Flags window layer j-1 and j are
// the cube layers below and above plane j; layers outside [lay_lo, lay_hi)
// do not exist.
struct MaskCount {
  const uint8_t* flags;
  uint8_t* masks;
  int X, Y;
  int j0, lay_lo, lay_hi;
  __device__ int flag(int j, int x, int y) const {
    if (j < lay_lo || j >= lay_hi || x < 0 || y < 0 || x > X - 2 || y > Y - 2) return 0;
    return flags[((long long)j * Y + y) * X + x];
  }
  // item i at window plane j, column x, row y
  __device__ int count_at(long long i, int j, int x, int y) const {
    const long long XY = (long long)X * Y;
    // x-edge: edges 10 (cube x,y,j), 9 (x,y-1,j), 11 (x,y,j-1), 12 (x,y-1,j-1)
    const bool ex = (QJ_MC_EDGEMASK[flag(j, x, y)] >> 9 & 1) |
                    (QJ_MC_EDGEMASK[flag(j, x, y - 1)] >> 8 & 1) |
                    (QJ_MC_EDGEMASK[flag(j - 1, x, y)] >> 10 & 1) |
                    (QJ_MC_EDGEMASK[flag(j - 1, x, y - 1)] >> 11 & 1);
    // y-edge: edges 1 (x,y,j), 5 (x-1,y,j), 3 (x,y,j-1), 7 (x-1,y,j-1)
    const bool ey = (QJ_MC_EDGEMASK[flag(j, x, y)] >> 0 & 1) |
                    (QJ_MC_EDGEMASK[flag(j, x - 1, y)] >> 4 & 1) |
                    (QJ_MC_EDGEMASK[flag(j - 1, x, y)] >> 2 & 1) |
                    (QJ_MC_EDGEMASK[flag(j - 1, x - 1, y)] >> 6 & 1);
    // z-edge: edges 2 (x,y,j), 6 (x-1,y,j), 4 (x,y-1,j), 8 (x-1,y-1,j)
    const bool ez = (QJ_MC_EDGEMASK[flag(j, x, y)] >> 1 & 1) |
                    (QJ_MC_EDGEMASK[flag(j, x - 1, y)] >> 5 & 1) |
                    (QJ_MC_EDGEMASK[flag(j, x, y - 1)] >> 3 & 1) |
                    (QJ_MC_EDGEMASK[flag(j, x - 1, y - 1)] >> 7 & 1);
    const int m = (int)ex | ((int)ey << 1) | ((int)ez << 2);
    masks[(long long)j0 * XY + i] = (uint8_t)m;
    return __popc(m);
  }
};

// Pass 1 of the vertex-id scan over MaskCount, with the item coordinates
// advanced along x from one division per thread instead of three per item.
__global__ void __launch_bounds__(SCAN_T) mask_count_kernel(MaskCount op, long long n,
                                                            long long* bsum) {
  const long long base = (long long)blockIdx.x * SCAN_B + (long long)threadIdx.x * SCAN_V;
  long long c = 0;
  if (base < n) {
    const long long XY = (long long)op.X * op.Y;
    int j = (int)(base / XY);
    const int r = (int)(base - j * XY);
    int y = r / op.X, x = r - y * op.X;
    j += op.j0;
#pragma unroll
    for (int k = 0; k < SCAN_V; k++) {
      if (base + k < n) c += op.count_at(base + k, j, x, y);
      if (++x == op.X) {
        x = 0;
        if (++y == op.Y) {
          y = 0;
          j++;
        }
      }
    }
  }
  long long total;
  block_exclusive_scan(c, &total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// Vertex ids (global) of window planes [j0, ...) and the list of their edges
// (window voxel index * 4 + axis) in id order.
struct VertexEmit {
  const uint8_t* masks;
  int32_t* vbase;
  uint32_t* list;
  long long list_base;  // global id of list[0]
  long long XY;
  int j0;
  __device__ int count(long long i) const { return __popc(masks[j0 * XY + i]); }
  __device__ void emit(long long i, long long k) const {
    const long long w = j0 * XY + i;
    const int m = masks[w];
    vbase[w] = (int32_t)k;
    long long o = k - list_base;
#pragma unroll
    for (int a = 0; a < 3; a++)
      if (m >> a & 1) list[o++] = (uint32_t)(w * 4 + a);
  }
};

struct TriCount {
  const uint8_t* flags;
  long long XY;
  int j0;
  __device__ int count(long long i) const { return ntri_of(flags[j0 * XY + i]); }
};

struct TriEmit {
  const uint8_t* flags;
  const uint8_t* masks;
  const int32_t* vbase;
  int32_t* tris;
  long long cap;
  int X;
  long long XY;
  int j0;
  __device__ int count(long long i) const { return ntri_of(flags[j0 * XY + i]); }
  __device__ void emit(long long i, long long k) const {
    const long long w = j0 * XY + i;
    const int f = flags[w];
    const int r = (int)(i % XY);
    const int x = r % X, y = r / X, j = j0 + (int)(i / XY);
    for (int t = 0; t < QJ_MC_MAX_TRIS && QJ_MC_CASES[f][3 * t]; t++, k++) {
      if (k >= cap) continue;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const int e = QJ_MC_CASES[f][3 * t + c];
        const long long v = ((long long)(j + c_edge_off[e][2]) * XY) +
                            (long long)(y + c_edge_off[e][1]) * X + (x + c_edge_off[e][0]);
        const int a = c_edge_axis[e];
        tris[3 * k + c] = vbase[v] + __popc(masks[v] & ((1 << a) - 1));
      }
    }
  }
};

// Degenerate-triangle filter of TRIANGLE_MESH.cpp:737-756 (edge < 1e-7).
__device__ __forceinline__ double edge_len(const double* a, const double* b) {
  using namespace q64;
  const double d0 = sub(a[0], b[0]), d1 = sub(a[1], b[1]), d2 = sub(a[2], b[2]);
  return __dsqrt_rn(add(add(mul(d0, d0), mul(d1, d1)), mul(d2, d2)));
}

struct DegenCount {
  const int32_t* tris;
  const double* v;
  __device__ int count(long long t) const {
    const double* a = v + 3ll * tris[3 * t];
    const double* b = v + 3ll * tris[3 * t + 1];
    const double* c = v + 3ll * tris[3 * t + 2];
    const double eps = 1e-7;
    return !(edge_len(a, b) < eps || edge_len(a, c) < eps || edge_len(b, c) < eps);
  }
};

struct DegenEmit : DegenCount {
  int32_t* out;
  __device__ void emit(long long t, long long k) const {
    out[3 * k] = tris[3 * t];
    out[3 * k + 1] = tris[3 * t + 1];
    out[3 * k + 2] = tris[3 * t + 2];
  }
};

// ------------------------------------------------------------ vertices

// One vertex per listed edge: linear interpolation of the stored values
// (computeEdgeInterpolations) or the bisection of midpointSearch on the map.
// A bisection value log|q_N| - iso.  With HYBRID the FP32 orbit is tried
// first and trusted when its value clears its error bound and the 1e-8 stop
// test by a margin: then the FP64 value has the same sign and also fails the
// stop test, so every decision of the search is the one FP64 would make.
template <bool POW_REF>
__device__ __forceinline__ double value64(const MapParams& m, const GridParams& g,
                                          const IterParams& it, const double p[3], double iso,
                                          unsigned long long* e64) {
  (*e64)++;
  if (it.lagrange) return lagrange_value64<POW_REF>(m, it, p, g.slice, iso);
  int ni;
  double dd;
  return q64::sub(escape64<POW_REF, false>(m, it, p, g.slice, &ni, &dd), iso);
}

template <bool POW_REF, bool HYBRID>
__device__ __forceinline__ double bisect_value(const MapParams& m, const GridParams& g,
                                               const IterParams& it, const double p[3], double iso,
                                               unsigned long long* e32, unsigned long long* e64) {
  if (HYBRID) {
    float err;
    const float f = escape32(m, it, p, g.slice, &err);
    const float v = f - (float)iso;
    if (fabsf(v) > 1.01f * err + 1e-8f + 1e-6f * fabsf((float)iso)) {
      (*e32)++;
      return (double)v;
    }
  }
  return value64<POW_REF>(m, g, it, p, iso, e64);
}

template <bool BISECT, bool POW_REF, bool HYBRID>
__global__ void __launch_bounds__(128) vertex_kernel(const __grid_constant__ MapParams m,
                                                     const GridParams g, const IterParams it,
                                                     const uint32_t* __restrict__ list, long long n,
                                                     long long id0, int c0,
                                                     const double* __restrict__ src,
                                                     double* __restrict__ verts, double iso,
                                                     DevStats* st) {
  const long long XY = (long long)g.X * g.Y;
  unsigned long long evals = 0, evals32 = 0, unbracketed = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const uint32_t e = list[k];
    const int a = (int)(e & 3u);
    const long long w = e >> 2;
    const int z = c0 - 1 + (int)(w / XY);
    const int r = (int)(w % XY);
    const int x = r % g.X, y = r / g.X;
    const int x1 = x + (a == 0), y1 = y + (a == 1), z1 = z + (a == 2);
    double p0[3], p1[3], out[3];
    cell_center(g, x, y, z, p0);
    cell_center(g, x1, y1, z1, p1);
    using namespace q64;
    if (!BISECT) {
      // TRIANGLE_MESH.cpp:2399-2410: p0 + (d0 / (d0 - d1)) * (p1 - p0)
      const double d0 = src[(long long)(z - c0) * XY + r];
      const double d1 = src[(long long)(z1 - c0) * XY + (long long)y1 * g.X + x1];
      const double t = __ddiv_rn(d0, sub(d0, d1));
#pragma unroll
      for (int c = 0; c < 3; c++) out[c] = add(p0[c], mul(t, sub(p1[c], p0[c])));
    } else {
      // nonlinearValue at both ends (TRIANGLE_MESH.cpp:2060-2067)
      double f0 = bisect_value<POW_REF, HYBRID>(m, g, it, p0, iso, &evals32, &evals);
      double f1 = bisect_value<POW_REF, HYBRID>(m, g, it, p1, iso, &evals32, &evals);
      if (HYBRID && mul(f0, f1) >= 0.0) {
        // the end values decide the whole search: confirm a failed bracket in FP64
        f0 = value64<POW_REF>(m, g, it, p0, iso, &evals);
        f1 = value64<POW_REF>(m, g, it, p1, iso, &evals);
      }
      double pv[3], nv[3], pval = f0, nval = f1;
      bool bad = mul(f0, f1) >= 0.0;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        pv[c] = p0[c];
        nv[c] = p1[c];
      }
      if (f0 < 0) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
          pv[c] = p1[c];
          nv[c] = p0[c];
        }
        pval = f1;
        nval = f0;
      }
      // midpointSearch, TRIANGLE_MESH.cpp:2232-2271, as a loop
      for (int rec = 0;; rec++) {
#pragma unroll
        for (int c = 0; c < 3; c++) out[c] = mul(add(pv[c], nv[c]), 0.5);
        if (mul(pval, nval) >= 0.0) {
          bad = true;
          break;
        }
        if (rec >= 6) break;
        const double mv = bisect_value<POW_REF, HYBRID>(m, g, it, out, iso, &evals32, &evals);
        if (fabs(mv) < 1e-8) break;
        if (mv < 0) {
#pragma unroll
          for (int c = 0; c < 3; c++) nv[c] = out[c];
          nval = mv;
        } else {
#pragma unroll
          for (int c = 0; c < 3; c++) pv[c] = out[c];
          pval = mv;
        }
      }
      unbracketed += bad;
    }
    double* o = verts + 3 * (id0 + k);
    o[0] = out[0];
    o[1] = out[1];
    o[2] = out[2];
  }
  if (BISECT) {
    for (int o = 16; o; o >>= 1) {
      evals += __shfl_xor_sync(0xffffffffu, evals, o);
      evals32 += __shfl_xor_sync(0xffffffffu, evals32, o);
      unbracketed += __shfl_xor_sync(0xffffffffu, unbracketed, o);
    }
    if ((threadIdx.x & 31) == 0) {
      if (evals) atomicAdd(&st->aux[1], evals);
      if (unbracketed) atomicAdd(&st->aux[2], unbracketed);
      if (evals32) atomicAdd(&st->aux[3], evals32);
    }
  }
}

// ------------------------------------------------- vertices, FP32 first

// The FP32-first bisection with its FP64 evaluations taken out of line.  In
// vertex_kernel<BISECT, *, HYBRID> a warp whose lane needs one FP64 map
// evaluation waits for it at 1/64 of the FP32 rate while its other lanes
// idle.  Here each edge carries its bisection state; an edge that needs an
// FP64 value parks on a list, one kernel evaluates every parked point (a
// warp of FP64 work), and the edges resume.  The decisions, and so the
// vertices, are those of vertex_kernel.

struct EdgeState {
  double a[3], b[3];  // stages 0-3: the edge's ends p0, p1; stage 4: positive, negative end
  double va, vb;      // their values
  double pending;     // FP64 value of the point the edge waits for
  int stage;          // 0 f(p0), 1 f(p1), 2 FP64 f(p0), 3 FP64 f(p1), 4 bisection
  int rec;            // bisection level
  int flags;          // EDGE_* bits
  int pad;
};

enum : int { EDGE_PENDING = 1, EDGE_A64 = 2, EDGE_B64 = 4 };

__device__ __forceinline__ void edge_point(const EdgeState& e, double p[3]) {
  using namespace q64;
#pragma unroll
  for (int c = 0; c < 3; c++)
    p[c] = e.stage == 0 || e.stage == 2 ? e.a[c]
           : e.stage == 1 || e.stage == 3 ? e.b[c]
                                          : mul(add(e.a[c], e.b[c]), 0.5);
}

// Runs the edge until it is done (returns false; the vertex is written and
// *bad set) or needs an FP64 value (returns true).
template <bool POW_REF>
__device__ bool edge_advance(const MapParams& m, const GridParams& g, const IterParams& it,
                             EdgeState& e, double iso, double* vert, bool* bad,
                             unsigned long long* e32) {
  using namespace q64;
  for (;;) {
    double p[3];
    edge_point(e, p);
    if (e.stage == 4) {
      // midpointSearch, TRIANGLE_MESH.cpp:2232-2271
      if (mul(e.va, e.vb) >= 0.0 || e.rec >= 6) {
        *bad = mul(e.va, e.vb) >= 0.0;
        vert[0] = p[0];
        vert[1] = p[1];
        vert[2] = p[2];
        return false;
      }
    }
    double v;
    bool from64 = false;
    if (e.flags & EDGE_PENDING) {
      v = e.pending;
      e.flags &= ~EDGE_PENDING;
      from64 = true;
    } else if (e.stage == 2 || e.stage == 3) {
      return true;
    } else {
      float err;
      const float f = escape32(m, it, p, g.slice, &err);
      const float vf = f - (float)iso;
      if (!(fabsf(vf) > 1.01f * err + 1e-8f + 1e-6f * fabsf((float)iso))) return true;
      (*e32)++;
      v = (double)vf;
    }
    bool orient = false;
    switch (e.stage) {
      case 0:
        e.va = v;
        if (from64) e.flags |= EDGE_A64;
        e.stage = 1;
        break;
      case 1:
        e.vb = v;
        if (from64) e.flags |= EDGE_B64;
        if (mul(e.va, e.vb) >= 0.0) {
          // a failed bracket decides the whole edge: confirm it in FP64
          if (!(e.flags & EDGE_A64)) e.stage = 2;
          else if (!(e.flags & EDGE_B64)) e.stage = 3;
          else orient = true;
        } else {
          orient = true;
        }
        break;
      case 2:
        e.va = v;
        e.flags |= EDGE_A64;
        if (e.flags & EDGE_B64) orient = true;
        else e.stage = 3;
        break;
      case 3:
        e.vb = v;
        e.flags |= EDGE_B64;
        orient = true;
        break;
      default:
        if (fabs(v) < 1e-8) {
          vert[0] = p[0];
          vert[1] = p[1];
          vert[2] = p[2];
          *bad = false;
          return false;
        }
        if (v < 0) {
          e.b[0] = p[0];
          e.b[1] = p[1];
          e.b[2] = p[2];
          e.vb = v;
        } else {
          e.a[0] = p[0];
          e.a[1] = p[1];
          e.a[2] = p[2];
          e.va = v;
        }
        e.rec++;
    }
    if (orient) {
      // positive end first (TRIANGLE_MESH.cpp:2060-2080)
      if (e.va < 0) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const double t = e.a[c];
          e.a[c] = e.b[c];
          e.b[c] = t;
        }
        const double t = e.va;
        e.va = e.vb;
        e.vb = t;
      }
      e.stage = 4;
      e.rec = 0;
    }
  }
}

__device__ __forceinline__ void warp_push(bool want, uint32_t k, unsigned long long* count,
                                          uint32_t* list) {
  const unsigned mask = __ballot_sync(0xffffffffu, want);
  if (!mask) return;
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(mask));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (want) list[base + __popc(mask & ((1u << lane) - 1u))] = k;
}

__device__ __forceinline__ void edge_counts(unsigned long long e32, unsigned long long e64,
                                            unsigned long long bad, DevStats* st) {
  for (int o = 16; o; o >>= 1) {
    e32 += __shfl_xor_sync(0xffffffffu, e32, o);
    e64 += __shfl_xor_sync(0xffffffffu, e64, o);
    bad += __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (e64) atomicAdd(&st->aux[1], e64);
    if (bad) atomicAdd(&st->aux[2], bad);
    if (e32) atomicAdd(&st->aux[3], e32);
  }
}

// Starts every edge of the slab; edges that need FP64 go to `park`.
template <bool POW_REF>
__global__ void __launch_bounds__(128) edge_start_kernel(const __grid_constant__ MapParams m,
                                                         const GridParams g, const IterParams it,
                                                         const uint32_t* __restrict__ list,
                                                         long long n, long long id0, int c0,
                                                         EdgeState* __restrict__ es,
                                                         double* __restrict__ verts, double iso,
                                                         uint32_t* park,
                                                         unsigned long long* n_park,
                                                         DevStats* st) {
  const long long XY = (long long)g.X * g.Y;
  unsigned long long e32 = 0, nbad = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (blockIdx.x * (long long)blockDim.x + threadIdx.x) & ~31ll; base < n;
       base += stride) {
    const long long k = base + (threadIdx.x & 31);
    bool wait = false;
    if (k < n) {
      const uint32_t e = list[k];
      const int a = (int)(e & 3u);
      const long long w = e >> 2;
      const int z = c0 - 1 + (int)(w / XY);
      const int r = (int)(w % XY);
      const int x = r % g.X, y = r / g.X;
      EdgeState s;
      cell_center(g, x, y, z, s.a);
      cell_center(g, x + (a == 0), y + (a == 1), z + (a == 2), s.b);
      s.va = s.vb = s.pending = 0.0;
      s.stage = s.rec = s.flags = s.pad = 0;
      bool bad = false;
      wait = edge_advance<POW_REF>(m, g, it, s, iso, verts + 3 * (id0 + k), &bad, &e32);
      nbad += bad;
      if (wait) es[id0 + k] = s;
    }
    warp_push(wait, (uint32_t)(id0 + k), n_park, park);
  }
  edge_counts(e32, 0, nbad, st);
}

// Every parked edge's point in double-float first (integer exponents): where
// its tracked error bound decides what FP64 would (the sign, and in the
// bisection whether |value| < 1e-8), that value stands in for FP64's; the
// other edges, and the failed-bracket re-checks, go on to FP64 (`list64`).
__global__ void __launch_bounds__(128) edge_ff_kernel(const __grid_constant__ MapParams m,
                                                      const GridParams g, const IterParams it,
                                                      const uint32_t* __restrict__ park,
                                                      const unsigned long long* n_park,
                                                      EdgeState* __restrict__ es, double iso,
                                                      uint32_t* list64,
                                                      unsigned long long* n_list64,
                                                      DevStats* st) {
  const unsigned long long n = *n_park;
  unsigned long long eff = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long base = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) & ~31ull;
       base < n; base += stride) {
    const unsigned long long j = base + (threadIdx.x & 31);
    bool need64 = false;
    uint32_t k = 0;
    if (j < n) {
      k = park[j];
      EdgeState& e = es[k];
      need64 = true;
      if (m.all_int && e.stage != 2 && e.stage != 3) {
        double p[3];
        edge_point(e, p);
        float err;
        const double f = escape_ff(m, it, p, g.slice, &err);
        const double v = f - iso;
        // FP64 rounding of f - iso and of the reference's own |q| on top
        const double eb = 1.01 * (double)err + 1e-15 * (fabs(f) + fabs(iso));
        bool decided = isfinite(eb) && fabs(v) > eb;  // the sign
        if (e.stage == 4)  // and the bisection's stop test
          decided = isfinite(eb) && (fabs(v) > eb + 1e-8 || fabs(v) + eb < 1e-8);
        if (decided) {
          e.pending = v;
          e.flags |= EDGE_PENDING;
          need64 = false;
          eff++;
        }
      }
    }
    warp_push(need64, k, n_list64, list64);
  }
  for (int o = 16; o; o >>= 1) eff += __shfl_xor_sync(0xffffffffu, eff, o);
  if ((threadIdx.x & 31) == 0 && eff) atomicAdd(&st->ff_evals, eff);
}

// The FP64 value of every parked edge's point.
template <bool POW_REF>
__global__ void __launch_bounds__(128) edge_fp64_kernel(const __grid_constant__ MapParams m,
                                                        const GridParams g, const IterParams it,
                                                        const uint32_t* __restrict__ park,
                                                        const unsigned long long* n_park,
                                                        EdgeState* __restrict__ es, double iso,
                                                        DevStats* st) {
  const unsigned long long n = *n_park;
  unsigned long long e64 = 0;
  for (unsigned long long j = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; j < n;
       j += (unsigned long long)gridDim.x * blockDim.x) {
    EdgeState& e = es[park[j]];
    double p[3];
    edge_point(e, p);
    e.pending = value64<POW_REF>(m, g, it, p, iso, &e64);
    e.flags |= EDGE_PENDING;
  }
  for (int o = 16; o; o >>= 1) e64 += __shfl_xor_sync(0xffffffffu, e64, o);
  if ((threadIdx.x & 31) == 0 && e64) atomicAdd(&st->aux[1], e64);
}

// Resumes the parked edges; those that need FP64 again go to `next`.
template <bool POW_REF>
__global__ void __launch_bounds__(128) edge_resume_kernel(const __grid_constant__ MapParams m,
                                                          const GridParams g, const IterParams it,
                                                          const uint32_t* __restrict__ park,
                                                          const unsigned long long* n_park,
                                                          EdgeState* __restrict__ es,
                                                          double* __restrict__ verts, double iso,
                                                          uint32_t* next,
                                                          unsigned long long* n_next,
                                                          DevStats* st) {
  const unsigned long long n = *n_park;
  unsigned long long e32 = 0, nbad = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long base = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) & ~31ull;
       base < n; base += stride) {
    const unsigned long long j = base + (threadIdx.x & 31);
    bool wait = false;
    uint32_t k = 0;
    if (j < n) {
      k = park[j];
      EdgeState s = es[k];
      bool bad = false;
      wait = edge_advance<POW_REF>(m, g, it, s, iso, verts + 3 * (long long)k, &bad, &e32);
      nbad += bad;
      if (wait) es[k] = s;
    }
    warp_push(wait, k, n_next, next);
  }
  edge_counts(e32, 0, nbad, st);
}

__global__ void to_float_kernel(const double* __restrict__ a, float* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n;
}

}  // namespace

size_t mesh_edge_state_bytes() { return sizeof(EdgeState); }

long long mesh_scan_blocks(long long n) { return (n + SCAN_B - 1) / SCAN_B + 1; }

cudaError_t mesh_flags(const double* src, int X, int Y, long long n_layers, uint8_t* flags,
                       cudaStream_t s) {
  if (n_layers <= 0) return cudaSuccess;
  const long long n = n_layers * X * Y;
  (void)n;
  const long long XY = (long long)X * Y;
  flags_kernel<<<(unsigned)((XY + 127) / 128), 128, 0, s>>>(src, X, Y, n_layers, flags);
  return cudaGetLastError();
}

cudaError_t mesh_vertex_ids(MeshWindow& w, int j0, int j1, int lay_lo, int lay_hi,
                            long long running, long long* n_new, cudaStream_t s,
                            const std::function<cudaError_t(long long)>& ensure_list) {
  const long long XY = (long long)w.X * w.Y;
  const long long n = (long long)(j1 - j0) * XY;
  MaskCount mc{w.flags, w.masks, w.X, w.Y, j0, lay_lo, lay_hi};
  // the emit pass needs the list buffer, which ensure_list sizes first
  cudaError_t err = cudaSuccess;
  const long long nb = (n + SCAN_B - 1) / SCAN_B;
  if (n == 0) {
    *n_new = 0;
    return cudaSuccess;
  }
  mask_count_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(mc, n, w.bsum);
  scan_bsum_kernel<<<1, 1024, 0, s>>>(w.bsum, nb);
  if ((err = cudaMemcpyAsync(n_new, w.bsum + nb, sizeof(long long), cudaMemcpyDeviceToHost, s)))
    return err;
  if ((err = cudaStreamSynchronize(s))) return err;
  if ((err = ensure_list(*n_new))) return err;
  VertexEmit ve{w.masks, w.vbase, w.list, running, XY, j0};
  emit_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(ve, n, w.bsum, running);
  return cudaGetLastError();
}

template <bool POW_REF>
static cudaError_t parked_start(const MapParams& m, const GridParams& g, const IterParams& it,
                                const MeshWindow& w, long long n, long long id0, int c0,
                                double* verts, double iso, DevStats* st, const EdgeScratch& sc,
                                cudaStream_t s) {
  const int blocks = (int)std::min<long long>((n + 127) / 128, (long long)sm_count() * 32);
  edge_start_kernel<POW_REF><<<blocks, 128, 0, s>>>(m, g, it, w.list, n, id0, c0,
                                                    static_cast<EdgeState*>(sc.state), verts, iso,
                                                    sc.list[0], sc.count, st);
  return cudaGetLastError();
}

template <bool POW_REF>
static cudaError_t parked_finish(const MapParams& m, const GridParams& g, const IterParams& it,
                                 double* verts, double iso, DevStats* st, const EdgeScratch& sc,
                                 cudaStream_t s) {
  EdgeState* es = static_cast<EdgeState*>(sc.state);
  cudaError_t err;
  // each round gives every parked edge one value (double-float where its
  // bound decides, else FP64); an edge asks for at most 2 at its ends (one
  // each, or a re-check of a failed bracket) and 6 in the bisection
  for (int round = 0, cur = 0;; round++, cur ^= 1) {
    unsigned long long parked = 0;
    if ((err = cudaMemcpyAsync(&parked, sc.count + cur, sizeof parked, cudaMemcpyDeviceToHost, s)))
      return err;
    if ((err = cudaStreamSynchronize(s))) return err;
    if (parked == 0) return cudaGetLastError();
    if (round == 8) return cudaErrorInvalidValue;  // cannot happen: see the count above
    const int pb = (int)std::min<long long>(((long long)parked + 127) / 128,
                                            (long long)sm_count() * 32);
    // double-float first; what it cannot decide, in FP64
    if ((err = cudaMemsetAsync(sc.count + 2, 0, sizeof(unsigned long long), s))) return err;
    edge_ff_kernel<<<pb, 128, 0, s>>>(m, g, it, sc.list[cur], sc.count + cur, es, iso,
                                      sc.list[2], sc.count + 2, st);
    edge_fp64_kernel<POW_REF><<<pb, 128, 0, s>>>(m, g, it, sc.list[2], sc.count + 2, es, iso,
                                                 st);
    if ((err = cudaMemsetAsync(sc.count + (cur ^ 1), 0, sizeof(unsigned long long), s)))
      return err;
    edge_resume_kernel<POW_REF><<<pb, 128, 0, s>>>(m, g, it, sc.list[cur], sc.count + cur, es,
                                                   verts, iso, sc.list[cur ^ 1],
                                                   sc.count + (cur ^ 1), st);
  }
}

cudaError_t mesh_parked_finish(const MapParams& m, const GridParams& g, const IterParams& it,
                               bool pow_ref, double* verts, double iso, DevStats* st,
                               const EdgeScratch& sc, cudaStream_t s) {
  return pow_ref ? parked_finish<true>(m, g, it, verts, iso, st, sc, s)
                 : parked_finish<false>(m, g, it, verts, iso, st, sc, s);
}

cudaError_t mesh_vertices(const MapParams& m, const GridParams& g, const IterParams& it,
                          int edge_mode, bool pow_ref, bool hybrid, const MeshWindow& w,
                          long long n, long long id0, int c0, const double* src, double* verts,
                          double iso, DevStats* st, const EdgeScratch* scratch, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (edge_mode != 0 && hybrid && scratch)
    return pow_ref ? parked_start<true>(m, g, it, w, n, id0, c0, verts, iso, st, *scratch, s)
                   : parked_start<false>(m, g, it, w, n, id0, c0, verts, iso, st, *scratch, s);
  const int blocks = (int)std::min<long long>((n + 127) / 128, (long long)sm_count() * 32);
#define QJ_VK(B, P, H) \
  vertex_kernel<B, P, H><<<blocks, 128, 0, s>>>(m, g, it, w.list, n, id0, c0, src, verts, iso, st)
  if (edge_mode == 0)
    QJ_VK(false, false, false);
  else if (pow_ref)
    hybrid ? QJ_VK(true, true, true) : QJ_VK(true, true, false);
  else
    hybrid ? QJ_VK(true, false, true) : QJ_VK(true, false, false);
#undef QJ_VK
  return cudaGetLastError();
}

cudaError_t mesh_triangles(MeshWindow& w, int j0, int j1, long long running, int32_t* tris,
                           long long cap, long long* n_new, cudaStream_t s) {
  const long long XY = (long long)w.X * w.Y;
  const long long n = (long long)(j1 - j0) * XY;
  if (n <= 0) {
    *n_new = 0;
    return cudaSuccess;
  }
  const long long nb = (n + SCAN_B - 1) / SCAN_B;
  TriCount tc{w.flags, XY, j0};
  count_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(tc, n, w.bsum);
  scan_bsum_kernel<<<1, 1024, 0, s>>>(w.bsum, nb);
  cudaError_t err;
  if ((err = cudaMemcpyAsync(n_new, w.bsum + nb, sizeof(long long), cudaMemcpyDeviceToHost, s)))
    return err;
  TriEmit te{w.flags, w.masks, w.vbase, tris, cap, w.X, XY, j0};
  emit_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(te, n, w.bsum, running);
  if ((err = cudaGetLastError())) return err;
  return cudaStreamSynchronize(s);
}

cudaError_t mesh_filter(const int32_t* tris, long long n, const double* verts, int32_t* out,
                        long long* bsum, long long* n_keep, cudaStream_t s) {
  if (n == 0) {
    *n_keep = 0;
    return cudaSuccess;
  }
  const long long nb = (n + SCAN_B - 1) / SCAN_B;
  DegenCount dc{tris, verts};
  count_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(dc, n, bsum);
  scan_bsum_kernel<<<1, 1024, 0, s>>>(bsum, nb);
  DegenEmit de;
  de.tris = tris;
  de.v = verts;
  de.out = out;
  emit_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(de, n, bsum, 0);
  cudaError_t err;
  if ((err = cudaMemcpyAsync(n_keep, bsum + nb, sizeof(long long), cudaMemcpyDeviceToHost, s)))
    return err;
  return cudaStreamSynchronize(s);
}

cudaError_t mesh_to_float(const double* a, float* b, long long n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int blocks = (int)std::min<long long>((n + 255) / 256, (long long)sm_count() * 16);
  to_float_kernel<<<blocks, 256, 0, s>>>(a, b, n);
  return cudaGetLastError();
}

}  // namespace qj
