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
// exclusive prefix and writes the block total to *total.  T is long long or
// unsigned long long (packed counters whose fields never carry into each
// other).
template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* total) {
  __shared__ T warp_sums[SCAN_T / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T n = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += n;
  }
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = lane < SCAN_T / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T n = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += n;
    }
    if (lane < SCAN_T / 32) warp_sums[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  const T warp_base = warp ? warp_sums[warp - 1] : 0;
  *total = warp_sums[SCAN_T / 32 - 1];
  __syncthreads();
  return warp_base + inc - v;
}

// Generic pass 1: per-block sums of op.count(i) over items [0, n) (n read
// from n_dev when given).
template <class Op>
__global__ void __launch_bounds__(SCAN_T) count_kernel(Op op, long long n, long long* bsum,
                                                       const long long* n_dev) {
  if (n_dev) n = *n_dev;
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
// op.count over items [0, n) (n and running read from n_dev and run_dev
// when given).
template <class Op>
__global__ void __launch_bounds__(SCAN_T) emit_kernel(Op op, long long n, const long long* bsum,
                                                      long long running, const long long* n_dev,
                                                      const long long* run_dev) {
  if (n_dev) n = *n_dev;
  if (run_dev) running = *run_dev;
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

// The vertex of an edge: the reference places one on every edge that a
// triangle of some cube uses.  Every case of its table uses exactly the edges
// whose endpoint signs differ, except case 158, which leaves out the three
// edges of its isolated corner (edges 10, 5, 6: the x-, y- and z-edges at the
// cube's (1, 0, 0) corner).  An interior edge always has another cube that
// uses it, so the sign changes give the vertex set except on three lines of
// the grid where the case-158 cube is the edge's only cube: x-edges at
// (y, z) = (0, 0), y-edges at (x, z) = (X-1, 0), z-edges at (x, y) = (X-1, 0)
// (mc_fix158_kernel).
//
// Classification of one slab reads the FP64 field once and works on sign
// bits only.  A warp takes a row segment of MC_SEG = 64 voxels of MC_ROWS
// rows and walks the slab's planes; per plane it loads MC_ROWS + 1 rows
// (one 16-byte load per lane and row: x = xb + 2 lane and xb + 2 lane + 1)
// and turns each into two 32-bit sign words with __ballot_sync, E (even x)
// and O (odd x), plus the sign at xb + 64.  Edge masks and mixed cubes
// (neither all inside nor all outside) come from word-wide bit operations,
// identical in every lane, with the words of the plane below kept in
// registers, so no lane works per voxel here.  Outputs per unit (64 voxels
// of one row of one plane, numbered in scan order (plane, row, segment)):
// the sign words (every unit), and for units with activity (an edge with a
// vertex or a cube with triangles) the packed counts of vertices and of
// mixed cubes and the two activity words.  The unit counts start at zero.
// An exclusive scan of the counts gives every voxel's first vertex id and
// every cube's place in the cube list in the reference's order (vertices by
// (z, y, x, axis) of the edge's lower endpoint, cubes in scan order); the
// sparse pass (mc_emit_kernel) forms edge masks and cube flags (corner
// weights NNN=1 NNP=2 NPN=4 NPP=8 PNN=16 PNP=32 PPN=64 PPP=128 with letters
// x, y, z, TRIANGLE_MESH.cpp:4929-4931) of the active voxels from the sign
// words, and a scan over the cube list gives each cube's first triangle.
//
// Plain 16-byte loads are used: on the large workload's slab (2200^2 x 65
// planes) they stream the field at about 7.6 TB/s with the classification
// taken out, where per-warp TMA boxes of 66 x 5 doubles reached 2.6 TB/s.
constexpr int MC_SEG = 64;     // voxels per unit (one warp's row segment)
constexpr int MC_WORDS = 2;    // words per unit: even x, odd x
constexpr int MC_ROWS = 4;     // rows per warp
constexpr int MC_WARPS = 4;    // warps per classify block
static_assert(MC_WORDS == MESH_UNIT_WORDS, "words per unit");
// packed unit counts: vertices (<= 192) | mixed cubes (<= 64) << 8
__device__ __forceinline__ uint32_t unit_pack(int nv, int nc) {
  return (uint32_t)nv | (uint32_t)nc << 8;
}
// widened for sums over a scan block of SCAN_B units
__device__ __forceinline__ unsigned long long unit_widen(uint32_t c) {
  return (unsigned long long)(c & 255u) | (unsigned long long)(c >> 8) << 32;
}

// bit i of v (< 2^16) to bit 2i
__device__ __forceinline__ uint32_t spread16(uint32_t v) {
  v = (v | (v << 8)) & 0x00FF00FFu;
  v = (v | (v << 4)) & 0x0F0F0F0Fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}
// the even/odd words of a unit as 64 bits in x order
__device__ __forceinline__ unsigned long long natural64(uint2 w) {
  const uint32_t lo = spread16(w.x & 0xFFFFu) | spread16(w.y & 0xFFFFu) << 1;
  const uint32_t hi = spread16(w.x >> 16) | spread16(w.y >> 16) << 1;
  return (unsigned long long)lo | (unsigned long long)hi << 32;
}

struct McSlab {
  const double* src;  // field planes gz0 .. gz0 + P - 1 (plane stride XY)
  int X, Y, S;        // S: units per row
  int P, Pv;          // planes in src; voxel planes classified (P - 1, or P on the last slab)
  int gz0;            // global index of src plane 0
  long long XY;
  uint2* sign;        // [plane < P][Y][S]: sign words of every unit
  uint2* bits;        // [Pv][Y][S]: activity words of units with activity
  uint32_t* ucount;   // [Pv][Y][S]: packed counts (zero where nothing is active)
};

// Column validity of a segment starting at xb: x < X for even (vE) and odd
// (vO) bits, x + 1 < X (v1E, v1O).
struct McCols {
  uint32_t vE, vO, v1E, v1O;
};
__device__ __forceinline__ uint32_t low_bits(int n) {
  return n >= 32 ? 0xffffffffu : n <= 0 ? 0u : (1u << n) - 1u;
}
__device__ __forceinline__ McCols mc_cols(int X, int xb) {
  McCols v;
  v.vE = low_bits((X - xb + 1) / 2);   // xb + 2k < X
  v.vO = low_bits((X - xb) / 2);       // xb + 2k + 1 < X
  v.v1E = v.vO;
  v.v1O = low_bits((X - xb - 1) / 2);  // xb + 2k + 2 < X
  return v;
}

// v > 0.0 with integer operations (GB300's FP64 pipe, which a double
// comparison would use, is narrow): positive values from the smallest
// denormal up to +inf are the bit patterns 1 .. 0x7FF0000000000000; zeros,
// negatives and NaNs fall outside.
__device__ __forceinline__ bool positive(double v) {
  return (unsigned long long)__double_as_longlong(v) - 1ull < 0x7FF0000000000000ull;
}

// Sign words of rows y0 .. y0 + MC_ROWS of one plane: E[r] bit k = (value at
// xb + 2k > 0), O[r] the same at xb + 2k + 1, bit r of *N the sign at
// xb + 64.  Values outside the grid read as 0 (their edges and cubes are
// masked).  Every load is issued before the first ballot.
template <bool VEC>
__device__ __forceinline__ void plane_signs(const double* __restrict__ plane, int X, int Y, int y0,
                                            int xb, int lane, uint32_t (&E)[MC_ROWS + 1],
                                            uint32_t (&O)[MC_ROWS + 1], uint32_t* N) {
  const int x = xb + 2 * lane;
  double a[MC_ROWS + 1], b[MC_ROWS + 1];
#pragma unroll
  for (int r = 0; r <= MC_ROWS; r++) {
    a[r] = 0.0;
    b[r] = 0.0;
    if (y0 + r < Y) {
      const double* row = plane + (long long)(y0 + r) * X;
      if (VEC) {
        if (x < X) {  // X even: x + 1 < X too
          const double2 v = __ldg(reinterpret_cast<const double2*>(row + x));
          a[r] = v.x;
          b[r] = v.y;
        }
      } else {
        if (x < X) a[r] = __ldg(row + x);
        if (x + 1 < X) b[r] = __ldg(row + x + 1);
      }
    }
  }
  double nx = 0.0;
  if (lane <= MC_ROWS && y0 + lane < Y && xb + MC_SEG < X)
    nx = __ldg(plane + (long long)(y0 + lane) * X + xb + MC_SEG);
#pragma unroll
  for (int r = 0; r <= MC_ROWS; r++) {
    E[r] = __ballot_sync(0xffffffffu, positive(a[r]));
    O[r] = __ballot_sync(0xffffffffu, positive(b[r]));
  }
  *N = __ballot_sync(0xffffffffu, positive(nx));
}

// lanes 0 .. MC_ROWS - 1: the sign words of their row of plane p
__device__ __forceinline__ void store_signs(const McSlab& c, int p, int y0, int seg, int lane,
                                            const uint32_t (&E)[MC_ROWS + 1],
                                            const uint32_t (&O)[MC_ROWS + 1]) {
  uint2 w = make_uint2(0u, 0u);
#pragma unroll
  for (int r = 0; r < MC_ROWS; r++)
    if (lane == r) w = make_uint2(E[r], O[r]);
  if (lane < MC_ROWS && y0 + lane < c.Y) c.sign[((long long)p * c.Y + y0 + lane) * c.S + seg] = w;
}

// Voxel plane p of rows y0 .. y0 + MC_ROWS - 1 of segment seg, from the sign
// words of planes p (l*) and p + 1 (h*, zero when the plane does not exist).
// A cube is mixed when its eight corners are neither all inside nor all
// outside: with the z-pair words zo = l | h and za = l & h per row, the
// corners of the cube at (x, y) are the bits x and x + 1 of rows y and y + 1.
__device__ __forceinline__ void mc_classify_plane(const McSlab& c, int p, bool hz, int y0, int seg,
                                                  int lane, const McCols& v,
                                                  const uint32_t (&lE)[MC_ROWS + 1],
                                                  const uint32_t (&lO)[MC_ROWS + 1], uint32_t lN,
                                                  const uint32_t (&hE)[MC_ROWS + 1],
                                                  const uint32_t (&hO)[MC_ROWS + 1], uint32_t hN) {
  const int xb = seg * MC_SEG;
  // Where all MC_ROWS + 1 rows and the next column exist, a block whose two
  // planes are all inside or all outside has no vertex and no mixed cube
  if (hz && y0 + MC_ROWS < c.Y && xb + MC_SEG < c.X) {
    uint32_t any = 0u, all = 0xffffffffu;
#pragma unroll
    for (int r = 0; r <= MC_ROWS; r++) {
      any |= lE[r] | lO[r] | hE[r] | hO[r];
      all &= lE[r] & lO[r] & hE[r] & hO[r];
    }
    constexpr uint32_t rows = (1u << (MC_ROWS + 1)) - 1u;
    if ((any == 0u && ((lN | hN) & rows) == 0u) || (all == 0xffffffffu && (lN & hN & rows) == rows))
      return;
  }
  // the x + 1 neighbour of even bit k is odd bit k, of odd bit k even bit
  // k + 1 (bit 31: the next segment's first column, from the N words)
  uint32_t l1[MC_ROWS + 1], anyE[MC_ROWS + 1], anyO[MC_ROWS + 1], allE[MC_ROWS + 1],
      allO[MC_ROWS + 1];
#pragma unroll
  for (int r = 0; r <= MC_ROWS; r++) {
    l1[r] = (lE[r] >> 1) | (lN << (31 - r) & 0x80000000u);
    anyE[r] = anyO[r] = allE[r] = allO[r] = 0u;
    if (hz) {
      const uint32_t h1 = (hE[r] >> 1) | (hN << (31 - r) & 0x80000000u);
      const uint32_t zoE = lE[r] | hE[r], zoO = lO[r] | hO[r], zo1 = l1[r] | h1;
      const uint32_t zaE = lE[r] & hE[r], zaO = lO[r] & hO[r], za1 = l1[r] & h1;
      anyE[r] = zoE | zoO;  // columns x, x+1 of an even voxel
      allE[r] = zaE & zaO;
      anyO[r] = zoO | zo1;  // columns x, x+1 of an odd voxel
      allO[r] = zaO & za1;
    }
  }
  uint32_t cnt_lane = 0;       // lane r: the packed counts of row r
  uint2 bits_lane = {0u, 0u};  // lane r: the activity words of row r
#pragma unroll
  for (int r = 0; r < MC_ROWS; r++) {
    const int y = y0 + r;
    if (y >= c.Y) break;
    const bool hy = y + 1 < c.Y;
    const uint32_t AE = lE[r], AO = lO[r];
    const uint32_t xeE = (AE ^ AO) & v.v1E, xeO = (AO ^ l1[r]) & v.v1O;
    const uint32_t yeE = hy ? (AE ^ lE[r + 1]) & v.vE : 0u, yeO = hy ? (AO ^ lO[r + 1]) & v.vO : 0u;
    const uint32_t zeE = hz ? (AE ^ hE[r]) & v.vE : 0u, zeO = hz ? (AO ^ hO[r]) & v.vO : 0u;
    uint32_t mxE = 0u, mxO = 0u;
    if (hy && hz) {
      mxE = (anyE[r] | anyE[r + 1]) & ~(allE[r] & allE[r + 1]) & v.v1E;
      mxO = (anyO[r] | anyO[r + 1]) & ~(allO[r] & allO[r + 1]) & v.v1O;
    }
    const uint32_t actE = xeE | yeE | zeE | mxE, actO = xeO | yeO | zeO | mxO;
    if (!(actE | actO)) continue;  // uniform over the warp
    const int nv = __popc(xeE) + __popc(xeO) + __popc(yeE) + __popc(yeO) + __popc(zeE) + __popc(zeO);
    const int nc = __popc(mxE) + __popc(mxO);
    if (lane == r) {
      cnt_lane = unit_pack(nv, nc);
      bits_lane = make_uint2(actE, actO);
    }
  }
  if (lane < MC_ROWS && cnt_lane) {
    const long long u = ((long long)p * c.Y + y0 + lane) * c.S + seg;
    c.ucount[u] = cnt_lane;
    c.bits[u] = bits_lane;
  }
}

// One warp per task (segment, row group).
template <bool VEC>
__global__ void __launch_bounds__(32 * MC_WARPS) mc_classify_kernel(const McSlab c) {
  const int lane = threadIdx.x & 31;
  const long long task = (long long)blockIdx.x * MC_WARPS + (threadIdx.x >> 5);
  const int groups = (c.Y + MC_ROWS - 1) / MC_ROWS;
  if (task >= (long long)groups * c.S) return;  // the whole warp
  const int seg = (int)(task % c.S);
  const int y0 = (int)(task / c.S) * MC_ROWS;
  const int xb = seg * MC_SEG;
  const McCols v = mc_cols(c.X, xb);
  uint32_t lE[MC_ROWS + 1], lO[MC_ROWS + 1], lN;
  plane_signs<VEC>(c.src, c.X, c.Y, y0, xb, lane, lE, lO, &lN);
  for (int p = 0; p < c.Pv; p++) {
    const bool hz = p + 1 < c.P;
    uint32_t hE[MC_ROWS + 1], hO[MC_ROWS + 1], hN = 0;
#pragma unroll
    for (int r = 0; r <= MC_ROWS; r++) hE[r] = hO[r] = 0u;
    if (hz) plane_signs<VEC>(c.src + (long long)(p + 1) * c.XY, c.X, c.Y, y0, xb, lane, hE, hO, &hN);
    store_signs(c, p, y0, seg, lane, lE, lO);
    mc_classify_plane(c, p, hz, y0, seg, lane, v, lE, lO, lN, hE, hO, hN);
#pragma unroll
    for (int r = 0; r <= MC_ROWS; r++) {
      lE[r] = hE[r];
      lO[r] = hO[r];
    }
    lN = hN;
  }
  // the window's top plane when it is not classified itself (the emit pass
  // reads it as the plane above)
  if (c.Pv < c.P) store_signs(c, c.Pv, y0, seg, lane, lE, lO);
}

// Form for fields whose rows are 16-byte aligned (X even): each lane copies
// its own values of MC_ASTAGES planes ahead into a shared-memory ring with
// cp.async (16 bytes per row; lanes 0 .. MC_ROWS also the next column's 8
// bytes; zero-filled outside the grid), so a warp keeps several planes of
// loads in flight without holding them in registers.  A lane reads back only
// what it copied itself, so cp.async.wait_group alone orders the reads.
constexpr int MC_ASTAGES = 4;
constexpr int MC_NEXT_OFF = (MC_ROWS + 1) * 32 * 16;        // next-column values
constexpr int MC_ASTAGE_BYTES = MC_NEXT_OFF + 8 * (MC_ROWS + 1 + 1) / 16 * 16 + 16;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src),
               "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(dst)), "l"(src),
               "r"(valid ? 8 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_ahead() {
  asm volatile("cp.async.wait_group %0;" ::"n"(MC_ASTAGES - 1) : "memory");
}

// this lane's copies of plane q (q >= n_load: an empty group)
__device__ __forceinline__ void async_plane(const McSlab& c, unsigned char* stage, int q, int n_load,
                                            int y0, int xb, int lane) {
  if (q < n_load) {
    const double* plane = c.src + (long long)q * c.XY;
    const int x = xb + 2 * lane;
#pragma unroll
    for (int r = 0; r <= MC_ROWS; r++) {
      const bool ok = y0 + r < c.Y && x < c.X;
      cp_async16(stage + (r * 32 + lane) * 16, ok ? plane + (long long)(y0 + r) * c.X + x : c.src, ok);
    }
    if (lane <= MC_ROWS) {
      const bool ok = y0 + lane < c.Y && xb + MC_SEG < c.X;
      cp_async8(stage + MC_NEXT_OFF + lane * 8,
                ok ? plane + (long long)(y0 + lane) * c.X + xb + MC_SEG : c.src, ok);
    }
  }
  cp_async_commit();
}

__device__ __forceinline__ void stage_signs(const unsigned char* stage, int lane,
                                            uint32_t (&E)[MC_ROWS + 1], uint32_t (&O)[MC_ROWS + 1],
                                            uint32_t* N) {
#pragma unroll
  for (int r = 0; r <= MC_ROWS; r++) {
    const double2 v = *reinterpret_cast<const double2*>(stage + (r * 32 + lane) * 16);
    E[r] = __ballot_sync(0xffffffffu, positive(v.x));
    O[r] = __ballot_sync(0xffffffffu, positive(v.y));
  }
  const double nx = lane <= MC_ROWS ? *reinterpret_cast<const double*>(stage + MC_NEXT_OFF + lane * 8) : 0.0;
  *N = __ballot_sync(0xffffffffu, positive(nx));
}

__global__ void __launch_bounds__(32 * MC_WARPS) mc_classify_async_kernel(const McSlab c) {
  __shared__ __align__(16) unsigned char ring[MC_WARPS][MC_ASTAGES][MC_ASTAGE_BYTES];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long task = (long long)blockIdx.x * MC_WARPS + warp;
  const int groups = (c.Y + MC_ROWS - 1) / MC_ROWS;
  if (task >= (long long)groups * c.S) return;  // the whole warp
  const int seg = (int)(task % c.S);
  const int y0 = (int)(task / c.S) * MC_ROWS;
  const int xb = seg * MC_SEG;
  const McCols v = mc_cols(c.X, xb);
  const int n_load = min(c.Pv + 1, c.P);  // planes read
#pragma unroll
  for (int q = 0; q < MC_ASTAGES; q++) async_plane(c, ring[warp][q], q, n_load, y0, xb, lane);
  uint32_t lE[MC_ROWS + 1], lO[MC_ROWS + 1], lN = 0;
  for (int q = 0; q < n_load; q++) {
    unsigned char* st = ring[warp][q % MC_ASTAGES];
    cp_async_wait_ahead();  // plane q has landed (this lane's copies)
    uint32_t hE[MC_ROWS + 1], hO[MC_ROWS + 1], hN;
    stage_signs(st, lane, hE, hO, &hN);
    async_plane(c, st, q + MC_ASTAGES, n_load, y0, xb, lane);
    if (q > 0) {  // voxel plane q - 1 between planes q - 1 and q
      store_signs(c, q - 1, y0, seg, lane, lE, lO);
      mc_classify_plane(c, q - 1, true, y0, seg, lane, v, lE, lO, lN, hE, hO, hN);
    }
#pragma unroll
    for (int r = 0; r <= MC_ROWS; r++) {
      lE[r] = hE[r];
      lO[r] = hO[r];
    }
    lN = hN;
  }
  // the last plane read: classified itself on the grid's last slab (no plane
  // above), else stored as the window's top plane
  store_signs(c, n_load - 1, y0, seg, lane, lE, lO);
  if (c.Pv == n_load) {
    uint32_t zE[MC_ROWS + 1], zO[MC_ROWS + 1];
#pragma unroll
    for (int r = 0; r <= MC_ROWS; r++) zE[r] = zO[r] = 0u;
    mc_classify_plane(c, n_load - 1, false, y0, seg, lane, v, lE, lO, lN, zE, zO, 0u);
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Flag of the cube at (cx, cy) of window plane p, from the field.
__device__ __forceinline__ int cube_flag_src(const McSlab& c, int cx, int cy, int p) {
  int f = 0;
#pragma unroll
  for (int dx = 0; dx < 2; dx++)
#pragma unroll
    for (int dy = 0; dy < 2; dy++)
#pragma unroll
      for (int dz = 0; dz < 2; dz++)
        f |= (int)(c.src[(long long)(p + dz) * c.XY + (long long)(cy + dy) * c.X + cx + dx] > 0.0)
             << (4 * dx + 2 * dy + dz);
  return f;
}

// The edges case 158 leaves without a vertex: candidates k < X-1 are the
// x-edges at (k, 0, 0), the next Y-1 the y-edges at (X-1, k, 0) (both on
// the grid's first plane), the next Pv the z-edges at (X-1, 0, p).  An edge
// loses its vertex when its one cube has flag 158; the edge changes sign, so
// its voxel's unit counted it, and the count drops by one (the emit pass
// applies the same rule).
__global__ void mc_fix158_kernel(const McSlab c) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  int x, y, p, cx;
  bool zline = false;
  if (k < c.X - 1) {
    x = k, y = 0, p = 0, cx = k;
  } else if (k < c.X - 1 + c.Y - 1) {
    x = c.X - 1, y = k - (c.X - 1), p = 0, cx = c.X - 2;
  } else if (k < c.X - 1 + c.Y - 1 + c.Pv) {
    x = c.X - 1, y = 0, p = k - (c.X - 1 + c.Y - 1), cx = c.X - 2, zline = true;
  } else {
    return;
  }
  if (!zline && c.gz0 != 0) return;  // only the grid's first plane
  if (p + 1 >= c.P) return;          // no cube above this plane
  if (cube_flag_src(c, cx, y, p) != 158) return;
  atomicSub(&c.ucount[((long long)p * c.Y + y) * c.S + x / MC_SEG], 1u);
}

// Per scan block of SCAN_B units: the sums of the two counts.
__global__ void __launch_bounds__(SCAN_T) mc_unit_sums_kernel(const uint32_t* __restrict__ ucount,
                                                              long long U, long long* bsum2) {
  const long long base = (long long)blockIdx.x * SCAN_B + (long long)threadIdx.x * SCAN_V;
  unsigned long long w = 0;
#pragma unroll
  for (int k = 0; k < SCAN_V; k++)
    if (base + k < U) w += unit_widen(ucount[base + k]);
  unsigned long long total;
  block_exclusive_scan(w, &total);
  if (threadIdx.x == 0) {
    bsum2[2 * blockIdx.x] = (long long)(total & 0xFFFFFFFFull);
    bsum2[2 * blockIdx.x + 1] = (long long)(total >> 32);
  }
}

// Exclusive scan of the nb block sums (two counts) in place; the totals go
// to tot->nv and tot->nc.
__global__ void __launch_bounds__(1024) mc_scan_sums_kernel(long long* bsum2, long long nb,
                                                            McTotals* tot) {
  __shared__ long long sh[2][32];
  __shared__ long long carry[2];
  if (threadIdx.x < 2) carry[threadIdx.x] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long c0 = 0; c0 < nb; c0 += 1024) {
    const long long i = c0 + threadIdx.x;
    long long v[2], inc[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
      v[q] = i < nb ? bsum2[2 * i + q] : 0;
      inc[q] = v[q];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, inc[q], o);
        if (lane >= o) inc[q] += t;
      }
      if (lane == 31) sh[q][warp] = inc[q];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
      for (int q = 0; q < 2; q++) {
        long long w = sh[q][lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const long long t = __shfl_up_sync(0xffffffffu, w, o);
          if (lane >= o) w += t;
        }
        sh[q][lane] = w;
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 2; q++)
      if (i < nb) bsum2[2 * i + q] = carry[q] + (warp ? sh[q][warp - 1] : 0) + inc[q] - v[q];
    __syncthreads();
    if (threadIdx.x < 2) carry[threadIdx.x] += sh[threadIdx.x][31];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    tot->nv = carry[0];
    tot->nc = carry[1];
  }
}

// Pass 3: the slab's vertices and cubes in scan order.  Each thread takes
// SCAN_V consecutive units; for the active voxels of its units it forms the
// edge mask and cube flag from the sign words of the voxel's unit, the unit
// above it (y + 1), the units of the plane above, and the first column of the
// next unit of each, and writes the vertex id base and mask of the voxel
// (window plane p + 1), one edge-list entry per vertex (window voxel index
// * 4 + axis) and one entry per mixed cube (its cell, global plane and
// flag; the first triangle comes from the cube scan).
struct McEmit {
  McSlab c;
  const long long* bpre;  // exclusive prefixes of the scan blocks (2 per block)
  uint8_t* masks;
  int32_t* vbase;
  uint32_t* list;         // this slab's vertices, from list[0]
  McCube* cubes;          // this slab's cube entries, from cubes[0]
  long long id0;          // global id of the slab's first vertex
  long long u_split;      // first unit of the slab's last cube layer (-1: none)
  McTotals* tot;
  const McRun* run;       // when set: id0 = run->nv, cubes from cubes + run->n_carry
};

// the unit's sign words in x order, with the next unit's first sign as bit 64
struct McRow {
  unsigned long long w;
  uint32_t next;
};
__device__ __forceinline__ McRow load_row(const McSlab& c, int p, int y, int seg) {
  McRow r{0ull, 0u};
  if (p >= c.P || y >= c.Y) return r;
  const long long u = ((long long)p * c.Y + y) * c.S + seg;
  r.w = natural64(c.sign[u]);
  if (seg + 1 < c.S) r.next = c.sign[u + 1].x & 1u;
  return r;
}
__device__ __forceinline__ uint32_t bit_at(const McRow& r, int i) {
  return i < 64 ? (uint32_t)(r.w >> i) & 1u : r.next;
}

__global__ void __launch_bounds__(SCAN_T) mc_emit_kernel(const McEmit e, long long U) {
  const McSlab& c = e.c;
  long long id0 = e.id0;
  McCube* cubes = e.cubes;
  if (e.run) {
    if (e.run->overflow) return;
    id0 = e.run->nv;
    cubes += e.run->n_carry;
  }
  const long long base = (long long)blockIdx.x * SCAN_B + (long long)threadIdx.x * SCAN_V;
  uint32_t cnt[SCAN_V];
  unsigned long long w = 0;
#pragma unroll
  for (int k = 0; k < SCAN_V; k++) {
    cnt[k] = base + k < U ? c.ucount[base + k] : 0u;
    w += unit_widen(cnt[k]);
  }
  unsigned long long total;
  const unsigned long long ex = block_exclusive_scan(w, &total);
  long long vp = e.bpre[2 * blockIdx.x] + (long long)(ex & 0xFFFFFFFFull);
  long long cp = e.bpre[2 * blockIdx.x + 1] + (long long)(ex >> 32);
  for (int k = 0; k < SCAN_V; k++) {
    const long long u = base + k;
    if (u == e.u_split) e.tot->split = cp;
    if (!cnt[k]) continue;
    const int seg = (int)(u % c.S);
    const long long py = u / c.S;
    const int y = (int)(py % c.Y);
    const int p = (int)(py / c.Y);
    const int gz = c.gz0 + p;
    const int xb = seg * MC_SEG;
    const McRow A = load_row(c, p, y, seg), C = load_row(c, p, y + 1, seg);
    const McRow B = load_row(c, p + 1, y, seg), D = load_row(c, p + 1, y + 1, seg);
    const bool hy = y + 1 < c.Y, hz = p + 1 < c.P;
    const long long r0 = (long long)y * c.X;
    unsigned long long act = natural64(c.bits[u]);
    while (act) {
      const int i = __ffsll((long long)act) - 1;
      act &= act - 1;
      const int x = xb + i;
      const bool hx = x + 1 < c.X;
      const uint32_t a0 = bit_at(A, i), a1 = bit_at(A, i + 1);
      const uint32_t b0 = bit_at(B, i), c0 = bit_at(C, i);
      int m = (int)(hx & (a0 != a1)) | (int)(hy & (a0 != c0)) << 1 | (int)(hz & (a0 != b0)) << 2;
      int f = 0;
      if (hx && hy && hz)
        f = (int)(a0 | b0 << 1 | c0 << 2 | bit_at(D, i) << 3 | a1 << 4 | bit_at(B, i + 1) << 5 |
                  bit_at(C, i + 1) << 6 | bit_at(D, i + 1) << 7);
      // the case-158 edges on the grid's boundary lines (mc_fix158_kernel)
      if ((m & 1) && y == 0 && gz == 0 && f == 158) m &= ~1;
      if (x == c.X - 1 && (m & 6)) {
        if ((m & 2) && gz == 0 && cube_flag_src(c, x - 1, y, p) == 158) m &= ~2;
        if ((m & 4) && y == 0 && cube_flag_src(c, x - 1, 0, p) == 158) m &= ~4;
      }
      const long long wv = (long long)(p + 1) * c.XY + r0 + x;
      if (m) {
        e.vbase[wv] = (int32_t)(id0 + vp);
        e.masks[wv] = (uint8_t)m;
#pragma unroll
        for (int a = 0; a < 3; a++)
          if (m >> a & 1) e.list[vp++] = (uint32_t)(wv * 4 + a);
      }
      if (f != 0 && f != 255) {
        McCube q;
        q.r = (uint32_t)(r0 + x);
        q.gzf = (uint32_t)gz | (uint32_t)f << 24;
        q.tb = 0;
        cubes[cp++] = q;
      }
    }
  }
}

// The cube scan: each cube's first triangle, in cube-list order.
struct CubeTris {
  McCube* cubes;
  __device__ int count(long long i) const { return ntri_of((int)(cubes[i].gzf >> 24)); }
  __device__ void emit(long long i, long long k) const { cubes[i].tb = k; }
};
// ... over the run's new entries (from cubes + run->n_carry)
struct CubeTrisRun {
  McCube* cubes;
  const McRun* run;
  __device__ int count(long long i) const {
    return ntri_of((int)(cubes[run->n_carry + i].gzf >> 24));
  }
  __device__ void emit(long long i, long long k) const { cubes[run->n_carry + i].tb = k; }
};

// Pass 4: the triangles of cube entries [0, n) with n = n_carry + the
// slab's entries below its last cube layer (all of them on the last slab):
// vertex id of edge (voxel v, axis a) = vbase[v] + the set mask bits of v
// below a.  The case table is staged in shared memory (lanes read different
// cases).
struct McTris {
  const McCube* cubes;
  long long n_carry;
  int last;
  const McTotals* tot;
  const uint8_t* masks;
  const int32_t* vbase;
  int32_t* tris;
  long long cap;
  int X;
  long long XY;
  int zbase;  // global plane of window plane 0
  const McRun* run;  // when set: n_carry and the entry count from here
};

__global__ void __launch_bounds__(128) mc_tris_kernel(const McTris t, long long n_all) {
  __shared__ uint8_t cases[256][16];
  long long n_carry = t.n_carry;
  if (t.run) {
    if (t.run->overflow) return;
    n_carry = t.run->n_carry;
    n_all = n_carry + t.run->nc;
  }
  for (int i = threadIdx.x; i < 256 * 16; i += blockDim.x) cases[i >> 4][i & 15] = QJ_MC_CASES[i >> 4][i & 15];
  __syncthreads();
  const long long n = t.last ? n_all : n_carry + t.tot->split;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const McCube q = t.cubes[i];
    const int f = (int)(q.gzf >> 24);
    const int j = (int)(q.gzf & 0xFFFFFFu) - t.zbase;
    const int y = (int)(q.r / (uint32_t)t.X), x = (int)(q.r - (uint32_t)y * (uint32_t)t.X);
    long long k = q.tb;
    for (int tr = 0; tr < QJ_MC_MAX_TRIS && cases[f][3 * tr]; tr++, k++) {
      if (k >= t.cap) continue;
#pragma unroll
      for (int cc = 0; cc < 3; cc++) {
        const int ed = cases[f][3 * tr + cc];
        const long long v = (long long)(j + c_edge_off[ed][2]) * t.XY +
                            (long long)(y + c_edge_off[ed][1]) * t.X + (x + c_edge_off[ed][0]);
        const int a = c_edge_axis[ed];
        t.tris[3 * k + cc] = t.vbase[v] + __popc(t.masks[v] & ((1 << a) - 1));
      }
    }
  }
}

// The entries of the slab's last cube layer move to the front of the other
// cube list for the next slab: [n_carry + split, n_carry + nc) -> [0, ...).
__global__ void mc_carry_kernel(const McCube* __restrict__ src, McCube* __restrict__ dst,
                                long long n_carry, long long nc, const McTotals* tot,
                                const McRun* run) {
  if (run) {
    if (run->overflow) return;
    n_carry = run->n_carry;
    nc = run->nc;
  }
  const long long s0 = n_carry + tot->split;
  const long long n = n_carry + nc - s0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[s0 + i];
}

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
template <int POW_REF>
__device__ __forceinline__ double value64(const MapParams& m, const GridParams& g,
                                          const IterParams& it, const double p[3], double iso,
                                          unsigned long long* e64) {
  (*e64)++;
  if (it.lagrange) return lagrange_value64<POW_REF>(m, it, p, g.slice, iso);
  int ni;
  double dd;
  return q64::sub(escape64<POW_REF, false>(m, it, p, g.slice, &ni, &dd), iso);
}

template <int POW_REF, bool HYBRID>
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

template <bool BISECT, int POW_REF, bool HYBRID>
__global__ void __launch_bounds__(128) vertex_kernel(const __grid_constant__ MapParams m,
                                                     const GridParams g, const IterParams it,
                                                     const uint32_t* __restrict__ list, long long n,
                                                     long long id0, int c0,
                                                     const double* __restrict__ src,
                                                     double* __restrict__ verts, double iso,
                                                     DevStats* st, const McRun* run) {
  if (run) {
    if (run->overflow) return;
    n = run->n_new;
    id0 = run->nv;
  }
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
template <int POW_REF>
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
template <int POW_REF>
__global__ void __launch_bounds__(128) edge_start_kernel(const __grid_constant__ MapParams m,
                                                         const GridParams g, const IterParams it,
                                                         const uint32_t* __restrict__ list,
                                                         long long n, long long id0, int c0,
                                                         EdgeState* __restrict__ es,
                                                         double* __restrict__ verts, double iso,
                                                         uint32_t* park,
                                                         unsigned long long* n_park,
                                                         DevStats* st, const McRun* run) {
  if (run) {
    if (run->overflow) return;
    n = run->n_new;
    id0 = run->nv;
  }
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
template <int POW_REF>
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
template <int POW_REF>
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

// ------------------------------------------------ the run's bookkeeping

__global__ void mc_run_init_kernel(McRun* r, long long cap_v, long long cap_list,
                                   long long cap_cubes, long long cap_t) {
  McRun z{};
  z.cap_v = cap_v;
  z.cap_list = cap_list;
  z.cap_cubes = cap_cubes;
  z.cap_t = cap_t;
  *r = z;
}

__global__ void mc_run_slab_kernel(McRun* r, const McTotals* tot, int first) {
  if (!r->overflow) {
    const long long n_carry = first ? 0 : r->prev_nc - tot->split;
    if (!first) r->nt += tot->nt;
    const long long n_new = tot->nv, nc = tot->nc;
    if (r->nv + n_new > r->cap_v || n_new > r->cap_list || n_carry + nc > r->cap_cubes ||
        r->nv + n_new > 0x7FFFFFFFll) {
      r->overflow = 1;
    } else {
      r->n_carry = n_carry;
      r->n_new = n_new;
      r->nc = nc;
      return;
    }
  }
  // nothing more is written: every later phase sees empty counts
  r->n_carry = r->n_new = r->nc = 0;
}

__global__ void mc_run_next_kernel(McRun* r) {
  if (r->overflow) return;
  r->nv += r->n_new;
  r->prev_nc = r->nc;
}

__global__ void mc_run_final_kernel(McRun* r, const McTotals* tot, int any_slab) {
  if (!r->overflow && any_slab) r->nt += tot->nt;
  if (r->nt > r->cap_t) r->overflow = 1;
  r->n_filter = r->overflow ? 0 : r->nt;
}

// the run's outputs: vertices (FP64 and/or FP32) and the kept triangles
__global__ void mc_copy_out_kernel(const double* __restrict__ verts, double* __restrict__ v64,
                                   float* __restrict__ v32, const int32_t* __restrict__ kept,
                                   int32_t* __restrict__ tris, const McRun* run) {
  if (run->overflow) return;
  const long long nv3 = 3 * run->nv, nt3 = 3 * run->keep;
  const long long n = nv3 > nt3 ? nv3 : nt3;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < nv3) {
      if (v64) v64[i] = verts[i];
      if (v32) v32[i] = (float)verts[i];
    }
    if (i < nt3) tris[i] = kept[i];
  }
}

__global__ void mc_stats_add_kernel(DevStats* acc, const DevStats* st) {
  acc->voxel_iters += st->voxel_iters;
  acc->refined += st->refined;
  acc->nonfinite += st->nonfinite;
  for (int k = 0; k < 4; k++) acc->aux[k] += st->aux[k];
  acc->rerun += st->rerun;
  acc->rerun_iters += st->rerun_iters;
  acc->ff_evals += st->ff_evals;
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

long long mesh_units(int X, int Y, int planes) {
  return (long long)planes * Y * ((X + MC_SEG - 1) / MC_SEG);
}

static McSlab slab_of(const MeshWindow& w, const double* src, int P, int Pv, int gz0) {
  McSlab c;
  c.src = src;
  c.X = w.X;
  c.Y = w.Y;
  c.S = (w.X + MC_SEG - 1) / MC_SEG;
  c.P = P;
  c.Pv = Pv;
  c.gz0 = gz0;
  c.XY = (long long)w.X * w.Y;
  c.sign = reinterpret_cast<uint2*>(w.sign);
  c.bits = reinterpret_cast<uint2*>(w.bits);
  c.ucount = w.ucount;
  return c;
}

cudaError_t mesh_classify(const MeshWindow& w, const double* src, int P, int Pv, int gz0,
                          cudaStream_t s) {
  const McSlab c = slab_of(w, src, P, Pv, gz0);
  const long long U = mesh_units(w.X, w.Y, Pv);
  cudaError_t err;
  // units without activity keep these zero counts (the kernel stores the others)
  if ((err = cudaMemsetAsync(w.ucount, 0, (size_t)U * sizeof(uint32_t), s))) return err;
  const long long tasks = (long long)c.S * ((c.Y + MC_ROWS - 1) / MC_ROWS);
  const unsigned blocks = (unsigned)((tasks + MC_WARPS - 1) / MC_WARPS);
  if ((w.X % 2 == 0) && ((reinterpret_cast<uintptr_t>(src) & 15u) == 0))
    mc_classify_async_kernel<<<blocks, 32 * MC_WARPS, 0, s>>>(c);
  else
    mc_classify_kernel<false><<<blocks, 32 * MC_WARPS, 0, s>>>(c);
  const int nfix = w.X - 1 + w.Y - 1 + Pv;
  mc_fix158_kernel<<<(nfix + 127) / 128, 128, 0, s>>>(c);
  const long long nb = (U + SCAN_B - 1) / SCAN_B;
  mc_unit_sums_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(w.ucount, U, w.bsum);
  mc_scan_sums_kernel<<<1, 1024, 0, s>>>(w.bsum, nb, w.tot);
  return cudaGetLastError();
}

cudaError_t mesh_emit(const MeshWindow& w, const double* src, int P, int Pv, int gz0,
                      long long u_split, long long id0, McCube* cubes, cudaStream_t s) {
  McEmit e;
  e.c = slab_of(w, src, P, Pv, gz0);
  e.bpre = w.bsum;
  e.masks = w.masks;
  e.vbase = w.vbase;
  e.list = w.list;
  e.cubes = cubes;
  e.id0 = id0;
  e.u_split = u_split;
  e.tot = w.tot;
  e.run = nullptr;
  const long long U = mesh_units(w.X, w.Y, Pv);
  const long long nb = (U + SCAN_B - 1) / SCAN_B;
  mc_emit_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(e, U);
  return cudaGetLastError();
}

cudaError_t mesh_cube_scan(const MeshWindow& w, McCube* cubes, long long nc, long long t0,
                           cudaStream_t s) {
  if (nc <= 0) return cudaMemsetAsync(&w.tot->nt, 0, sizeof(long long), s);
  const long long nb = (nc + SCAN_B - 1) / SCAN_B;
  CubeTris op{cubes};
  count_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(op, nc, w.bsum, nullptr);
  scan_bsum_kernel<<<1, 1024, 0, s>>>(w.bsum, nb);
  emit_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(op, nc, w.bsum, t0, nullptr, nullptr);
  cudaError_t err = cudaGetLastError();
  if (err) return err;
  return cudaMemcpyAsync(&w.tot->nt, w.bsum + nb, sizeof(long long), cudaMemcpyDeviceToDevice, s);
}

cudaError_t mesh_triangles(const MeshWindow& w, const McCube* cubes, long long n_carry,
                           long long nc, bool last, int zbase, McCube* next, int32_t* tris,
                           long long cap, cudaStream_t s) {
  const long long n_all = n_carry + nc;
  if (n_all > 0) {
    McTris t;
    t.cubes = cubes;
    t.n_carry = n_carry;
    t.last = last ? 1 : 0;
    t.tot = w.tot;
    t.masks = w.masks;
    t.vbase = w.vbase;
    t.tris = tris;
    t.cap = cap;
    t.X = w.X;
    t.XY = (long long)w.X * w.Y;
    t.zbase = zbase;
    t.run = nullptr;
    const int blocks = (int)std::min<long long>((n_all + 127) / 128, (long long)sm_count() * 16);
    mc_tris_kernel<<<blocks, 128, 0, s>>>(t, n_all);
  }
  if (!last && nc > 0) {
    const int blocks = (int)std::min<long long>((nc + 255) / 256, (long long)sm_count() * 8);
    mc_carry_kernel<<<blocks, 256, 0, s>>>(cubes, next, n_carry, nc, w.tot, nullptr);
  }
  return cudaGetLastError();
}

template <int POW_REF>
static cudaError_t parked_start(const MapParams& m, const GridParams& g, const IterParams& it,
                                const MeshWindow& w, long long n, long long id0, int c0,
                                double* verts, double iso, DevStats* st, const EdgeScratch& sc,
                                cudaStream_t s) {
  const int blocks = (int)std::min<long long>((n + 127) / 128, (long long)sm_count() * 32);
  edge_start_kernel<POW_REF><<<blocks, 128, 0, s>>>(m, g, it, w.list, n, id0, c0,
                                                    static_cast<EdgeState*>(sc.state), verts, iso,
                                                    sc.list[0], sc.count, st, nullptr);
  return cudaGetLastError();
}

template <int POW_REF>
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
                               int pow_mode, double* verts, double iso, DevStats* st,
                               const EdgeScratch& sc, cudaStream_t s) {
  return pow_mode == 2 ? parked_finish<2>(m, g, it, verts, iso, st, sc, s)
         : pow_mode   ? parked_finish<1>(m, g, it, verts, iso, st, sc, s)
                      : parked_finish<0>(m, g, it, verts, iso, st, sc, s);
}

cudaError_t mesh_vertices(const MapParams& m, const GridParams& g, const IterParams& it,
                          int edge_mode, int pow_mode, bool hybrid, const MeshWindow& w,
                          long long n, long long id0, int c0, const double* src, double* verts,
                          double iso, DevStats* st, const EdgeScratch* scratch, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (edge_mode != 0 && hybrid && scratch)
    return pow_mode == 2 ? parked_start<2>(m, g, it, w, n, id0, c0, verts, iso, st, *scratch, s)
           : pow_mode   ? parked_start<1>(m, g, it, w, n, id0, c0, verts, iso, st, *scratch, s)
                        : parked_start<0>(m, g, it, w, n, id0, c0, verts, iso, st, *scratch, s);
  const int blocks = (int)std::min<long long>((n + 127) / 128, (long long)sm_count() * 32);
#define QJ_VK(B, P, H) \
  vertex_kernel<B, P, H><<<blocks, 128, 0, s>>>(m, g, it, w.list, n, id0, c0, src, verts, iso, st, \
                                                nullptr)
  if (edge_mode == 0)
    QJ_VK(false, 0, false);
  else if (pow_mode == 2)
    hybrid ? QJ_VK(true, 2, true) : QJ_VK(true, 2, false);
  else if (pow_mode)
    hybrid ? QJ_VK(true, 1, true) : QJ_VK(true, 1, false);
  else
    hybrid ? QJ_VK(true, 0, true) : QJ_VK(true, 0, false);
#undef QJ_VK
  return cudaGetLastError();
}

cudaError_t mesh_filter(const int32_t* tris, long long n, const double* verts, int32_t* out,
                        long long* bsum, long long* n_keep, cudaStream_t s) {
  if (n == 0) {
    *n_keep = 0;
    return cudaSuccess;
  }
  const long long nb = (n + SCAN_B - 1) / SCAN_B;
  DegenCount dc{tris, verts};
  count_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(dc, n, bsum, nullptr);
  scan_bsum_kernel<<<1, 1024, 0, s>>>(bsum, nb);
  DegenEmit de;
  de.tris = tris;
  de.v = verts;
  de.out = out;
  emit_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(de, n, bsum, 0, nullptr, nullptr);
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

// ---------------------------------------------- the fixed launch sequence

cudaError_t mesh_run_init(McRun* run, long long cap_v, long long cap_list, long long cap_cubes,
                          long long cap_t, cudaStream_t s) {
  mc_run_init_kernel<<<1, 1, 0, s>>>(run, cap_v, cap_list, cap_cubes, cap_t);
  return cudaGetLastError();
}

cudaError_t mesh_run_slab(McRun* run, const McTotals* tot, bool first, cudaStream_t s) {
  mc_run_slab_kernel<<<1, 1, 0, s>>>(run, tot, first ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t mesh_run_next(McRun* run, cudaStream_t s) {
  mc_run_next_kernel<<<1, 1, 0, s>>>(run);
  return cudaGetLastError();
}

cudaError_t mesh_run_final(McRun* run, const McTotals* tot, bool any_slab, cudaStream_t s) {
  mc_run_final_kernel<<<1, 1, 0, s>>>(run, tot, any_slab ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t mesh_emit_run(const MeshWindow& w, const double* src, int P, int Pv, int gz0,
                          long long u_split, McCube* cubes, const McRun* run, cudaStream_t s) {
  McEmit e;
  e.c = slab_of(w, src, P, Pv, gz0);
  e.bpre = w.bsum;
  e.masks = w.masks;
  e.vbase = w.vbase;
  e.list = w.list;
  e.cubes = cubes;
  e.id0 = 0;
  e.u_split = u_split;
  e.tot = w.tot;
  e.run = run;
  const long long U = mesh_units(w.X, w.Y, Pv);
  const long long nb = (U + SCAN_B - 1) / SCAN_B;
  mc_emit_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(e, U);
  return cudaGetLastError();
}

// The scan runs over as many blocks as the list could hold; blocks past the
// run's count sum to zero.  w.bsum holds mesh_scan_blocks(cap_cubes).
cudaError_t mesh_cube_scan_run(const MeshWindow& w, McCube* cubes, McRun* run,
                               long long cap_cubes, cudaStream_t s) {
  const long long nb = (std::max(cap_cubes, 1ll) + SCAN_B - 1) / SCAN_B;
  CubeTrisRun op{cubes, run};
  count_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(op, 0, w.bsum, &run->nc);
  scan_bsum_kernel<<<1, 1024, 0, s>>>(w.bsum, nb);
  emit_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(op, 0, w.bsum, 0, &run->nc, &run->nt);
  cudaError_t err = cudaGetLastError();
  if (err) return err;
  return cudaMemcpyAsync(&w.tot->nt, w.bsum + nb, sizeof(long long), cudaMemcpyDeviceToDevice, s);
}

cudaError_t mesh_vertices_run(const MapParams& m, const GridParams& g, const IterParams& it,
                              int edge_mode, int pow_mode, bool hybrid, const MeshWindow& w,
                              int c0, const double* src, double* verts, double iso, DevStats* st,
                              const EdgeScratch* scratch, const McRun* run, cudaStream_t s) {
  const int blocks = sm_count() * 32;
  if (edge_mode != 0 && hybrid && scratch) {
#define QJ_ES(P)                                                                              \
  edge_start_kernel<P><<<blocks, 128, 0, s>>>(m, g, it, w.list, 0, 0, c0,                    \
                                              static_cast<EdgeState*>(scratch->state), verts, \
                                              iso, scratch->list[0], scratch->count, st, run)
    if (pow_mode == 2)
      QJ_ES(2);
    else if (pow_mode)
      QJ_ES(1);
    else
      QJ_ES(0);
#undef QJ_ES
    return cudaGetLastError();
  }
#define QJ_VK(B, P, H) \
  vertex_kernel<B, P, H><<<blocks, 128, 0, s>>>(m, g, it, w.list, 0, 0, c0, src, verts, iso, st, run)
  if (edge_mode == 0)
    QJ_VK(false, 0, false);
  else if (pow_mode == 2)
    hybrid ? QJ_VK(true, 2, true) : QJ_VK(true, 2, false);
  else if (pow_mode)
    hybrid ? QJ_VK(true, 1, true) : QJ_VK(true, 1, false);
  else
    hybrid ? QJ_VK(true, 0, true) : QJ_VK(true, 0, false);
#undef QJ_VK
  return cudaGetLastError();
}

template <int POW_REF>
static cudaError_t parked_finish_fixed(const MapParams& m, const GridParams& g,
                                       const IterParams& it, double* verts, double iso,
                                       DevStats* st, const EdgeScratch& sc, cudaStream_t s) {
  EdgeState* es = static_cast<EdgeState*>(sc.state);
  const int pb = sm_count() * 32;
  cudaError_t err;
  // each round gives every parked edge one value; no edge needs more than 8
  for (int round = 0, cur = 0; round < 8; round++, cur ^= 1) {
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
  return cudaGetLastError();
}

cudaError_t mesh_parked_finish_fixed(const MapParams& m, const GridParams& g,
                                     const IterParams& it, int pow_mode, double* verts,
                                     double iso, DevStats* st, const EdgeScratch& sc,
                                     cudaStream_t s) {
  return pow_mode == 2 ? parked_finish_fixed<2>(m, g, it, verts, iso, st, sc, s)
         : pow_mode   ? parked_finish_fixed<1>(m, g, it, verts, iso, st, sc, s)
                      : parked_finish_fixed<0>(m, g, it, verts, iso, st, sc, s);
}

cudaError_t mesh_triangles_run(const MeshWindow& w, const McCube* cubes, bool last, int zbase,
                               McCube* next, int32_t* tris, long long cap, const McRun* run,
                               cudaStream_t s) {
  McTris t;
  t.cubes = cubes;
  t.n_carry = 0;
  t.last = last ? 1 : 0;
  t.tot = w.tot;
  t.masks = w.masks;
  t.vbase = w.vbase;
  t.tris = tris;
  t.cap = cap;
  t.X = w.X;
  t.XY = (long long)w.X * w.Y;
  t.zbase = zbase;
  t.run = run;
  mc_tris_kernel<<<sm_count() * 16, 128, 0, s>>>(t, 0);
  if (!last) mc_carry_kernel<<<sm_count() * 8, 256, 0, s>>>(cubes, next, 0, 0, w.tot, run);
  return cudaGetLastError();
}

cudaError_t mesh_filter_run(const int32_t* tris, const double* verts, int32_t* out,
                            long long* bsum, McRun* run, long long cap_t, cudaStream_t s) {
  const long long nb = (std::max(cap_t, 1ll) + SCAN_B - 1) / SCAN_B;
  DegenCount dc{tris, verts};
  count_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(dc, 0, bsum, &run->n_filter);
  scan_bsum_kernel<<<1, 1024, 0, s>>>(bsum, nb);
  DegenEmit de;
  de.tris = tris;
  de.v = verts;
  de.out = out;
  emit_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(de, 0, bsum, 0, &run->n_filter, nullptr);
  cudaError_t err = cudaGetLastError();
  if (err) return err;
  return cudaMemcpyAsync(&run->keep, bsum + nb, sizeof(long long), cudaMemcpyDeviceToDevice, s);
}

cudaError_t mesh_copy_out_run(const double* verts, double* v64, float* v32, const int32_t* kept,
                              int32_t* tris, const McRun* run, cudaStream_t s) {
  mc_copy_out_kernel<<<sm_count() * 8, 256, 0, s>>>(verts, v64, v32, kept, tris, run);
  return cudaGetLastError();
}

cudaError_t mesh_stats_add(DevStats* acc, const DevStats* st, cudaStream_t s) {
  mc_stats_add_kernel<<<1, 1, 0, s>>>(acc, st);
  return cudaGetLastError();
}

}  // namespace qj
