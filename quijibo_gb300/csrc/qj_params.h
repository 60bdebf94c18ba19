// Launch parameter blocks shared by the host library and the kernels.
// They are passed to kernels by value, so they live in the constant bank:
// every thread of a launch reads the same roots, which the constant cache
// broadcasts.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define QJ_MAX_ROOTS 128     // top + bottom roots of one map
#define QJ_MAX_INT_EXP 16    // largest exponent taken by the integer-power path

namespace qj {

// One rational map s * prod (q - t_i)^(sigma_t e_i) / prod (q - b_j)^(sigma_b f_j).
// Roots [0, nt) are top roots, [nt, nt + nb) bottom roots.
struct MapParams {
  int nt, nb;
  int all_int;                  // every effective exponent is an integer in [1, QJ_MAX_INT_EXP]
  int lagrange;                 // the FP32 and double-float tiers apply the map in
                                // RATIONAL_4D::evaluateLagrange order (set per call from
                                // the iteration form; the FP64 tier reads IterParams)
  double scale;                 // s (OPTIMIZE_3D::_expScaling)
  float scalef;
  float pad2_;
  double sigma[2];              // power scalars (top, bottom)
  alignas(16) double r64[QJ_MAX_ROOTS][4];  // roots (w, x, y, z)
  double e64[QJ_MAX_ROOTS];     // effective exponent sigma * e_i
  double ep[QJ_MAX_ROOTS];      // the root's own exponent e_i (POLYNOMIAL_4D::powers())
  alignas(16) float r32[QJ_MAX_ROOTS][4];
  alignas(8) float x32[QJ_MAX_ROOTS][2];  // {+e (top) or -e (bottom), integer exponent bits}
  float e32[QJ_MAX_ROOTS];
  int ie[QJ_MAX_ROOTS];         // integer exponent, or 0 when the exponent is not an integer
  // the two-voxel FP32 path: every value doubled into a (voxel A, voxel B) pair
  alignas(16) float2 rn2[QJ_MAX_ROOTS][4];  // (-t_c, -t_c) for c = w, x, y, z
  alignas(8) float2 ex2[QJ_MAX_ROOTS];      // (x32[i][0], x32[i][0])
  // the double-float head: each root coordinate and the scale as hi + lo
  alignas(8) float rff[QJ_MAX_ROOTS][4][2];
  float scale_ff[2];
};

// Cell-centred grid geometry (FIELD_3D) and the z-range of one launch.
struct GridParams {
  int X, Y, Z;       // full grid resolution
  int z0, z1;        // slices [z0, z1) are computed; outputs are indexed from z0
  double center[3];
  double half[3];    // lengths * 0.5
  double dx[3];      // lengths / res
  double R[3][3];    // rotation matrix of the grid quaternion
  double slice;      // the fourth (k) coordinate of every start point
  // the cell centre as an affine map of (x, y, z), p_c = a_c + sum_k b_ck idx_k,
  // as double-float pairs (hi, lo): the double-float re-run starts from it
  // without FP64 arithmetic
  float ffa[3][2];
  float ffb[3][3][2];
  float ffslice[2];
};

// A FIELD_3D sampled by trilinear lookup: first cell centre and 1/dx
// (FIELD_3D.cpp:971-980).
struct WeightGrid {
  int X, Y, Z;
  double corner[3];
  double inv[3];
};

// Escape-time iteration settings.
struct IterParams {
  int max_it;
  int want_de;
  double escape;     // escape radius (the reference hard-codes 2000; the workloads use 2)
  double band;       // FP32 voxels with |d| < band are re-evaluated in FP64
  double field_tol;  // ... and so are voxels with |log|q|| < field_tol
  // voxels whose tracked FP32 error exceeds est_tol * |log|q|| (est_tol is the
  // caller's rel_tol) are re-run:
  // with ff_head double-float iterations first (integer exponents), or in
  // FP64 when ff_head is 0.  est_tol 0 = off.
  double est_tol;
  int ff_head;
  int lagrange;      // the map in RATIONAL_4D::evaluateLagrange order (FP64 form)
  float field_tolf;  // field_tol and est_tol as FP32 (the FP32 kernels' tests)
  float est_tolf;
};

// Device-side counters of one field or mesh call.
struct DevStats {
  unsigned long long voxel_iters;   // executed map applications
  unsigned long long refined;       // voxels re-evaluated in FP64
  unsigned long long nonfinite;     // FP32 voxels that overflowed or underflowed
  unsigned long long tiles_done;    // work-queue position of the tile scheduler
  unsigned long long aux[4];
  unsigned long long rerun;         // length of the double-float re-run list
  unsigned long long rerun_iters;   // map applications of the re-runs
  unsigned long long ff_evals;      // mesher: double-float evaluations that decided a point
};

}  // namespace qj
