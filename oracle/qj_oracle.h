/*
 * CPU oracle for the QUIJIBO hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement, in double precision, of the reference's per-voxel
 * rational quaternion map, escape-time field, marching-cubes mesher and
 * tanh-weighted fitting energy.  Every function follows the operation order
 * of the reference routine it cites so that, on the same inputs, it rounds
 * like the reference's `Real=double` build.  It is the checker for the CUDA
 * library: only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark may call it.  The product path never does.
 *
 * Parity of this oracle is pinned against outputs of the reference itself,
 * compiled from its own sources in the development container (the fixtures
 * under tests/golden/ and the script that produced them).
 */
#ifndef QJ_ORACLE_H
#define QJ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A root-product polynomial: prod_i (q - roots[i])^(power_scalar * powers[i]).
 * roots are n quaternions stored (w, x, y, z). */
typedef struct {
  int n;
  const double* roots;
  const double* powers;
  double power_scalar;
} qjo_poly;

/* A rational map q -> s * top(q) / bottom(q) (bottom omitted when n == 0). */
typedef struct {
  qjo_poly top;
  qjo_poly bottom;
  double scale; /* OPTIMIZE_3D::_expScaling */
  int lagrange; /* 1: RATIONAL_4D::evaluateLagrange order (and lagrangeNonlinearValue) */
} qjo_map;

/* A cell-centred grid (FIELD_3D geometry).  rot is a quaternion (w,x,y,z)
 * rotating cell centres about center; slice is the fourth coordinate. */
typedef struct {
  int res[3];
  double center[3];
  double lengths[3];
  double rot[4];
  double slice;
} qjo_grid;

/* MT19937 draws as MERSENNETWISTER(seed).rand(): n values in [0,1]. */
void qjo_mt_rand(uint32_t seed, int n, double* out);

/* Cell centre of voxel (x,y,z). */
void qjo_cell_center(const qjo_grid* g, int x, int y, int z, double out[3]);

/* Quaternion power (w,x,y,z) -> q^e. */
void qjo_quat_pow(const double q[4], double e, double out[4]);

/* 0: qjo_quat_pow and the escape loops call the C library's acos/log/exp/sin/cos (as the
 * reference does); 1: the correctly rounded functions of qj_crmath.h. */
void qjo_set_libm(int correctly_rounded);

/* The correctly rounded functions themselves: fn 0 exp, 1 log, 2 sin,
 * 3 cos, 4 acos. */
double qjo_crm(int fn, double x);

/* prod_i (q - r_i)^(sigma e_i), left to right. */
void qjo_eval_factored(const qjo_poly* p, const double q[4], double out[4]);

/* One application of the map: out = s * top(q) / bottom(q). */
void qjo_map_apply(const qjo_map* m, const double q[4], double out[4]);

/* Escape-time field over z-slices [z0, z1): field[(z-z0)*X*Y + y*X + x] =
 * log|q_N|; de (optional) = |q_N| log|q_N| / |q_N'|; iters (optional) = the
 * executed iteration count.  nthreads <= 0 uses every core.
 * Returns the number of executed root terms (iterations x roots). */
int64_t qjo_field(const qjo_map* m, const qjo_grid* g, int max_it, double escape,
                  int z0, int z1, double* field, double* de, int32_t* iters,
                  int nthreads);

/* qjo_field restricted to the cells x in [x0, x1), y in [y0, y1) of slices
 * [z0, z1) of the same grid; field is (z1-z0) x (y1-y0) x (x1-x0). */
void qjo_field_window(const qjo_map* m, const qjo_grid* g, int max_it, double escape, int x0,
                      int x1, int y0, int y1, int z0, int z1, double* field, int nthreads);

/* log|q_N| - iso at an arbitrary point (TRIANGLE_MESH::nonlinearValue). */
double qjo_nonlinear_value(const qjo_map* m, const double p[3], double slice,
                           int max_it, double escape, double iso);

/* Marching cubes.
 *   classify: the full grid of values whose sign (> 0) classifies corners.
 *   mode 0: linear edge vertices from `classify` (computeStagedMarchingCubes);
 *   mode 1: bisection on the map (computeNonlinearEdgeInterpolations*).
 * Outputs: verts (3 doubles each, capacity max_verts), tris (3 ints each,
 * capacity max_tris, degenerate triangles removed), counts in *n_verts,
 * *n_tris.  *n_unbracketed counts edges whose end values do not bracket
 * zero.  Returns 0, or -1 when a capacity is too small. */
int qjo_mesh(const qjo_map* m, const qjo_grid* g, const double* classify, int mode,
             int max_it, double escape, double iso, double* verts, int64_t max_verts,
             int32_t* tris, int64_t max_tris, int64_t* n_verts, int64_t* n_tris,
             int64_t* n_unbracketed, int nthreads);

/* Trilinear lookup into a cell-centred weight grid (FIELD_3D::operator()(VEC3F)). */
double qjo_trilinear(const qjo_grid* g, const double* data, const double p[3]);

/* Tanh-weighted fitting score and its one-iteration analytic gradients
 * (OPTIMIZE_3D::computeScoreAP, computeExpGradientAP, computeTopGradientAP,
 * computeBottomGradientAP, compute{Top,Bottom}BulkScalarGradientAP).
 * grad layout: [log s, bottom exps (nb), top exps (nt), sigma_top, sigma_bottom].
 * Returns the score. */
double qjo_tanh_score_grad(const qjo_map* m, const qjo_grid* g, const qjo_grid* wg,
                           const double* weights, int max_it, double alpha,
                           double threshold, double* grad, double* field);

/* Central-difference root gradients of OPTIMIZE_3D's binary-score
 * objectives, step eps = lengths[0] / res[0], entry 4 k + c:
 *   kind 0: computeLogRationalCenteredGradient (OPTIMIZE_3D.cpp:2872-2951),
 *           top then bottom roots; kind 1: computeLogRationalBottomCenteredGradient
 *           (:2956-3008); both the binary score (:2275-2297) of
 *           computeLogRationalMap (:1907-1985);
 *   kind 2: computeCenteredGradient (:2761-2812), (binary + curvature score
 *           (:2497-2537)) / 2 of computeMap (:853-980), top roots.
 * dist / curv are fields on g.  *score (optional): the unmoved map's score. */
void qjo_centered_gradient(const qjo_map* m, const qjo_grid* g, int max_it, int kind,
                           const double* dist, const double* curv, double* grad, double* score);

/* Squared-error energy sum_k (D tanh(d(x_k)/D) - t_k)^2 of the distance
 * estimate d, D = d_sat (d_sat <= 0: sum (d - t)^2). */
double qjo_sqerr_energy(const qjo_map* m, int64_t n, const double* xyz, const double* target,
                        double slice, int max_it, double escape, double d_sat, int32_t* iters);

#ifdef __cplusplus
}
#endif
#endif
