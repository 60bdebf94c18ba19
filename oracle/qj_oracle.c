/*
 * CPU oracle for the QUIJIBO hot path -- TEST INFRASTRUCTURE ONLY (see
 * qj_oracle.h).  Compile with -ffp-contract=off so that no multiply-add is
 * fused: the reference's x86-64 double build rounds every product and sum
 * separately, and so does this file.
 *
 * Reference files cited below are paths inside the QUIJIBO project.
 */
#include "qj_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../quijibo_gb300/csrc/mc_cases.h"
#include "../quijibo_gb300/csrc/qj_crmath.h"

/* Transcendentals of qjo_quat_pow and of the escape loops' final log: the
 * C library's (the reference build's) or, with qjo_set_libm(1), the
 * correctly rounded ones of qj_crmath.h. */
static int g_libm_cr = 0;
void qjo_set_libm(int correctly_rounded) { g_libm_cr = correctly_rounded != 0; }

double qjo_crm(int fn, double x) {
  switch (fn) {
    case 0: return crm_exp(x);
    case 1: return crm_log(x);
    case 2: return crm_sin(x);
    case 3: return crm_cos(x);
    default: return crm_acos(x);
  }
}

/* SETTINGS.h:60 -- REAL_MIN is FLT_MIN whatever Real is. */
#define QJO_REAL_MIN ((double)FLT_MIN)

/* ------------------------------------------------------------------ */
/* MT19937 as MERSENNETWISTER (src/util/MERSENNETWISTER.h:147, 287-330):
 * Matsumoto & Nishimura's init_genrand seeding and tempering; rand()
 * scales a 32-bit draw by 1/(2^32-1). */
void qjo_mt_rand(uint32_t seed, int n, double* out) {
  uint32_t mt[624];
  int idx = 624;
  mt[0] = seed;
  for (int i = 1; i < 624; i++)
    mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
  for (int k = 0; k < n; k++) {
    if (idx >= 624) {
      for (int i = 0; i < 624; i++) {
        uint32_t y = (mt[i] & 0x80000000u) | (mt[(i + 1) % 624] & 0x7fffffffu);
        mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
      }
      idx = 0;
    }
    uint32_t y = mt[idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    out[k] = (double)y * (1.0 / 4294967295.0);
  }
}

/* ------------------------------------------------------------------ */
/* Quaternion helpers, all (w, x, y, z). */

/* QUATERNION::operator*= and operator*(q, q): QUATERNION.h:51-58,
 * QUATERNION.cpp:154-162 (identical formulas and order). */
static inline void qmul(const double a[4], const double b[4], double o[4]) {
  const double x = a[2] * b[3] - a[3] * b[2] + b[0] * a[1] + a[0] * b[1];
  const double y = a[3] * b[1] - a[1] * b[3] + b[0] * a[2] + a[0] * b[2];
  const double z = a[1] * b[2] - a[2] * b[1] + b[0] * a[3] + a[0] * b[3];
  const double w = a[0] * b[0] - a[1] * b[1] - b[2] * a[2] - a[3] * b[3];
  o[0] = w; o[1] = x; o[2] = y; o[3] = z;
}

/* QUATERNION::magnitude, QUATERNION.h:93. */
static inline double qmag(const double q[4]) {
  return sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
}

/* operator/(q, q): QUATERNION.cpp:174-182 -- l * (conj(r) * (1/|r|^2)). */
static inline void qdiv(const double l[4], const double r[4], double o[4]) {
  const double m2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3];
  const double inv = 1.0 / m2; /* operator/(QUATERNION, Real), QUATERNION.cpp:195-199 */
  double ri[4] = {r[0] * inv, -r[1] * inv, -r[2] * inv, -r[3] * inv};
  qmul(l, ri, o);
}

/* QUATERNION::pow, QUATERNION.cpp:375-393. */
void qjo_quat_pow(const double q[4], double e, double out[4]) {
  const double partial = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  const double qm = sqrt(partial + q[0] * q[0]);
  const double vm = sqrt(partial);
  const double vminv = (vm > 0.0) ? 1.0 / vm : 0.0;
  const double scale = e * (g_libm_cr ? crm_acos(q[0] / qm) : acos(q[0] / qm)) * vminv;
  const double mag = scale * vm;
  const double maginv = (mag > 0.0) ? 1.0 / mag : 0.0;
  const double exps = g_libm_cr ? crm_exp(e * crm_log(qm)) : exp(e * log(qm));
  double sn, cs;
  if (g_libm_cr) {
    crm_sincos(mag, &sn, &cs);
  } else {
    sn = sin(mag);
    cs = cos(mag);
  }
  const double scale2 = scale * exps * maginv * sn;
  out[0] = exps * cs;
  out[1] = scale2 * q[1];
  out[2] = scale2 * q[2];
  out[3] = scale2 * q[3];
}

/* POLYNOMIAL_4D::evaluateScaledPowerFactored, POLYNOMIAL_4D.cpp:912-923. */
void qjo_eval_factored(const qjo_poly* p, const double q[4], double out[4]) {
  double d[4], t[4], r[4];
  for (int c = 0; c < 4; c++) d[c] = q[c] - p->roots[c];
  qjo_quat_pow(d, p->power_scalar * p->powers[0], r);
  for (int i = 1; i < p->n; i++) {
    for (int c = 0; c < 4; c++) d[c] = q[c] - p->roots[4 * i + c];
    qjo_quat_pow(d, p->power_scalar * p->powers[i], t);
    double o[4];
    qmul(r, t, o);
    memcpy(r, o, sizeof r);
  }
  memcpy(out, r, sizeof r);
}

/* POLYNOMIAL_4D::evaluateRoot, POLYNOMIAL_4D.cpp:928-940. */
static void root_term(const qjo_poly* p, int i, const double q[4], double out[4]) {
  double d[4];
  for (int c = 0; c < 4; c++) d[c] = q[c] - p->roots[4 * i + c];
  qjo_quat_pow(d, p->power_scalar * p->powers[i], out);
}

/* RATIONAL_4D::evaluateLagrange, RATIONAL_4D.cpp:27-73: top and bottom
 * factors interleaved (times top_k, then divided by bottom_k), the leftovers
 * of the longer side after; without bottom roots the plain factored top. */
static void lagrange_apply(const qjo_map* m, const double q[4], double out[4]) {
  const int nt = m->top.n, nb = m->bottom.n;
  double r[4] = {1, 0, 0, 0}, t[4], o[4];
  const int same = nt > nb ? nb : nt;
  for (int k = 0; k < same; k++) {
    root_term(&m->top, k, q, t);
    qmul(r, t, o);
    root_term(&m->bottom, k, q, t);
    qdiv(o, t, r);
  }
  if (nt > nb) {
    for (int k = same; k < nt; k++) {
      root_term(&m->top, k, q, t);
      qmul(r, t, o);
      memcpy(r, o, sizeof r);
    }
  } else {
    for (int k = same; k < nb; k++) {
      root_term(&m->bottom, k, q, t);
      qdiv(r, t, o);
      memcpy(r, o, sizeof r);
    }
  }
  memcpy(out, r, sizeof r);
}

/* One map application as in the escape loop of
 * OPTIMIZE_3D::computeLogScaledPowerRationalMap (OPTIMIZE_3D.cpp:1331-1350),
 * or in the Lagrange order (TRIANGLE_MESH::computeLagrangeNonlinearSlice,
 * TRIANGLE_MESH.cpp:281-322). */
void qjo_map_apply(const qjo_map* m, const double q[4], double out[4]) {
  if (m->lagrange && m->bottom.n > 0) {
    lagrange_apply(m, q, out);
    for (int c = 0; c < 4; c++) out[c] *= m->scale;
    return;
  }
  double t[4];
  qjo_eval_factored(&m->top, q, t);
  if (m->bottom.n > 0) {
    double b[4];
    qjo_eval_factored(&m->bottom, q, b);
    qdiv(t, b, out);
  } else {
    memcpy(out, t, sizeof t);
  }
  for (int c = 0; c < 4; c++) out[c] *= m->scale;
}

/* |grad_q log|R(q)|| for the distance estimate: the norm of
 * sigma_t sum e_i (q-t_i)/|q-t_i|^2 - sigma_b sum f_j (q-b_j)/|q-b_j|^2.
 * (No reference counterpart; the reference tracks no derivative for this map.) */
static double log_gradient_norm(const qjo_map* m, const double q[4]) {
  double g[4] = {0, 0, 0, 0};
  for (int side = 0; side < 2; side++) {
    const qjo_poly* p = side ? &m->bottom : &m->top;
    const double sgn = side ? -1.0 : 1.0;
    for (int i = 0; i < p->n; i++) {
      double d[4];
      for (int c = 0; c < 4; c++) d[c] = q[c] - p->roots[4 * i + c];
      const double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3];
      const double k = sgn * p->power_scalar * p->powers[i] / d2;
      for (int c = 0; c < 4; c++) g[c] += k * d[c];
    }
  }
  return qmag(g);
}

/* FIELD_3D::cellCenter, FIELD_3D.cpp:818-841, with the rotation matrix of
 * QUATERNION::toRotationMatrix (QUATERNION.cpp:395-411) and the row-dot
 * MATRIX3 * VEC3 of MATRIX3.h:200-201. */
void qjo_cell_center(const qjo_grid* g, int x, int y, int z, double out[3]) {
  const double dx[3] = {g->lengths[0] / g->res[0], g->lengths[1] / g->res[1],
                        g->lengths[2] / g->res[2]};
  const int idx[3] = {x, y, z};
  double f[3];
  for (int c = 0; c < 3; c++) {
    const double half = g->lengths[c] * 0.5;
    f[c] = g->center[c] - half;
    f[c] += idx[c] * dx[c];
  }
  for (int c = 0; c < 3; c++) f[c] += dx[c] * 0.5;
  for (int c = 0; c < 3; c++) f[c] -= g->center[c];
  const double w = g->rot[0], qx = g->rot[1], qy = g->rot[2], qz = g->rot[3];
  double R[3][3];
  R[0][0] = 1 - 2 * qy * qy - 2 * qz * qz;
  R[0][1] = 2 * qx * qy - 2 * w * qz;
  R[0][2] = 2 * qx * qz + 2 * w * qy;
  R[1][0] = 2 * qx * qy + 2 * w * qz;
  R[1][1] = 1 - 2 * qx * qx - 2 * qz * qz;
  R[1][2] = 2 * qy * qz - 2 * w * qx;
  R[2][0] = 2 * qx * qz - 2 * w * qy;
  R[2][1] = 2 * qy * qz + 2 * w * qx;
  R[2][2] = 1 - 2 * qx * qx - 2 * qy * qy;
  double r[3];
  for (int c = 0; c < 3; c++) r[c] = R[c][0] * f[0] + R[c][1] * f[1] + R[c][2] * f[2];
  for (int c = 0; c < 3; c++) out[c] = r[c] + g->center[c];
}

/* The escape-time loop of OPTIMIZE_3D::computeLogScaledPowerRationalMap
 * (OPTIMIZE_3D.cpp:1317-1362) and TRIANGLE_MESH::nonlinearValue
 * (TRIANGLE_MESH.cpp:1755-1795) with the escape radius as a parameter.
 * The initial iterate is QUATERNION(x, y, z, slice): w = x, and the slice is
 * the k component.  Returns log|q_N|; *de and *iters are optional. */
static double escape_value(const qjo_map* m, const double p[3], double slice, int max_it,
                           double escape, double* de, int32_t* iters) {
  double q[4] = {p[0], p[1], p[2], slice};
  double mag = qmag(q);
  int it = 0, executed = 0;
  double dnorm = 1.0; /* |q_n'| */
  while (mag < escape && it < max_it) {
    double nq[4];
    if (de) dnorm *= log_gradient_norm(m, q);
    qjo_map_apply(m, q, nq);
    memcpy(q, nq, sizeof q);
    mag = qmag(q);
    if (de) dnorm *= mag;
    it++;
    executed++;
    if (mag < 10.0 * QJO_REAL_MIN) it = max_it;
  }
  const double f = g_libm_cr ? crm_log(mag) : log(mag);
  if (de) *de = mag * f / dnorm;
  if (iters) *iters = executed;
  return f;
}

int64_t qjo_field(const qjo_map* m, const qjo_grid* g, int max_it, double escape, int z0,
                  int z1, double* field, double* de, int32_t* iters, int nthreads) {
  const int X = g->res[0], Y = g->res[1];
  const int64_t slab = (int64_t)X * Y;
  const int rows = (z1 - z0) * Y;
  int64_t terms = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic) num_threads(nthreads) reduction(+ : terms)
#endif
  for (int r = 0; r < rows; r++) {
    const int z = z0 + r / Y, y = r % Y;
    for (int x = 0; x < X; x++) {
      double p[3], d;
      int32_t n;
      qjo_cell_center(g, x, y, z, p);
      const int64_t i = (int64_t)(z - z0) * slab + (int64_t)y * X + x;
      field[i] = escape_value(m, p, g->slice, max_it, escape, de ? &d : NULL, &n);
      if (de) de[i] = d;
      if (iters) iters[i] = n;
      terms += (int64_t)n * (m->top.n + m->bottom.n);
    }
  }
  return terms;
}

/* qjo_field over the window x in [x0, x1), y in [y0, y1) of slices
 * [z0, z1): the same cells of the same grid (cell centres of the full grid),
 * field[((z-z0)*(y1-y0) + (y-y0))*(x1-x0) + (x-x0)]. */
void qjo_field_window(const qjo_map* m, const qjo_grid* g, int max_it, double escape, int x0,
                      int x1, int y0, int y1, int z0, int z1, double* field, int nthreads) {
  const int W = x1 - x0, H = y1 - y0;
  const int rows = (z1 - z0) * H;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
#endif
  for (int r = 0; r < rows; r++) {
    const int z = z0 + r / H, y = y0 + r % H;
    for (int x = x0; x < x1; x++) {
      double p[3];
      int32_t n;
      qjo_cell_center(g, x, y, z, p);
      field[(int64_t)r * W + (x - x0)] = escape_value(m, p, g->slice, max_it, escape, NULL, &n);
    }
  }
}

/* TRIANGLE_MESH::lagrangeNonlinearValue, TRIANGLE_MESH.cpp:1684-1747: an
 * overflowing iterate reverts to the previous one and stops; an infinite
 * value returns FLT_MAX.  (The reference leaves the "previous" magnitude
 * unset when the first application overflows; here it is |q_0|.) */
static double lagrange_value(const qjo_map* m, const double p[3], double slice, int max_it,
                             double escape, double iso) {
  double q[4] = {p[0], p[1], p[2], slice}, prev[4];
  double mag = qmag(q), prev_mag = mag;
  memcpy(prev, q, sizeof q);
  int it = 0;
  while (mag < escape && it < max_it) {
    double nq[4];
    qjo_map_apply(m, q, nq);
    memcpy(q, nq, sizeof q);
    mag = qmag(q);
    if (isinf(mag)) {
      memcpy(q, prev, sizeof q);
      mag = prev_mag;
      break;
    }
    memcpy(prev, q, sizeof q);
    prev_mag = mag;
    it++;
    if (mag < 10.0 * QJO_REAL_MIN) it = max_it;
  }
  const double f = (g_libm_cr ? crm_log(mag) : log(mag)) - iso;
  return isinf(f) ? 3.40282346638528859812e+38 : f;
}

double qjo_nonlinear_value(const qjo_map* m, const double p[3], double slice, int max_it,
                           double escape, double iso) {
  if (m->lagrange) return lagrange_value(m, p, slice, max_it, escape, iso);
  return escape_value(m, p, slice, max_it, escape, NULL, NULL) - iso;
}

/* ------------------------------------------------------------------ */
/* Marching cubes. */

/* Edge id -> (lower-endpoint corner offset, axis), TRIANGLE_MESH.cpp:1569-1665. */
static const int EDGE_OFF[13][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 1}, {0, 1, 0},
                                    {1, 0, 0}, {1, 0, 0}, {1, 0, 1}, {1, 1, 0}, {0, 1, 0},
                                    {0, 0, 0}, {0, 0, 1}, {0, 1, 1}};
static const int EDGE_AXIS[13] = {0, 1, 2, 1, 2, 1, 2, 1, 2, 0, 0, 0, 0};

static inline int cube_flag(const double* v, int X, int64_t slab, int x, int y, int z) {
  const int64_t i = (int64_t)z * slab + (int64_t)y * X + x;
  /* corner weights NNN=1 NNP=2 NPN=4 NPP=8 PNN=16 PNP=32 PPN=64 PPP=128,
   * TRIANGLE_MESH.cpp:4929-4931 (first letter x, then y, then z) */
  return (v[i] > 0) + 2 * (v[i + slab] > 0) + 4 * (v[i + X] > 0) + 8 * (v[i + X + slab] > 0) +
         16 * (v[i + 1] > 0) + 32 * (v[i + 1 + slab] > 0) + 64 * (v[i + 1 + X] > 0) +
         128 * (v[i + 1 + X + slab] > 0);
}

/* TRIANGLE_MESH::midpointSearch, TRIANGLE_MESH.cpp:2232-2271. */
static void midpoint_search(const qjo_map* m, double slice, int max_it, double escape,
                            double iso, const double pv[3], double pval, const double nv[3],
                            double nval, int rec, double out[3], int* unbracketed) {
  double mid[3];
  for (int c = 0; c < 3; c++) mid[c] = pv[c] + nv[c];
  for (int c = 0; c < 3; c++) mid[c] *= 0.5;
  if (pval * nval >= 0.0) {
    *unbracketed = 1;
    memcpy(out, mid, sizeof mid);
    return;
  }
  if (rec >= 6) {
    memcpy(out, mid, sizeof mid);
    return;
  }
  const double mval = qjo_nonlinear_value(m, mid, slice, max_it, escape, iso);
  if (fabs(mval) < 1e-8) {
    memcpy(out, mid, sizeof mid);
    return;
  }
  if (mval < 0)
    midpoint_search(m, slice, max_it, escape, iso, pv, pval, mid, mval, rec + 1, out, unbracketed);
  else
    midpoint_search(m, slice, max_it, escape, iso, mid, mval, nv, nval, rec + 1, out, unbracketed);
}

int qjo_mesh(const qjo_map* m, const qjo_grid* g, const double* v, int mode, int max_it,
             double escape, double iso, double* verts, int64_t max_verts, int32_t* tris,
             int64_t max_tris, int64_t* n_verts, int64_t* n_tris, int64_t* n_unbracketed,
             int nthreads) {
  const int X = g->res[0], Y = g->res[1], Z = g->res[2];
  const int64_t slab = (int64_t)X * Y, N = slab * Z;
  /* 1. Active edges: every edge some cube's case places a vertex on
   * (the union of the per-cube std::map inserts, TRIANGLE_MESH.cpp:1471-1481).
   * Edge key = 3 * lower-endpoint linear index + axis; ascending key order
   * equals the std::map order of (VEC3I, VEC3I) pairs (VEC3.h:181-205). */
  unsigned char* used = (unsigned char*)calloc((size_t)N, 1); /* bit axis */
  for (int z = 0; z < Z - 1; z++)
    for (int y = 0; y < Y - 1; y++)
      for (int x = 0; x < X - 1; x++) {
        const int f = cube_flag(v, X, slab, x, y, z);
        const unsigned short mask = QJ_MC_EDGEMASK[f];
        for (int e = 1; e <= 12; e++)
          if (mask & (1 << (e - 1))) {
            const int64_t i = (int64_t)(z + EDGE_OFF[e][2]) * slab +
                              (int64_t)(y + EDGE_OFF[e][1]) * X + (x + EDGE_OFF[e][0]);
            used[i] |= (unsigned char)(1 << EDGE_AXIS[e]);
          }
      }
  /* 2. Vertex numbering: rank in key order. */
  int64_t* base = (int64_t*)malloc(sizeof(int64_t) * (size_t)(N + 1));
  int64_t nv = 0;
  for (int64_t i = 0; i < N; i++) {
    base[i] = nv;
    nv += (used[i] & 1) + ((used[i] >> 1) & 1) + ((used[i] >> 2) & 1);
  }
  base[N] = nv;
  *n_verts = nv;
  if (nv > max_verts) {
    free(used);
    free(base);
    return -1;
  }
  /* 3. Edge vertices (computeEdgeInterpolations TRIANGLE_MESH.cpp:2373-2425, or
   * computeNonlinearEdgeInterpolationsHuge TRIANGLE_MESH.cpp:2034-2123). */
  int64_t unbr = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads) reduction(+ : unbr)
#endif
  for (int64_t i = 0; i < N; i++) {
    if (!used[i]) continue;
    const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / slab);
    int64_t k = base[i];
    for (int a = 0; a < 3; a++) {
      if (!(used[i] & (1 << a))) continue;
      const int x1 = x + (a == 0), y1 = y + (a == 1), z1 = z + (a == 2);
      double p0[3], p1[3], out[3];
      qjo_cell_center(g, x, y, z, p0);
      qjo_cell_center(g, x1, y1, z1, p1);
      if (mode == 0) {
        double off[3];
        for (int c = 0; c < 3; c++) off[c] = p1[c] - p0[c];
        const double d0 = v[i], d1 = v[(int64_t)z1 * slab + (int64_t)y1 * X + x1];
        const double t = d0 / (d0 - d1);
        for (int c = 0; c < 3; c++) out[c] = p0[c] + t * off[c];
      } else {
        const double f0 = qjo_nonlinear_value(m, p0, g->slice, max_it, escape, iso);
        const double f1 = qjo_nonlinear_value(m, p1, g->slice, max_it, escape, iso);
        int bad = (f0 * f1 >= 0.0);
        const double *pv = p0, *nvx = p1;
        double pval = f0, nval = f1;
        if (f0 < 0) {
          pv = p1; nvx = p0; pval = f1; nval = f0;
        }
        midpoint_search(m, g->slice, max_it, escape, iso, pv, pval, nvx, nval, 0, out, &bad);
        unbr += bad;
      }
      memcpy(verts + 3 * k, out, sizeof out);
      k++;
    }
  }
  *n_unbracketed = unbr;
  /* 4. Triangles in cube scan order (z, y, x), the case's triangles in table
   * order, then the degenerate filter of TRIANGLE_MESH.cpp:737-756. */
  int64_t nt = 0;
  int overflow = 0;
  for (int z = 0; z < Z - 1; z++)
    for (int y = 0; y < Y - 1; y++)
      for (int x = 0; x < X - 1; x++) {
        const int f = cube_flag(v, X, slab, x, y, z);
        const unsigned char* c = QJ_MC_CASES[f];
        for (int t = 0; t < QJ_MC_MAX_TRIS && c[3 * t]; t++) {
          int64_t id[3];
          for (int j = 0; j < 3; j++) {
            const int e = c[3 * t + j];
            const int64_t i = (int64_t)(z + EDGE_OFF[e][2]) * slab +
                              (int64_t)(y + EDGE_OFF[e][1]) * X + (x + EDGE_OFF[e][0]);
            const int a = EDGE_AXIS[e];
            id[j] = base[i] + ((a > 0) ? (used[i] & 1) : 0) + ((a > 1) ? ((used[i] >> 1) & 1) : 0);
          }
          const double* v0 = verts + 3 * id[0];
          const double* v1 = verts + 3 * id[1];
          const double* v2 = verts + 3 * id[2];
          double d01[3], d02[3], d12[3];
          for (int q = 0; q < 3; q++) {
            d01[q] = v0[q] - v1[q];
            d02[q] = v0[q] - v2[q];
            d12[q] = v1[q] - v2[q];
          }
          const double e0 = sqrt(d01[0] * d01[0] + d01[1] * d01[1] + d01[2] * d01[2]);
          const double e1 = sqrt(d02[0] * d02[0] + d02[1] * d02[1] + d02[2] * d02[2]);
          const double e2 = sqrt(d12[0] * d12[0] + d12[1] * d12[1] + d12[2] * d12[2]);
          const double eps = 1e-7;
          if (e0 < eps || e1 < eps || e2 < eps) continue;
          if (nt >= max_tris) {
            overflow = 1;
            nt++;
            continue;
          }
          for (int j = 0; j < 3; j++) tris[3 * nt + j] = (int32_t)id[j];
          nt++;
        }
      }
  *n_tris = nt;
  free(used);
  free(base);
  return overflow ? -1 : 0;
}

/* ------------------------------------------------------------------ */
/* FIELD_3D::operator()(const VEC3F&), FIELD_3D.cpp:966-1029: clamped
 * trilinear interpolation with float weights. */
double qjo_trilinear(const qjo_grid* g, const double* data, const double p[3]) {
  const int X = g->res[0], Y = g->res[1], Z = g->res[2];
  const int64_t slab = (int64_t)X * Y;
  const double dx[3] = {g->lengths[0] / X, g->lengths[1] / Y, g->lengths[2] / Z};
  const double inv[3] = {1.0 / dx[0], 1.0 / dx[1], 1.0 / dx[2]};
  double pc[3], corner[3];
  for (int c = 0; c < 3; c++) corner[c] = g->center[c] - 0.5 * g->lengths[c];
  for (int c = 0; c < 3; c++) corner[c] += 0.5 * dx[c];
  for (int c = 0; c < 3; c++) pc[c] = p[c] - corner[c];
  for (int c = 0; c < 3; c++) pc[c] *= inv[c];
  int x0 = (int)pc[0], y0 = (int)pc[1], z0 = (int)pc[2];
  int x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
  x0 = x0 < 0 ? 0 : x0; y0 = y0 < 0 ? 0 : y0; z0 = z0 < 0 ? 0 : z0;
  x1 = x1 < 0 ? 0 : x1; y1 = y1 < 0 ? 0 : y1; z1 = z1 < 0 ? 0 : z1;
  x0 = x0 > X - 1 ? X - 1 : x0; y0 = y0 > Y - 1 ? Y - 1 : y0; z0 = z0 > Z - 1 ? Z - 1 : z0;
  x1 = x1 > X - 1 ? X - 1 : x1; y1 = y1 > Y - 1 ? Y - 1 : y1; z1 = z1 > Z - 1 ? Z - 1 : z1;
  const float s1 = (float)(pc[0] - x0), s0 = 1.0f - s1;
  const float t1 = (float)(pc[1] - y0), t0 = 1.0f - t1;
  const float u1 = (float)(pc[2] - z0), u0 = 1.0f - u1;
#define AT(xx, yy, zz) data[(xx) + (int64_t)(yy) * X + (int64_t)(zz) * slab]
  return u0 * (s0 * (t0 * AT(x0, y0, z0) + t1 * AT(x0, y1, z0)) +
               s1 * (t0 * AT(x1, y0, z0) + t1 * AT(x1, y1, z0))) +
         u1 * (s0 * (t0 * AT(x0, y0, z1) + t1 * AT(x0, y1, z1)) +
               s1 * (t0 * AT(x1, y0, z1) + t1 * AT(x1, y1, z1)));
#undef AT
}

/* ------------------------------------------------------------------ */
/* Tanh-weighted fitting score and its analytic gradients. */

/* QUATERNION::log, QUATERNION.cpp:352-365. */
static void qlog(const double q[4], double o[4]) {
  const double qm = qmag(q);
  const double vm = sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double vn[3] = {0, 0, 0};
  if (vm > 0)
    for (int c = 0; c < 3; c++) vn[c] = q[1 + c] / vm;
  const double a = acos(q[0] / qm);
  o[0] = log(qm);
  for (int c = 0; c < 3; c++) o[1 + c] = vn[c] * a;
}

/* QUATERNION::inverse, QUATERNION.cpp:167-172. */
static void qinv(const double q[4], double o[4]) {
  const double m2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  const double inv = 1.0 / m2;
  o[0] = q[0] * inv;
  o[1] = -q[1] * inv;
  o[2] = -q[2] * inv;
  o[3] = -q[3] * inv;
}

static double qdot(const double a[4], const double b[4]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
}

/* Per-voxel state of computeRationalMapAP (OPTIMIZE_3D.cpp:1374-1488) for
 * the gradient passes: the field value, whether the voxel overflowed, and
 * the factors P_i of the last iteration's products (evaluated at the last
 * iterate, as the POLYNOMIAL_CACHE forward/backward vectors are). */
typedef struct {
  double field;
  int overflowed, skipped;
  double *P; /* (nt + nb) x 4 */
} ap_voxel;

static void ap_eval(const qjo_map* m, const double p[3], double slice, int max_it,
                    ap_voxel* v) {
  const int nt = m->top.n, nb = m->bottom.n;
  double q[4] = {p[0], p[1], p[2], slice};
  double mag = qmag(q);
  v->overflowed = 0;
  v->skipped = 0;
  if (mag < 1e-8) { /* "if we hit the origin, move on" */
    v->skipped = 1;
    v->field = 0.0;
    return;
  }
  int it = 0;
  const double escape = 20.0;
  /* the reference reads the last iteration's caches; a voxel that never
   * iterates has none (its gradient terms are skipped here) */
  if (!(mag < escape && it < max_it)) v->skipped = 1;
  while (mag < escape && it < max_it) {
    double T[4], B[4], d[4];
    for (int side = 0; side < 2; side++) {
      const qjo_poly* pl = side ? &m->bottom : &m->top;
      double* acc = side ? B : T;
      double* Pbase = v->P + 4 * (side ? nt : 0);
      for (int i = 0; i < pl->n; i++) {
        for (int c = 0; c < 4; c++) d[c] = q[c] - pl->roots[4 * i + c];
        qjo_quat_pow(d, pl->power_scalar * pl->powers[i], Pbase + 4 * i);
        if (i == 0) {
          memcpy(acc, Pbase, 4 * sizeof(double));
        } else {
          double o[4];
          qmul(acc, Pbase + 4 * i, o);
          memcpy(acc, o, sizeof o);
        }
      }
    }
    if (nb > 0)
      qdiv(T, B, q);
    else
      memcpy(q, T, sizeof T);
    for (int c = 0; c < 4; c++) {
      if (isinf(T[c]) || isnan(T[c]) || (nb > 0 && (isinf(B[c]) || isnan(B[c])))) v->overflowed = 1;
      q[c] *= m->scale;
    }
    mag = qmag(q);
    if (isinf(mag) || isnan(mag)) v->overflowed = 1;
    it++;
  }
  v->field = log(mag);
}

double qjo_tanh_score_grad(const qjo_map* m, const qjo_grid* g, const qjo_grid* wg,
                           const double* weights, int max_it, double alpha, double threshold,
                           double* grad, double* field) {
  const int nt = m->top.n, nb = m->bottom.n;
  const int X = g->res[0], Y = g->res[1], Z = g->res[2];
  const int64_t N = (int64_t)X * Y * Z;
  const int P = 3 + nt + nb;
  double* acc = (double*)calloc((size_t)P, sizeof(double));
  double score = 0.0;
  ap_voxel v;
  v.P = (double*)malloc(sizeof(double) * 4 * (size_t)(nt + nb));
  double* S = (double*)malloc(sizeof(double) * 4 * (size_t)(nt + nb)); /* suffix products */
  const double logs = log(m->scale);
  /* voxel order z, y, x (weightScore's linear order; the reference's
   * gradient passes run y, z, x -- sums differ only by rounding) */
  for (int64_t idx = 0; idx < N; idx++) {
    const int x = (int)(idx % X), y = (int)((idx / X) % Y), z = (int)(idx / ((int64_t)X * Y));
    double p[3];
    qjo_cell_center(g, x, y, z, p);
    ap_eval(m, p, g->slice, max_it, &v);
    if (field) field[idx] = v.field;
    const double w = qjo_trilinear(wg, weights, p);
    /* weightScore, OPTIMIZE_3D.cpp:4502-4517 */
    score += (-tanh(alpha * v.field)) * w;
    /* computeExpGradientAP, OPTIMIZE_3D.cpp:3589-3625: every cell */
    {
      const double St = tanh(alpha * (v.field - threshold));
      acc[0] += -alpha * w * ((double)1.0 - St * St);
    }
    if (v.overflowed || v.skipped) continue;
    /* R and F from the last iteration's products */
    double T[4], B[4] = {1, 0, 0, 0}, R[4];
    for (int side = 0; side < 2; side++) {
      const int lo = side ? nt : 0, n = side ? nb : nt;
      if (n == 0) continue;
      double* dst = side ? B : T;
      memcpy(dst, v.P + 4 * lo, 4 * sizeof(double));
      for (int i = 1; i < n; i++) {
        double o[4];
        qmul(dst, v.P + 4 * (lo + i), o);
        memcpy(dst, o, sizeof o);
      }
      /* suffix products, POLYNOMIAL_4D.cpp:1066-1072 */
      memcpy(S + 4 * (lo + n - 1), v.P + 4 * (lo + n - 1), 4 * sizeof(double));
      for (int i = n - 2; i >= 0; i--) qmul(v.P + 4 * (lo + i), S + 4 * (lo + i + 1), S + 4 * (lo + i));
    }
    qdiv(T, B, R);
    const double Rm = qmag(R);
    if (Rm <= 0.0 || isinf(Rm)) continue;
    const double F = log(Rm) + logs;
    const double th = tanh(alpha * (F - threshold));
    const double dSdF = -alpha * w * (1 - th * th);
    const double RR = 1.0 / qdot(R, R);
    const double q0[4] = {p[0], p[1], p[2], g->slice};
    /* top roots: computeTopGradientAP (OPTIMIZE_3D.cpp:8905-9006) and the
     * bulk sigma_top term computeTopBulkScalarGradientAP (:9250-9358) */
    double left[4] = {1, 0, 0, 0};
    double bulk_top = 0.0, bulk_bot = 0.0;
    for (int i = 0; i < nt; i++) {
      /* left = forward[i-1] (advanced below), right = backward[i+1] */
      double right[4] = {1, 0, 0, 0};
      if (nt > 1 && i < nt - 1) memcpy(right, S + 4 * (i + 1), sizeof right);
      double base[4], pw[4], lg[4], mid[4], t1[4], dT[4], dR[4];
      for (int c = 0; c < 4; c++) base[c] = q0[c] - m->top.roots[4 * i + c];
      qjo_quat_pow(base, m->top.power_scalar * m->top.powers[i], pw);
      qlog(base, lg);
      for (int pass = 0; pass < 2; pass++) {
        const double k = pass == 0 ? m->top.power_scalar : m->top.powers[i];
        double kp[4] = {pw[0] * k, pw[1] * k, pw[2] * k, pw[3] * k};
        qmul(kp, lg, mid);
        qmul(left, mid, t1);
        qmul(t1, right, dT);
        qdiv(dT, B, dR);
        const double dFdt = RR * qdot(R, dR);
        const double dSdt = dSdF * dFdt;
        if (isnan(dSdt) || isinf(dSdt)) continue;
        if (pass == 0)
          acc[1 + nb + i] += dSdt;
        else
          bulk_top += dSdt;
      }
      /* advance the prefix: forward[i] */
      if (i == 0)
        memcpy(left, v.P, sizeof left);
      else {
        double o[4];
        qmul(left, v.P + 4 * i, o);
        memcpy(left, o, sizeof o);
      }
    }
    /* bottom roots: computeBottomGradientAP (:10012-10116) and
     * computeBottomBulkScalarGradientAP (:10360-10470) */
    double lb[4] = {1, 0, 0, 0};
    for (int j = 0; j < nb; j++) {
      double right[4] = {1, 0, 0, 0};
      if (nb > 1 && j < nb - 1) memcpy(right, S + 4 * (nt + j + 1), sizeof right);
      double base[4], pw[4], lg[4], li[4], mid[4], t0[4], t1[4], dB[4], dR[4];
      for (int c = 0; c < 4; c++) base[c] = q0[c] - m->bottom.roots[4 * j + c];
      qjo_quat_pow(base, m->bottom.power_scalar * m->bottom.powers[j], pw);
      qlog(base, lg);
      qinv(lg, li);
      const double minus1[4] = {-1, 0, 0, 0};
      for (int pass = 0; pass < 2; pass++) {
        if (pass == 0 && !(m->bottom.power_scalar > 0.0)) continue;
        if (pass == 1 && m->bottom.powers[j] < 1e-8) continue;
        const double k = 1.0 / (pass == 0 ? m->bottom.power_scalar : m->bottom.powers[j]);
        double kp[4] = {pw[0] * k, pw[1] * k, pw[2] * k, pw[3] * k};
        qmul(kp, li, mid);
        qmul(minus1, lb, t0);
        qmul(t0, mid, t1);
        qmul(t1, right, dB);
        qdiv(T, dB, dR);
        const double dFdt = RR * qdot(R, dR);
        const double dSdt = dSdF * dFdt;
        if (isnan(dSdt) || isinf(dSdt)) continue;
        if (pass == 0)
          acc[1 + j] += dSdt;
        else
          bulk_bot += dSdt;
      }
      if (j == 0)
        memcpy(lb, v.P + 4 * nt, sizeof lb);
      else {
        double o[4];
        qmul(lb, v.P + 4 * (nt + j), o);
        memcpy(lb, o, sizeof o);
      }
    }
    acc[1 + nb + nt] += bulk_top;
    acc[2 + nb + nt] += bulk_bot;
  }
  for (int k = 0; k < P; k++) grad[k] = acc[k];
  free(acc);
  free(v.P);
  free(S);
  return score;
}

/* Squared-error energy sum_k (d(x_k) - t_k)^2 of the distance estimate
 * (no reference counterpart; d as in qjo_field's de output). */
double qjo_sqerr_energy(const qjo_map* m, int64_t n, const double* xyz, const double* target,
                        double slice, int max_it, double escape, double d_sat, int32_t* iters) {
  double e = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : e)
#endif
  for (int64_t k = 0; k < n; k++) {
    double d;
    int32_t it;
    escape_value(m, xyz + 3 * k, slice, max_it, escape, &d, &it);
    if (iters) iters[k] = it;
    /* fitted value D tanh(d/D); +-D beyond |d| > 20 D (and for non-finite d) */
    double v = d;
    if (d_sat > 0) {
      if (!(fabs(d) <= 20.0 * d_sat))
        v = (d < 0 ? -1.0 : 1.0) * d_sat;
      else
        v = d_sat * tanh(d / d_sat);
    }
    const double r = v - target[k];
    e += r * r;
  }
  return e;
}

/* ------------------------------------------------------------------ */
/* Central-difference root gradients (qjo_centered_gradient). */

/* POLYNOMIAL_4D::evaluateFactored (POLYNOMIAL_4D.cpp:1080-1088): the roots'
 * plain product (q - r_0)(q - r_1)..., left to right. */
static void fd_factored(const double* roots, int n, const double q[4], double out[4]) {
  double r[4], d[4], t[4];
  for (int c = 0; c < 4; c++) r[c] = q[c] - roots[c];
  for (int i = 1; i < n; i++) {
    for (int c = 0; c < 4; c++) d[c] = q[c] - roots[4 * i + c];
    qmul(r, d, t);
    memcpy(r, t, sizeof r);
  }
  memcpy(out, r, sizeof r);
}

/* computeLogRationalMap (OPTIMIZE_3D.cpp:1907-1985) at one cell: escape 20,
 * iterate = s * (q top(q)) / (q bottom(q)); returns log|q|. */
static double fd_lograt_value(const double* top, int nt, const double* bot, int nb, double s,
                              const double p[3], double slice, int max_it) {
  double q[4] = {p[0], p[1], p[2], slice}, f[4], T[4], B[4], o[4];
  double mag = qmag(q);
  int it = 0;
  while (mag < 20.0 && it < max_it) {
    fd_factored(top, nt, q, f);
    qmul(q, f, T);
    if (nb > 0) {
      fd_factored(bot, nb, q, f);
      qmul(q, f, B);
      qdiv(T, B, o);
    } else {
      memcpy(o, T, sizeof o);
    }
    for (int c = 0; c < 4; c++) q[c] = o[c] * s;
    mag = qmag(q);
    it++;
  }
  return log(mag);
}

/* computeMap (OPTIMIZE_3D.cpp:853-980) at one cell: escape 10, iterate =
 * top.evaluateFactored(iterate); -1 if the orbit stays, else +1. */
static double fd_poly_value(const double* top, int nt, const double p[3], double slice,
                            int max_it) {
  double q[4] = {p[0], p[1], p[2], slice}, o[4];
  double mag = qmag(q);
  int it = 0;
  while (mag < 10.0 && it < max_it) {
    fd_factored(top, nt, q, o);
    memcpy(q, o, sizeof q);
    mag = qmag(q);
    it++;
  }
  return (it == max_it || mag < 10.0) ? -1.0 : 1.0;
}

/* OPTIMIZE_3D::kahanAdd (OPTIMIZE_3D.cpp:2486-2492) */
static void fd_kahan(double* sum, double add, double* err) {
  const double y = add - *err;
  const double t = *sum + y;
  *err = (t - *sum) - y;
  *sum = t;
}

/* computeScore / computeLogRationalScore of one root placement: the field,
 * then computeBinaryScore (:2275-2297) and, for kind 2,
 * computeCurvatureScore (:2497-2537). */
static double fd_score(const qjo_map* m, const double* top, const double* bot,
                       const qjo_grid* g, int max_it, int kind, const double* dist,
                       const double* curv, double* fractal) {
  const int X = g->res[0], Y = g->res[1], Z = g->res[2];
  const int64_t N = (int64_t)X * Y * Z;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic)
#endif
  for (int64_t i = 0; i < N; i++) {
    double p[3];
    qjo_cell_center(g, (int)(i % X), (int)((i / X) % Y), (int)(i / ((int64_t)X * Y)), p);
    fractal[i] = kind == 2 ? fd_poly_value(top, m->top.n, p, g->slice, max_it)
                           : fd_lograt_value(top, m->top.n, bot, m->bottom.n, m->scale, p,
                                             g->slice, max_it);
  }
  double score = 0.0;
  for (int64_t i = 0; i < N; i++) {
    double p[3];
    qjo_cell_center(g, (int)(i % X), (int)((i / X) % Y), (int)(i / ((int64_t)X * Y)), p);
    const double dt = (qjo_trilinear(g, dist, p) < 0) ? -1 : 1;
    const double ft = (fractal[i] > 0) ? -1 : 1;
    score += ft * dt;
  }
  const double binary = score / (double)N;
  if (kind != 2) return binary;
  double cs = 0.0, cs_err = 0.0, sum = 0.0, sum_err = 0.0;
  for (int64_t i = 0; i < N; i++) {
    const double sign = (dist[i] < 0) ? 1 : -1;
    const double adding = sign * curv[i];
    fd_kahan(&cs, adding * fractal[i], &cs_err);
    fd_kahan(&sum, fabs(adding), &sum_err);
  }
  return (binary + cs / sum) * 0.5;
}

void qjo_centered_gradient(const qjo_map* m, const qjo_grid* g, int max_it, int kind,
                           const double* dist, const double* curv, double* grad, double* score) {
  const int nt = m->top.n, nb = m->bottom.n;
  const int64_t N = (int64_t)g->res[0] * g->res[1] * g->res[2];
  const double eps = g->lengths[0] / g->res[0];
  double* top = (double*)malloc(sizeof(double) * 4 * (nt > 0 ? nt : 1));
  double* bot = (double*)malloc(sizeof(double) * 4 * (nb > 0 ? nb : 1));
  double* fractal = (double*)malloc(sizeof(double) * (size_t)N);
  if (nt > 0) memcpy(top, m->top.roots, sizeof(double) * 4 * (size_t)nt);
  if (nb > 0) memcpy(bot, m->bottom.roots, sizeof(double) * 4 * (size_t)nb);
  const int k0 = kind == 1 ? nt : 0;
  const int nk = kind == 0 ? nt + nb : kind == 1 ? nb : nt;
  for (int k = 0; k < nk; k++) {
    double* root = (k0 + k < nt) ? top + 4 * (k0 + k) : bot + 4 * (k0 + k - nt);
    for (int c = 0; c < 4; c++) {
      const double keep = root[c];
      root[c] = keep + eps;
      const double right = fd_score(m, top, bot, g, max_it, kind, dist, curv, fractal);
      root[c] = keep - eps;
      const double left = fd_score(m, top, bot, g, max_it, kind, dist, curv, fractal);
      root[c] = keep;
      grad[4 * k + c] = (right - left) / (2.0 * eps);
    }
  }
  if (score) *score = fd_score(m, top, bot, g, max_it, kind, dist, curv, fractal);
  free(top);
  free(bot);
  free(fractal);
}
