// Device-side building blocks of the QUIJIBO hot path on sm_103a.
//
// Quaternions are (w, x, y, z) as in the reference's QUATERNION
// (src/algebra/QUATERNION.h:150-154).  Two arithmetic families live here:
//
//  * q64:: reference-exact FP64.  Every product and sum is rounded on its
//    own (__dmul_rn / __dadd_rn, never fused), in the reference's operation
//    order, so that the FP64 field rounds like the reference's Real=double
//    build except inside the libm transcendentals.
//  * q32:: FP32 bulk arithmetic written for the FMA pipe (fused, reordered).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qj_crmath.h"
#include "qj_params.h"

namespace qj {

// --------------------------------------------------------------------- FP64
namespace q64 {

struct Q {
  double w, x, y, z;
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// QUATERNION::operator*= / operator*(q,q): QUATERNION.h:51-58, QUATERNION.cpp:154-162.
__device__ __forceinline__ Q qmul(const Q& a, const Q& b) {
  Q o;
  o.x = add(add(sub(mul(a.y, b.z), mul(a.z, b.y)), mul(b.w, a.x)), mul(a.w, b.x));
  o.y = add(add(sub(mul(a.z, b.x), mul(a.x, b.z)), mul(b.w, a.y)), mul(a.w, b.y));
  o.z = add(add(sub(mul(a.x, b.y), mul(a.y, b.x)), mul(b.w, a.z)), mul(a.w, b.z));
  o.w = sub(sub(sub(mul(a.w, b.w), mul(a.x, b.x)), mul(b.y, a.y)), mul(a.z, b.z));
  return o;
}

// sum of squares in the order of QUATERNION::magnitude (QUATERNION.h:93)
__device__ __forceinline__ double norm2(const Q& q) {
  return add(add(add(mul(q.w, q.w), mul(q.x, q.x)), mul(q.y, q.y)), mul(q.z, q.z));
}

__device__ __forceinline__ double mag(const Q& q) { return __dsqrt_rn(norm2(q)); }

// operator/(q,q), QUATERNION.cpp:174-182: l * (conj(r) * (1 / |r|^2)).
__device__ __forceinline__ Q qdiv(const Q& l, const Q& r) {
  const double inv = __ddiv_rn(1.0, norm2(r));
  Q ri;
  ri.w = mul(r.w, inv);
  ri.x = mul(-r.x, inv);
  ri.y = mul(-r.y, inv);
  ri.z = mul(-r.z, inv);
  return qmul(l, ri);
}

// QUATERNION::pow, QUATERNION.cpp:375-393.
__device__ __forceinline__ Q qpow(const Q& q, double e) {
  const double partial = add(add(mul(q.x, q.x), mul(q.y, q.y)), mul(q.z, q.z));
  const double qm = __dsqrt_rn(add(partial, mul(q.w, q.w)));
  const double vm = __dsqrt_rn(partial);
  const double vminv = (vm > 0.0) ? __ddiv_rn(1.0, vm) : 0.0;
  const double scale = mul(mul(e, acos(__ddiv_rn(q.w, qm))), vminv);
  const double m = mul(scale, vm);
  const double minv = (m > 0.0) ? __ddiv_rn(1.0, m) : 0.0;
  const double exps = exp(mul(e, log(qm)));
  double s, c;
  sincos(m, &s, &c);
  const double scale2 = mul(mul(mul(scale, exps), minv), s);
  Q o;
  o.w = mul(exps, c);
  o.x = mul(scale2, q.x);
  o.y = mul(scale2, q.y);
  o.z = mul(scale2, q.z);
  return o;
}

// QUATERNION::pow with correctly rounded acos, log, exp, sin and cos
// (qj_crmath.h) in place of the device library's: the reference's operation
// order, and the values a C library with correctly rounded transcendentals
// would give.
__device__ __forceinline__ Q qpow_cr(const Q& q, double e) {
  const double partial = add(add(mul(q.x, q.x), mul(q.y, q.y)), mul(q.z, q.z));
  const double qm = __dsqrt_rn(add(partial, mul(q.w, q.w)));
  const double vm = __dsqrt_rn(partial);
  const double vminv = (vm > 0.0) ? __ddiv_rn(1.0, vm) : 0.0;
  const double scale = mul(mul(e, crm_acos(__ddiv_rn(q.w, qm))), vminv);
  const double m = mul(scale, vm);
  const double minv = (m > 0.0) ? __ddiv_rn(1.0, m) : 0.0;
  const double exps = crm_exp(mul(e, crm_log(qm)));
  double s, c;
  crm_sincos(m, &s, &c);
  const double scale2 = mul(mul(mul(scale, exps), minv), s);
  Q o;
  o.w = mul(exps, c);
  o.x = mul(scale2, q.x);
  o.y = mul(scale2, q.y);
  o.z = mul(scale2, q.z);
  return o;
}

// Integer power by repeated products (exact algebra, FP64 rounding).
__device__ __forceinline__ Q qpow_int(const Q& d, int n) {
  Q r = d;
  for (int k = 1; k < n; k++) r = qmul(r, d);
  return r;
}

}  // namespace q64

// --------------------------------------------------------------------- FP32
namespace q32 {

struct Q {
  float w, x, y, z;
};

__device__ __forceinline__ Q qmul(const Q& a, const Q& b) {
  Q o;
  o.w = fmaf(-a.z, b.z, fmaf(-a.y, b.y, fmaf(-a.x, b.x, a.w * b.w)));
  o.x = fmaf(-a.z, b.y, fmaf(a.y, b.z, fmaf(a.x, b.w, a.w * b.x)));
  o.y = fmaf(a.z, b.x, fmaf(a.y, b.w, fmaf(-a.x, b.z, a.w * b.y)));
  o.z = fmaf(a.z, b.w, fmaf(-a.y, b.x, fmaf(a.x, b.y, a.w * b.z)));
  return o;
}

// a * conj(b)
__device__ __forceinline__ Q qmul_conj(const Q& a, const Q& b) {
  Q o;
  o.w = fmaf(a.z, b.z, fmaf(a.y, b.y, fmaf(a.x, b.x, a.w * b.w)));
  o.x = fmaf(a.z, b.y, fmaf(-a.y, b.z, fmaf(a.x, b.w, -a.w * b.x)));
  o.y = fmaf(-a.z, b.x, fmaf(a.y, b.w, fmaf(a.x, b.z, -a.w * b.y)));
  o.z = fmaf(a.z, b.w, fmaf(a.y, b.x, fmaf(-a.x, b.y, -a.w * b.z)));
  return o;
}

__device__ __forceinline__ Q qsq(const Q& a) {
  Q o;
  const float w2 = a.w + a.w;
  o.w = fmaf(-a.z, a.z, fmaf(-a.y, a.y, fmaf(-a.x, a.x, a.w * a.w)));
  o.x = w2 * a.x;
  o.y = w2 * a.y;
  o.z = w2 * a.z;
  return o;
}

__device__ __forceinline__ float norm2(const Q& q) {
  return fmaf(q.z, q.z, fmaf(q.y, q.y, fmaf(q.x, q.x, q.w * q.w)));
}

// FP32 error tracking along an orbit.  err is a first-order estimate of the
// relative error of q_n: each map application scales the incoming relative
// error by |grad log|R|| * |q| (the log-derivative the distance estimate
// tracks) and adds ERR_STEP of fresh rounding (24-root maps round about
// 100 times per application; ERR_STEP = 64 ulp covers them in RMS).
constexpr float EPS32 = 5.9604645e-8f;  // 2^-24
constexpr float ERR_STEP = 64.f * EPS32;

__device__ __forceinline__ float propagate_err(float err, float gg, float m2_in) {
  float amp;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(amp) : "f"(gg * m2_in));
  return fmaf(err, amp, ERR_STEP);
}

// the same with another per-application step (the double-float model)
__device__ __forceinline__ float propagate_err_step(float err, float gg, float m2_in,
                                                    float step) {
  float amp;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(amp) : "f"(gg * m2_in));
  return fmaf(err, amp, step);
}

// |q|^2 = m2 is within its FP32 error of the escape radius squared
__device__ __forceinline__ bool near_radius(float m2, float esc2, float err) {
  return fabsf(m2 - esc2) < 2.f * err * esc2;
}

// 1/x by the MUFU reciprocal (PTX rcp.approx.ftz.f32): about 1 ulp, subnormal
// x taken as 0 (result inf).  Both FP32 paths use it so their values agree bit
// for bit.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Integer power 1..QJ_MAX_INT_EXP by square-and-multiply (powers of one
// quaternion commute, so any order is exact algebra).
__device__ __forceinline__ Q qpow_int(const Q& d, int n) {
  if (n == 1) return d;
  if (n == 2) return qsq(d);
  Q r = d, b = d;
  bool first = true;
  while (n) {
    if (n & 1) {
      r = first ? b : qmul(r, b);
      first = false;
    }
    n >>= 1;
    if (n) b = qsq(b);
  }
  return r;
}

// General power in FP32, the polar form of QUATERNION::pow (QUATERNION.cpp:375-393).
__device__ __forceinline__ Q qpow(const Q& q, float e) {
  const float partial = fmaf(q.z, q.z, fmaf(q.y, q.y, q.x * q.x));
  const float qm = sqrtf(fmaf(q.w, q.w, partial));
  const float vm = sqrtf(partial);
  const float vminv = (vm > 0.0f) ? 1.0f / vm : 0.0f;
  const float scale = e * acosf(q.w / qm) * vminv;
  const float m = scale * vm;
  const float minv = (m > 0.0f) ? 1.0f / m : 0.0f;
  const float exps = exp2f(e * log2f(qm));
  float s, c;
  sincosf(m, &s, &c);
  const float scale2 = scale * exps * minv * s;
  return Q{exps * c, scale2 * q.x, scale2 * q.y, scale2 * q.z};
}

}  // namespace q32

// ------------------------------------------------------- FP32, two voxels
// The q32 arithmetic on (voxel A, voxel B) pairs: every operation is the
// packed f32x2 form of the q32 one (fma.rn.f32x2 and friends, one issue slot
// for two lanes of work), in the same order, so each half of a result is
// bit-identical to the scalar q32 value of its voxel.
namespace q32x2 {

struct Q2 {
  float2 w, x, y, z;
};

__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 pair(float a) { return make_float2(a, a); }

__device__ __forceinline__ Q2 qmul(const Q2& a, const Q2& b) {
  Q2 o;
  o.w = fma2(neg2(a.z), b.z, fma2(neg2(a.y), b.y, fma2(neg2(a.x), b.x, mul2(a.w, b.w))));
  o.x = fma2(neg2(a.z), b.y, fma2(a.y, b.z, fma2(a.x, b.w, mul2(a.w, b.x))));
  o.y = fma2(a.z, b.x, fma2(a.y, b.w, fma2(neg2(a.x), b.z, mul2(a.w, b.y))));
  o.z = fma2(a.z, b.w, fma2(neg2(a.y), b.x, fma2(a.x, b.y, mul2(a.w, b.z))));
  return o;
}

__device__ __forceinline__ Q2 qmul_conj(const Q2& a, const Q2& b) {
  Q2 o;
  o.w = fma2(a.z, b.z, fma2(a.y, b.y, fma2(a.x, b.x, mul2(a.w, b.w))));
  o.x = fma2(a.z, b.y, fma2(neg2(a.y), b.z, fma2(a.x, b.w, mul2(neg2(a.w), b.x))));
  o.y = fma2(neg2(a.z), b.x, fma2(a.y, b.w, fma2(a.x, b.z, mul2(neg2(a.w), b.y))));
  o.z = fma2(a.z, b.w, fma2(a.y, b.x, fma2(neg2(a.x), b.y, mul2(neg2(a.w), b.z))));
  return o;
}

__device__ __forceinline__ Q2 qsq(const Q2& a) {
  Q2 o;
  const float2 w2 = add2(a.w, a.w);
  o.w = fma2(neg2(a.z), a.z, fma2(neg2(a.y), a.y, fma2(neg2(a.x), a.x, mul2(a.w, a.w))));
  o.x = mul2(w2, a.x);
  o.y = mul2(w2, a.y);
  o.z = mul2(w2, a.z);
  return o;
}

__device__ __forceinline__ float2 norm2(const Q2& q) {
  return fma2(q.z, q.z, fma2(q.y, q.y, fma2(q.x, q.x, mul2(q.w, q.w))));
}

__device__ __forceinline__ q32::Q lo(const Q2& a) { return q32::Q{a.w.x, a.x.x, a.y.x, a.z.x}; }
__device__ __forceinline__ q32::Q hi(const Q2& a) { return q32::Q{a.w.y, a.x.y, a.y.y, a.z.y}; }
__device__ __forceinline__ Q2 join(const q32::Q& a, const q32::Q& b) {
  return Q2{make_float2(a.w, b.w), make_float2(a.x, b.x), make_float2(a.y, b.y),
            make_float2(a.z, b.z)};
}

}  // namespace q32x2

// ----------------------------------------------------------------- geometry

// FIELD_3D::cellCenter (FIELD_3D.cpp:818-841) in reference operation order;
// R is QUATERNION::toRotationMatrix of the grid rotation, computed on the host.
__device__ __forceinline__ void cell_center(const GridParams& g, int x, int y, int z,
                                            double out[3]) {
  using namespace q64;
  const int idx[3] = {x, y, z};
  double f[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    f[c] = sub(g.center[c], g.half[c]);
    f[c] = add(f[c], mul((double)idx[c], g.dx[c]));
    f[c] = add(f[c], mul(g.dx[c], 0.5));
    f[c] = sub(f[c], g.center[c]);
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const double r = add(add(mul(g.R[c][0], f[0]), mul(g.R[c][1], f[1])), mul(g.R[c][2], f[2]));
    out[c] = add(r, g.center[c]);
  }
}

// FIELD_3D::operator()(const VEC3F&), FIELD_3D.cpp:966-1029.
__device__ __forceinline__ double trilinear(const WeightGrid& wg, const double* __restrict__ data,
                            const double p[3]) {
  using namespace q64;
  double pc[3];
#pragma unroll
  for (int c = 0; c < 3; c++) pc[c] = mul(sub(p[c], wg.corner[c]), wg.inv[c]);
  int x0 = (int)pc[0], y0 = (int)pc[1], z0 = (int)pc[2];
  int x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
  x0 = x0 < 0 ? 0 : x0; y0 = y0 < 0 ? 0 : y0; z0 = z0 < 0 ? 0 : z0;
  x1 = x1 < 0 ? 0 : x1; y1 = y1 < 0 ? 0 : y1; z1 = z1 < 0 ? 0 : z1;
  x0 = x0 > wg.X - 1 ? wg.X - 1 : x0; y0 = y0 > wg.Y - 1 ? wg.Y - 1 : y0;
  z0 = z0 > wg.Z - 1 ? wg.Z - 1 : z0;
  x1 = x1 > wg.X - 1 ? wg.X - 1 : x1; y1 = y1 > wg.Y - 1 ? wg.Y - 1 : y1;
  z1 = z1 > wg.Z - 1 ? wg.Z - 1 : z1;
  const float s1 = __double2float_rn(sub(pc[0], (double)x0)), s0 = __fsub_rn(1.0f, s1);
  const float t1 = __double2float_rn(sub(pc[1], (double)y0)), t0 = __fsub_rn(1.0f, t1);
  const float u1 = __double2float_rn(sub(pc[2], (double)z0)), u0 = __fsub_rn(1.0f, u1);
  const long long XY = (long long)wg.X * wg.Y;
  auto at = [&](int x, int y, int z) { return data[x + (long long)y * wg.X + z * XY]; };
  const double a = add(mul((double)s0, add(mul((double)t0, at(x0, y0, z0)), mul((double)t1, at(x0, y1, z0)))),
                       mul((double)s1, add(mul((double)t0, at(x1, y0, z0)), mul((double)t1, at(x1, y1, z0)))));
  const double b = add(mul((double)s0, add(mul((double)t0, at(x0, y0, z1)), mul((double)t1, at(x0, y1, z1)))),
                       mul((double)s1, add(mul((double)t0, at(x1, y0, z1)), mul((double)t1, at(x1, y1, z1)))));
  return add(mul((double)u0, a), mul((double)u1, b));
}

// ------------------------------------------------------- FP64 escape loop

// prod_{i in [lo, hi)} (q - r_i)^(e_i), left to right, as
// POLYNOMIAL_4D::evaluateScaledPowerFactored (POLYNOMIAL_4D.cpp:912-923);
// with DE, adds sign * sum e_i (q - r_i) / |q - r_i|^2 to g.
// One root term (q - r_i)^(e_i) (POLYNOMIAL_4D::evaluateRoot,
// POLYNOMIAL_4D.cpp:928-940); with DE, adds sign * e_i d/|d|^2 to g.
template <int POW_REF, bool DE>
__device__ __forceinline__ q64::Q term64(const MapParams& m, const q64::Q& q, int i, double sign,
                                         q64::Q& g) {
  using namespace q64;
  Q d;
  d.w = sub(q.w, m.r64[i][0]);
  d.x = sub(q.x, m.r64[i][1]);
  d.y = sub(q.y, m.r64[i][2]);
  d.z = sub(q.z, m.r64[i][3]);
  if (DE) {
    // no reference counterpart: gradient of log|R| for the distance estimate
    const double k = sign * m.e64[i] / norm2(d);
    g.w += k * d.w;
    g.x += k * d.x;
    g.y += k * d.y;
    g.z += k * d.z;
  }
  return POW_REF == 2 ? qpow_cr(d, m.e64[i]) : POW_REF ? qpow(d, m.e64[i]) : qpow_int(d, m.ie[i]);
}

template <int POW_REF, bool DE>
__device__ __forceinline__ q64::Q product64(const MapParams& m, const q64::Q& q, int lo, int hi,
                                            double sign, q64::Q& g) {
  using namespace q64;
  Q r = {1.0, 0.0, 0.0, 0.0};
#pragma unroll 1
  for (int i = lo; i < hi; i++) {
    const Q t = term64<POW_REF, DE>(m, q, i, sign, g);
    r = (i == lo) ? t : qmul(r, t);
  }
  return r;
}

// RATIONAL_4D::evaluateLagrange (RATIONAL_4D.cpp:27-73): from 1, times top
// term k then divided by bottom term k for the common k, then the longer
// side's leftovers; without bottom roots the plain factored top.
template <int POW_REF, bool DE>
__device__ __forceinline__ q64::Q lagrange64(const MapParams& m, const q64::Q& q, q64::Q& g) {
  using namespace q64;
  if (m.nb == 0) return product64<POW_REF, DE>(m, q, 0, m.nt, 1.0, g);
  Q r = {1.0, 0.0, 0.0, 0.0};
  const int same = m.nt < m.nb ? m.nt : m.nb;
#pragma unroll 1
  for (int k = 0; k < same; k++) {
    r = qmul(r, term64<POW_REF, DE>(m, q, k, 1.0, g));
    r = qdiv(r, term64<POW_REF, DE>(m, q, m.nt + k, -1.0, g));
  }
#pragma unroll 1
  for (int k = same; k < m.nt; k++) r = qmul(r, term64<POW_REF, DE>(m, q, k, 1.0, g));
#pragma unroll 1
  for (int k = same; k < m.nb; k++) r = qdiv(r, term64<POW_REF, DE>(m, q, m.nt + k, -1.0, g));
  return r;
}

// One application of the map in reference order (OPTIMIZE_3D.cpp:1331-1350),
// plus |grad log|R|| for the distance estimate when DE is set.
// With `lagrange`, the map in the Lagrange order (TRIANGLE_MESH.cpp:281-322).
template <int POW_REF, bool DE>
__device__ __forceinline__ q64::Q apply64(const MapParams& m, const q64::Q& q, double* gnorm,
                                          bool lagrange = false) {
  using namespace q64;
  Q g = {0.0, 0.0, 0.0, 0.0};
  Q out;
  if (lagrange) {
    out = lagrange64<POW_REF, DE>(m, q, g);
  } else {
    const Q top = product64<POW_REF, DE>(m, q, 0, m.nt, 1.0, g);
    out = top;
    if (m.nb > 0) {
      const Q bot = product64<POW_REF, DE>(m, q, m.nt, m.nt + m.nb, -1.0, g);
      out = qdiv(top, bot);
    }
  }
  out.w = mul(out.w, m.scale);
  out.x = mul(out.x, m.scale);
  out.y = mul(out.y, m.scale);
  out.z = mul(out.z, m.scale);
  if (DE) *gnorm = __dsqrt_rn(norm2(g));
  return out;
}

// The escape loop for one start point; returns log|q_N| and the executed
// iteration count; *de = |q_N| log|q_N| / |q_N'| when DE.
template <int POW_REF, bool DE>
__device__ __forceinline__ double escape64(const MapParams& m, const IterParams& it,
                                           const double p[3], double slice, int* iters,
                                           double* de) {
  using namespace q64;
  Q q = {p[0], p[1], p[2], slice};  // QUATERNION(x, y, z, slice): w = x
  double mg = mag(q);
  int n = 0, executed = 0;
  double dn = 1.0;
  const double tiny = 10.0 * 0x1p-126;  // 10 * FLT_MIN (SETTINGS.h:60)
  while (mg < it.escape && n < it.max_it) {
    double gn = 0.0;
    q = apply64<POW_REF, DE>(m, q, &gn, it.lagrange != 0);
    mg = mag(q);
    if (DE) dn = (dn * gn) * mg;
    n++;
    executed++;
    if (mg < tiny) n = it.max_it;  // the "black hole" exit, OPTIMIZE_3D.cpp:1358-1359
  }
  const double f = POW_REF == 2 ? crm_log(mg) : log(mg);
  *iters = executed;
  if (DE) *de = mg * f / dn;
  return f;
}

// TRIANGLE_MESH::lagrangeNonlinearValue (TRIANGLE_MESH.cpp:1684-1747): the
// Lagrange escape loop minus iso, where an overflowing iterate reverts to
// the previous one and stops, and an infinite value becomes FLT_MAX.  (The
// reference leaves the previous magnitude unset when the first application
// overflows; here it is |q_0|.)
template <int POW_REF>
__device__ __forceinline__ double lagrange_value64(const MapParams& m, const IterParams& it,
                                                   const double p[3], double slice, double iso) {
  using namespace q64;
  Q q = {p[0], p[1], p[2], slice};
  double mg = mag(q), prev_mg = mg;
  Q prev = q;
  int n = 0;
  const double tiny = 10.0 * 0x1p-126;
  while (mg < it.escape && n < it.max_it) {
    double gn;
    q = apply64<POW_REF, false>(m, q, &gn, true);
    mg = mag(q);
    if (isinf(mg)) {
      q = prev;
      mg = prev_mg;
      break;
    }
    prev = q;
    prev_mg = mg;
    n++;
    if (mg < tiny) n = it.max_it;
  }
  const double f = sub(POW_REF == 2 ? crm_log(mg) : log(mg), iso);
  return isinf(f) ? 3.40282346638528859812e+38 : f;
}

// ------------------------------------------------------- FP32 map

// Exponents other than 1 and 2 (kept out of line, off the hot path).
static __device__ __noinline__ q32::Q root_power_rare(q32::Q d, int ie, float e) {
  return ie > 0 ? q32::qpow_int(d, ie) : q32::qpow(d, e);
}

// One root term (q - r_i)^(e_i) in FP32; with DE, adds (+-e_i) d/|d|^2 to g.
// Root coordinates come as one 16-byte constant-bank load and {+-e, integer
// exponent} as one 8-byte load.
template <bool DE>
__device__ __forceinline__ q32::Q root_term32(const MapParams& m, const q32::Q& q, int i,
                                              q32::Q& g) {
  using namespace q32;
  const float4 root = *reinterpret_cast<const float4*>(m.r32[i]);
  const float2 ex = *reinterpret_cast<const float2*>(m.x32[i]);
  const Q d = {q.w - root.x, q.x - root.y, q.y - root.z, q.z - root.w};
  if (DE) {
    const float k = ex.x * rcp_approx(norm2(d));
    g.w = fmaf(k, d.w, g.w);
    g.x = fmaf(k, d.x, g.x);
    g.y = fmaf(k, d.y, g.y);
    g.z = fmaf(k, d.z, g.z);
  }
  const int ie = __float_as_int(ex.y);
  if (ie == 1) return d;
  if (ie == 2) return qsq(d);
  return root_power_rare(d, ie, m.e32[i]);
}

// prod_{i in [lo, hi)} (q - r_i)^(e_i) in left-to-right order; the first
// term starts the product and the rest go two per trip as r * (t0 * t1):
// the same algebra as (r * t0) * t1, with t0 * t1 off the serial chain
// through r, which halves the dependent-latency path of the loop.
template <bool DE>
__device__ __forceinline__ q32::Q product32(const MapParams& m, const q32::Q& q, int lo, int hi,
                                            q32::Q& g) {
  using namespace q32;
  Q r = root_term32<DE>(m, q, lo, g);
  int i = lo + 1;
#pragma unroll 1
  for (; i + 1 < hi; i += 2) {
    const Q t0 = root_term32<DE>(m, q, i, g);
    const Q t1 = root_term32<DE>(m, q, i + 1, g);
    r = qmul(r, qmul(t0, t1));
  }
  if (i < hi) r = qmul(r, root_term32<DE>(m, q, i, g));
  return r;
}

// RATIONAL_4D::evaluateLagrange's order in FP32 (RATIONAL_4D.cpp:27-73):
// times top term k, then divided by bottom term k (r conj(b) / |b|^2) for
// the common k, then the longer side's leftovers; with bottom roots only.
template <bool DE>
__device__ __forceinline__ q32::Q lagrange32(const MapParams& m, const q32::Q& q, q32::Q& g) {
  using namespace q32;
  const int same = m.nt < m.nb ? m.nt : m.nb;
  auto divide = [&](const Q& r, int i) {
    const Q b = root_term32<DE>(m, q, i, g);
    const float inv = rcp_approx(norm2(b));
    Q o = qmul_conj(r, b);
    o.w *= inv;
    o.x *= inv;
    o.y *= inv;
    o.z *= inv;
    return o;
  };
  Q r = root_term32<DE>(m, q, 0, g);
  r = divide(r, m.nt);
#pragma unroll 1
  for (int k = 1; k < same; k++) r = divide(qmul(r, root_term32<DE>(m, q, k, g)), m.nt + k);
#pragma unroll 1
  for (int k = same; k < m.nt; k++) r = qmul(r, root_term32<DE>(m, q, k, g));
#pragma unroll 1
  for (int k = same; k < m.nb; k++) r = divide(r, m.nt + k);
  return r;
}

template <bool DE>
__device__ __forceinline__ q32::Q apply32(const MapParams& m, const q32::Q& q, float* g2) {
  using namespace q32;
  Q g = {0.f, 0.f, 0.f, 0.f};
  if (m.lagrange && m.nb > 0) {
    Q out = lagrange32<DE>(m, q, g);
    out.w *= m.scalef;
    out.x *= m.scalef;
    out.y *= m.scalef;
    out.z *= m.scalef;
    if (DE) *g2 = norm2(g);
    return out;
  }
  const Q top = product32<DE>(m, q, 0, m.nt, g);
  Q out;
  if (m.nb > 0) {
    const Q bot = product32<DE>(m, q, m.nt, m.nt + m.nb, g);
    const float inv = m.scalef * rcp_approx(norm2(bot));
    out = qmul_conj(top, bot);
    out.w *= inv;
    out.x *= inv;
    out.y *= inv;
    out.z *= inv;
  } else {
    out = top;
    out.w *= m.scalef;
    out.x *= m.scalef;
    out.y *= m.scalef;
    out.z *= m.scalef;
  }
  if (DE) *g2 = norm2(g);
  return out;
}

// root_term32 / product32 / apply32 on a voxel pair.
template <bool DE>
__device__ __forceinline__ q32x2::Q2 root_term32x2(const MapParams& m, const q32x2::Q2& q, int i,
                                                   q32x2::Q2& g) {
  using namespace q32x2;
  const float4 rwx = *reinterpret_cast<const float4*>(&m.rn2[i][0]);
  const float4 ryz = *reinterpret_cast<const float4*>(&m.rn2[i][2]);
  const Q2 d = {add2(q.w, make_float2(rwx.x, rwx.y)), add2(q.x, make_float2(rwx.z, rwx.w)),
                add2(q.y, make_float2(ryz.x, ryz.y)), add2(q.z, make_float2(ryz.z, ryz.w))};
  if (DE) {
    const float2 n = norm2(d);
    const float2 k = mul2(m.ex2[i], make_float2(q32::rcp_approx(n.x), q32::rcp_approx(n.y)));
    g.w = fma2(k, d.w, g.w);
    g.x = fma2(k, d.x, g.x);
    g.y = fma2(k, d.y, g.y);
    g.z = fma2(k, d.z, g.z);
  }
  const int ie = m.ie[i];
  if (ie == 1) return d;
  if (ie == 2) return qsq(d);
  return join(root_power_rare(lo(d), ie, m.e32[i]), root_power_rare(hi(d), ie, m.e32[i]));
}

template <bool DE>
__device__ __forceinline__ q32x2::Q2 product32x2(const MapParams& m, const q32x2::Q2& q, int lo,
                                                 int hi, q32x2::Q2& g) {
  using namespace q32x2;
  Q2 r = root_term32x2<DE>(m, q, lo, g);
  int i = lo + 1;
#pragma unroll 1
  for (; i + 1 < hi; i += 2) {
    const Q2 t0 = root_term32x2<DE>(m, q, i, g);
    const Q2 t1 = root_term32x2<DE>(m, q, i + 1, g);
    r = qmul(r, qmul(t0, t1));
  }
  if (i < hi) r = qmul(r, root_term32x2<DE>(m, q, i, g));
  return r;
}

// product32x2 over a compile-time count N of roots from index LO: the same
// association, unrolled (fully up to 24 roots), so every root's constants sit
// at a fixed offset of the parameter bank.
template <bool DE, int LO, int N>
__device__ __forceinline__ q32x2::Q2 product32x2_fixed(const MapParams& m, const q32x2::Q2& q,
                                                       q32x2::Q2& g) {
  using namespace q32x2;
  Q2 r = root_term32x2<DE>(m, q, LO, g);
  if (N <= 24) {
#pragma unroll
    for (int k = 1; k + 1 < N; k += 2) {
      const Q2 t0 = root_term32x2<DE>(m, q, LO + k, g);
      const Q2 t1 = root_term32x2<DE>(m, q, LO + k + 1, g);
      r = qmul(r, qmul(t0, t1));
    }
  } else {
    // long maps: two pairs per trip (fully unrolled 48 / 24 roots overflow
    // the instruction cache; 2 per trip measured best of 1 to 8)
#pragma unroll 2
    for (int k = 1; k + 1 < N; k += 2) {
      const Q2 t0 = root_term32x2<DE>(m, q, LO + k, g);
      const Q2 t1 = root_term32x2<DE>(m, q, LO + k + 1, g);
      r = qmul(r, qmul(t0, t1));
    }
  }
  if (N % 2 == 0) r = qmul(r, root_term32x2<DE>(m, q, LO + N - 1, g));
  return r;
}

// lagrange32 on a voxel pair
template <bool DE>
__device__ __forceinline__ q32x2::Q2 lagrange32x2(const MapParams& m, const q32x2::Q2& q,
                                                  q32x2::Q2& g) {
  using namespace q32x2;
  const int same = m.nt < m.nb ? m.nt : m.nb;
  auto divide = [&](const Q2& r, int i) {
    const Q2 b = root_term32x2<DE>(m, q, i, g);
    const float2 n = norm2(b);
    const float2 inv = make_float2(q32::rcp_approx(n.x), q32::rcp_approx(n.y));
    Q2 o = qmul_conj(r, b);
    o.w = mul2(o.w, inv);
    o.x = mul2(o.x, inv);
    o.y = mul2(o.y, inv);
    o.z = mul2(o.z, inv);
    return o;
  };
  Q2 r = root_term32x2<DE>(m, q, 0, g);
  r = divide(r, m.nt);
#pragma unroll 1
  for (int k = 1; k < same; k++) r = divide(qmul(r, root_term32x2<DE>(m, q, k, g)), m.nt + k);
#pragma unroll 1
  for (int k = same; k < m.nt; k++) r = qmul(r, root_term32x2<DE>(m, q, k, g));
#pragma unroll 1
  for (int k = same; k < m.nb; k++) r = divide(r, m.nt + k);
  return r;
}

// NT, NB > 0: the root counts are compile-time constants (they must equal
// m.nt and m.nb; the quotient order only); 0: read from m.
template <bool DE, int NT = 0, int NB = 0>
__device__ __forceinline__ q32x2::Q2 apply32x2(const MapParams& m, const q32x2::Q2& q,
                                               float2* g2) {
  using namespace q32x2;
  Q2 g = {pair(0.f), pair(0.f), pair(0.f), pair(0.f)};
  if (NT == 0 && m.lagrange && m.nb > 0) {
    Q2 out = lagrange32x2<DE>(m, q, g);
    const float2 s = pair(m.scalef);
    out.w = mul2(out.w, s);
    out.x = mul2(out.x, s);
    out.y = mul2(out.y, s);
    out.z = mul2(out.z, s);
    if (DE) *g2 = norm2(g);
    return out;
  }
  const Q2 top = NT > 0 ? product32x2_fixed<DE, 0, (NT > 0 ? NT : 1)>(m, q, g)
                        : product32x2<DE>(m, q, 0, m.nt, g);
  Q2 out;
  if (NT > 0 ? NB > 0 : m.nb > 0) {
    const Q2 bot = NT > 0 ? product32x2_fixed<DE, (NT > 0 ? NT : 0), (NB > 0 ? NB : 1)>(m, q, g)
                          : product32x2<DE>(m, q, m.nt, m.nt + m.nb, g);
    const float2 n = norm2(bot);
    const float2 inv =
        mul2(pair(m.scalef), make_float2(q32::rcp_approx(n.x), q32::rcp_approx(n.y)));
    out = qmul_conj(top, bot);
    out.w = mul2(out.w, inv);
    out.x = mul2(out.x, inv);
    out.y = mul2(out.y, inv);
    out.z = mul2(out.z, inv);
  } else {
    const float2 s = pair(m.scalef);
    out.w = mul2(top.w, s);
    out.x = mul2(top.x, s);
    out.y = mul2(top.y, s);
    out.z = mul2(top.z, s);
  }
  if (DE) *g2 = norm2(g);
  return out;
}

// The FP32 escape loop at an arbitrary point: returns log|q_N| and, through
// *err, the first-order estimate of its FP32 error (the relative error of
// q_N carried by q32::propagate_err).  *err is infinite when FP32 cannot
// follow the orbit (|q| below 1e-18, overflow) or an iterate lies within its
// error of the escape radius.
__device__ __forceinline__ float escape32(const MapParams& m, const IterParams& it,
                                          const double p[3], double slice, float* err) {
  using namespace q32;
  Q q = {(float)p[0], (float)p[1], (float)p[2], (float)slice};
  const float esc2 = (float)(it.escape * it.escape);
  float m2 = norm2(q), e = q32::EPS32;
  int n = 0;
  bool bad = false, near = false;
  while (m2 < esc2 && n < it.max_it) {
    float gg = 0.f;
    q = apply32<true>(m, q, &gg);
    near = near || q32::near_radius(m2, esc2, e);
    e = q32::propagate_err(e, gg, m2);
    m2 = norm2(q);
    n++;
    if (m2 < 1e-36f) {
      bad = true;
      break;
    }
  }
  // an iterate within FP32 error of the escape radius may stop the FP64
  // orbit at another iterate: no bound holds across that step (the last
  // iterate of an orbit cut by max_it is the same iterate either way)
  bad = bad || near || (m2 >= esc2 && n < it.max_it && q32::near_radius(m2, esc2, e));
  const float f = 0.5f * logf(m2);
  *err = (bad || !isfinite(f) || !(e < 1.f)) ? __int_as_float(0x7f800000) : e;
  return f;
}

}  // namespace qj

