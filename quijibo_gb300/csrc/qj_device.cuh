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

// ------------------------------------------------------- FP64 escape loop

// prod_{i in [lo, hi)} (q - r_i)^(e_i), left to right, as
// POLYNOMIAL_4D::evaluateScaledPowerFactored (POLYNOMIAL_4D.cpp:912-923);
// with DE, adds sign * sum e_i (q - r_i) / |q - r_i|^2 to g.
template <bool POW_REF, bool DE>
__device__ __forceinline__ q64::Q product64(const MapParams& m, const q64::Q& q, int lo, int hi,
                                            double sign, q64::Q& g) {
  using namespace q64;
  Q r = {1.0, 0.0, 0.0, 0.0};
#pragma unroll 1
  for (int i = lo; i < hi; i++) {
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
    const Q t = POW_REF ? qpow(d, m.e64[i]) : qpow_int(d, m.ie[i]);
    r = (i == lo) ? t : qmul(r, t);
  }
  return r;
}

// One application of the map in reference order (OPTIMIZE_3D.cpp:1331-1350),
// plus |grad log|R|| for the distance estimate when DE is set.
template <bool POW_REF, bool DE>
__device__ __forceinline__ q64::Q apply64(const MapParams& m, const q64::Q& q, double* gnorm) {
  using namespace q64;
  Q g = {0.0, 0.0, 0.0, 0.0};
  const Q top = product64<POW_REF, DE>(m, q, 0, m.nt, 1.0, g);
  Q out = top;
  if (m.nb > 0) {
    const Q bot = product64<POW_REF, DE>(m, q, m.nt, m.nt + m.nb, -1.0, g);
    out = qdiv(top, bot);
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
template <bool POW_REF, bool DE>
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
    q = apply64<POW_REF, DE>(m, q, &gn);
    mg = mag(q);
    if (DE) dn = (dn * gn) * mg;
    n++;
    executed++;
    if (mg < tiny) n = it.max_it;  // the "black hole" exit, OPTIMIZE_3D.cpp:1358-1359
  }
  const double f = log(mg);
  *iters = executed;
  if (DE) *de = mg * f / dn;
  return f;
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
    const float k = __fdividef(ex.x, norm2(d));
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

// prod_{i in [lo, hi)} (q - r_i)^(e_i), left to right; the first term starts
// the product and the rest go two per trip.
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
    r = qmul(qmul(r, t0), t1);
  }
  if (i < hi) r = qmul(r, root_term32<DE>(m, q, i, g));
  return r;
}

template <bool DE>
__device__ __forceinline__ q32::Q apply32(const MapParams& m, const q32::Q& q, float* g2) {
  using namespace q32;
  Q g = {0.f, 0.f, 0.f, 0.f};
  const Q top = product32<DE>(m, q, 0, m.nt, g);
  Q out;
  if (m.nb > 0) {
    const Q bot = product32<DE>(m, q, m.nt, m.nt + m.nb, g);
    const float inv = __fdividef(m.scalef, norm2(bot));
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

// The FP32 escape loop at an arbitrary point with the distance estimate:
// returns log|q_N| and, through *err, a conservative bound on its FP32
// error: 64 * 2^-24 * (|q_0| + 1) * |q_N'| / |q_N|, the first-order growth
// of a relative perturbation of the start point through the orbit (64 covers
// the rounding of every root term and iteration).  *err is infinite when
// FP32 cannot follow the orbit (|q| below 1e-18, overflow).
__device__ __forceinline__ float escape32(const MapParams& m, const IterParams& it,
                                          const double p[3], double slice, float* err) {
  using namespace q32;
  Q q = {(float)p[0], (float)p[1], (float)p[2], (float)slice};
  const float q0 = sqrtf(norm2(q));
  const float esc2 = (float)(it.escape * it.escape);
  float m2 = norm2(q), l2d = 0.f;
  int n = 0;
  bool bad = false;
  while (m2 < esc2 && n < it.max_it) {
    float gg = 0.f;
    q = apply32<true>(m, q, &gg);
    m2 = norm2(q);
    l2d += 0.5f * (__log2f(gg) + __log2f(m2));
    n++;
    if (m2 < 1e-36f) {
      bad = true;
      break;
    }
  }
  const float f = 0.5f * logf(m2);
  const float e = 64.f * 5.9604645e-8f * (q0 + 1.f) * exp2f(l2d - 0.5f * __log2f(m2));
  *err = (bad || !isfinite(f) || isnan(e)) ? __int_as_float(0x7f800000) : e;
  return f;
}

}  // namespace qj

