// Correctly rounded FP64 exp, log, sin, cos and acos for the plain FP64
// form's QUATERNION::pow (src/algebra/QUATERNION.cpp:375-393 calls acos,
// log, exp, sin and cos once each per root term).
//
// Method (written for this library from the mathematics; no vendor or libm
// code): each function reduces its argument exactly or in double-double
// (Cody-Waite reduction with the constant split so the leading products are
// exact), looks up a table value at a nearby point (Tang's table-driven
// method: 2^(j/64), -log of 256 reciprocals, sin/cos(j/64), atan(j/64)), and
// evaluates a short Taylor series of the remainder, the terms above 2^-53 in
// double-double (Dekker/Knuth error-free sums and FMA products) and the rest
// in double.  The double-double result carries a relative error below about
// 2^-100, so its leading double is the correctly rounded value unless the
// exact value lies within 2^-100 (relative) of a rounding midpoint -- for
// random arguments a chance of about 2^-47 per call; no fallback is taken
// for those.  Not correctly rounded: subnormal exp results (rounded twice)
// and sin/cos of |x| >= 2^20 (the platform's sin/cos).
//
// The same source compiles as C (the CPU oracle, with -ffp-contract=off) and
// as CUDA device code (every operation an explicit round-to-nearest
// intrinsic), so both give the same bits.  Tables: qj_crmath_tables.h,
// written by gen_crmath_tables.py.
#pragma once

#ifdef __CUDACC__
#define CRM_FN static __device__ __forceinline__
#define CRM_API static __device__ __noinline__  // called, not inlined: keeps kernels small
#define CRM_TAB static __device__ const
#define CRM_ADD(a, b) __dadd_rn((a), (b))
#define CRM_SUB(a, b) __dsub_rn((a), (b))
#define CRM_MUL(a, b) __dmul_rn((a), (b))
#define CRM_DIV(a, b) __ddiv_rn((a), (b))
#define CRM_SQRT(a) __dsqrt_rn(a)
#define CRM_FMA(a, b, c) __fma_rn((a), (b), (c))
#define CRM_ABS(a) fabs(a)
#define CRM_PLATFORM_SIN(a) sin(a)
#define CRM_PLATFORM_COS(a) cos(a)
#else
#include <math.h>
#include <stdint.h>
#include <string.h>
#define CRM_FN static inline
#define CRM_API static inline
#define CRM_TAB static const
#define CRM_ADD(a, b) ((a) + (b))
#define CRM_SUB(a, b) ((a) - (b))
#define CRM_MUL(a, b) ((a) * (b))
#define CRM_DIV(a, b) ((a) / (b))
#define CRM_SQRT(a) sqrt(a)
#define CRM_FMA(a, b, c) fma((a), (b), (c))
#define CRM_ABS(a) fabs(a)
#define CRM_PLATFORM_SIN(a) sin(a)
#define CRM_PLATFORM_COS(a) cos(a)
#endif

typedef struct {
  double hi, lo;
} crm_dd;

#include "qj_crmath_tables.h"

CRM_FN unsigned long long crm_bits(double x) {
#ifdef __CUDACC__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}

CRM_FN double crm_from_bits(unsigned long long b) {
#ifdef __CUDACC__
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}

CRM_FN crm_dd crm_make(double hi, double lo) {
  crm_dd r;
  r.hi = hi;
  r.lo = lo;
  return r;
}

// ---------------------------------------------------------- double-double
// a + b = s + e exactly (Knuth)
CRM_FN crm_dd crm_two_sum(double a, double b) {
  const double s = CRM_ADD(a, b);
  const double bb = CRM_SUB(s, a);
  const double e = CRM_ADD(CRM_SUB(a, CRM_SUB(s, bb)), CRM_SUB(b, bb));
  return crm_make(s, e);
}

// a + b = s + e exactly when |a| >= |b| or a == 0 (Dekker)
CRM_FN crm_dd crm_fast_two_sum(double a, double b) {
  const double s = CRM_ADD(a, b);
  return crm_make(s, CRM_SUB(b, CRM_SUB(s, a)));
}

// a * b = p + e exactly
CRM_FN crm_dd crm_two_prod(double a, double b) {
  const double p = CRM_MUL(a, b);
  return crm_make(p, CRM_FMA(a, b, -p));
}

CRM_FN crm_dd crm_dd_add(crm_dd x, crm_dd y) {
  crm_dd s = crm_two_sum(x.hi, y.hi);
  const crm_dd t = crm_two_sum(x.lo, y.lo);
  s = crm_fast_two_sum(s.hi, CRM_ADD(s.lo, t.hi));
  return crm_fast_two_sum(s.hi, CRM_ADD(s.lo, t.lo));
}

CRM_FN crm_dd crm_dd_neg(crm_dd x) { return crm_make(-x.hi, -x.lo); }

CRM_FN crm_dd crm_dd_sub(crm_dd x, crm_dd y) { return crm_dd_add(x, crm_dd_neg(y)); }

CRM_FN crm_dd crm_dd_add_d(crm_dd x, double y) {
  const crm_dd s = crm_two_sum(x.hi, y);
  return crm_fast_two_sum(s.hi, CRM_ADD(s.lo, x.lo));
}

CRM_FN crm_dd crm_dd_mul(crm_dd x, crm_dd y) {
  const crm_dd p = crm_two_prod(x.hi, y.hi);
  const double e = CRM_FMA(x.hi, y.lo, CRM_MUL(x.lo, y.hi));
  return crm_fast_two_sum(p.hi, CRM_ADD(p.lo, e));
}

CRM_FN crm_dd crm_dd_mul_d(crm_dd x, double y) {
  const crm_dd p = crm_two_prod(x.hi, y);
  return crm_fast_two_sum(p.hi, CRM_FMA(x.lo, y, p.lo));
}

// x * y + c, the Horner step
CRM_FN crm_dd crm_dd_mad(crm_dd x, crm_dd y, crm_dd c) { return crm_dd_add(crm_dd_mul(x, y), c); }

CRM_FN crm_dd crm_dd_div(crm_dd a, crm_dd b) {
  const double q1 = CRM_DIV(a.hi, b.hi);
  crm_dd r = crm_dd_sub(a, crm_dd_mul_d(b, q1));
  const double q2 = CRM_DIV(r.hi, b.hi);
  r = crm_dd_sub(r, crm_dd_mul_d(b, q2));
  const double q3 = CRM_DIV(r.hi, b.hi);
  return crm_dd_add_d(crm_fast_two_sum(q1, q2), q3);
}

// sqrt of a > 0: one Newton correction of the correctly rounded sqrt(a.hi)
CRM_FN crm_dd crm_dd_sqrt(crm_dd a) {
  const double s = CRM_SQRT(a.hi);
  const crm_dd p = crm_two_prod(s, s);
  const double r = CRM_ADD(CRM_SUB(CRM_SUB(a.hi, p.hi), p.lo), a.lo);  // a.hi - p.hi is exact
  return crm_fast_two_sum(s, CRM_DIV(r, CRM_ADD(s, s)));
}

// x rounded to the nearest integer, ties to even (|x| < 2^51)
CRM_FN double crm_rint(double x) { return CRM_SUB(CRM_ADD(x, 0x1.8p52), 0x1.8p52); }

// h * 2^m with one rounding (h a normal double near 1)
CRM_FN double crm_scale(double h, int m) {
  if (m > 1023) return CRM_MUL(CRM_MUL(h, 0x1p1023), crm_from_bits((unsigned long long)m << 52));
  if (m < -1022)
    return CRM_MUL(CRM_MUL(h, crm_from_bits((unsigned long long)(m + 600 + 1023) << 52)), 0x1p-600);
  return CRM_MUL(h, crm_from_bits((unsigned long long)(m + 1023) << 52));
}

// --------------------------------------------------------------------- exp
CRM_API double crm_exp(double x) {
  if (!(x == x)) return CRM_ADD(x, x);
  if (x > 709.79) return CRM_MUL(x, 0x1p1023);  // overflows to +inf
  if (x < -745.2) return 0.0;
  // x = k ln2/64 + r, |r| <= ln2/128 (+ rounding)
  const double kd = crm_rint(CRM_MUL(x, CRM_INV_LN2_64));
  const long long k = (long long)kd;
  const int j = (int)(k & 63);
  const int m = (int)((k - j) / 64);
  const double r1 = CRM_SUB(x, CRM_MUL(kd, CRM_LN2_64_1));  // exact (Sterbenz)
  crm_dd t = crm_two_prod(kd, CRM_LN2_64_2);
  t.lo = CRM_FMA(kd, CRM_LN2_64_3, t.lo);
  const crm_dd r = crm_dd_sub(crm_make(r1, 0.0), t);
  // exp(r) = sum r^n / n!, n <= 11: n >= 6 in double, the rest in double-double
  double q = crm_inv_fact[11].hi;
  for (int n = 10; n >= 6; n--) q = CRM_FMA(q, r.hi, crm_inv_fact[n].hi);
  crm_dd acc = crm_make(q, 0.0);
  for (int n = 5; n >= 0; n--) acc = crm_dd_mad(acc, r, crm_inv_fact[n]);
  const crm_dd res = crm_dd_mul(crm_exp2_64[j], acc);
  return crm_scale(res.hi, m);
}

// --------------------------------------------------------------------- log
CRM_API double crm_log(double x) {
  if (!(x > 0.0)) {
    if (x == 0.0) return crm_from_bits(0xfff0000000000000ull);  // -inf
    return crm_from_bits(0xfff8000000000000ull);        // NaN (x < 0 or NaN)
  }
  unsigned long long b = crm_bits(x);
  if ((b >> 52) == 0x7ff) return x;  // +inf
  int e = (int)(b >> 52) - 1023;
  if (e == -1023) {  // subnormal
    b = crm_bits(CRM_MUL(x, 0x1p54));
    e = (int)(b >> 52) - 1023 - 54;
  }
  const unsigned long long mant = b & 0xfffffffffffffull;
  const int half = mant >= 0x6a09e667f3bcdull;  // y >= sqrt(2): use y / 2
  const double y = crm_from_bits(mant | ((unsigned long long)(1023 - half) << 52));
  e += half;
  const int idx = (int)(mant >> 45) + 128 * half;
  const double inv = crm_log_inv[idx];
  // t = y * inv - 1, exact as a double-double (p.hi - 1 is exact: p.hi is near 1)
  const crm_dd p = crm_two_prod(y, inv);
  const crm_dd t = crm_two_sum(CRM_SUB(p.hi, 1.0), p.lo);
  // log1p(t) = sum (-1)^(n+1) t^n / n, |t| < 2^-7, n <= 16: n >= 8 in double
  double q = crm_inv_n[16].hi * -1.0;
  for (int n = 15; n >= 8; n--) q = CRM_FMA(q, t.hi, (n & 1) ? crm_inv_n[n].hi : -crm_inv_n[n].hi);
  crm_dd acc = crm_make(q, 0.0);
  for (int n = 7; n >= 1; n--)
    acc = crm_dd_mad(acc, t, (n & 1) ? crm_inv_n[n] : crm_dd_neg(crm_inv_n[n]));
  acc = crm_dd_mul(acc, t);
  crm_dd res = crm_dd_add(crm_log_neg[idx], acc);
  if (e != 0) {
    const double ed = (double)e;
    crm_dd el = crm_two_prod(ed, CRM_LN2_HI);
    el = crm_fast_two_sum(el.hi, CRM_FMA(ed, CRM_LN2_LO, el.lo));
    res = crm_dd_add(el, res);
  }
  return res.hi;
}

// ----------------------------------------------------------------- sin, cos
// sin(x) and cos(x) of one argument (one reduction)
CRM_API void crm_sincos(double x, double* sp, double* cp) {
  if (!(CRM_SUB(x, x) == 0.0)) {  // inf or NaN
    *sp = *cp = CRM_SUB(x, x);
    return;
  }
  const double ax = CRM_ABS(x);
  if (ax < 0x1p-27) {
    *sp = x;
    *cp = 1.0;
    return;
  }
  if (ax >= 0x1p20) {
    *sp = CRM_PLATFORM_SIN(x);
    *cp = CRM_PLATFORM_COS(x);
    return;
  }
  // ax = k pi/2 + r, pi/2 = P1 + P2 + P3 + P4 (k*P1, k*P2 exact)
  const double kd = crm_rint(CRM_MUL(ax, CRM_2_PI));
  const int quad = (int)((long long)kd & 3);
  const double a1 = CRM_SUB(ax, CRM_MUL(kd, CRM_PIO2_1));  // exact (Sterbenz)
  crm_dd r = crm_two_sum(a1, -CRM_MUL(kd, CRM_PIO2_2));
  r = crm_dd_sub(r, crm_two_prod(kd, CRM_PIO2_3));
  r = crm_dd_add_d(r, -CRM_MUL(kd, CRM_PIO2_4));
  const int neg = r.hi < 0.0;
  if (neg) r = crm_dd_neg(r);
  // r = j/64 + d, |d| <= 1/128
  const int j = (int)CRM_ADD(CRM_MUL(r.hi, 64.0), 0.5);
  const double c0 = CRM_MUL((double)j, 0x1p-6);
  const crm_dd d = crm_fast_two_sum(CRM_SUB(r.hi, c0), r.lo);  // r.hi - c0 exact
  const crm_dd u = crm_dd_mul(d, d);
  // sin d = d (1 - u/3! + u^2/5! - ...), cos d = 1 - u/2! + u^2/4! - ...
  double qs = CRM_FMA(u.hi, crm_inv_fact[13].hi, -crm_inv_fact[11].hi);
  qs = CRM_FMA(qs, u.hi, crm_inv_fact[9].hi);
  qs = CRM_FMA(qs, u.hi, -crm_inv_fact[7].hi);
  crm_dd sd = crm_make(qs, 0.0);
  sd = crm_dd_mad(sd, u, crm_inv_fact[5]);
  sd = crm_dd_mad(sd, u, crm_dd_neg(crm_inv_fact[3]));
  sd = crm_dd_mad(sd, u, crm_inv_fact[1]);
  sd = crm_dd_mul(sd, d);
  double qc = CRM_FMA(u.hi, crm_inv_fact[12].hi, -crm_inv_fact[10].hi);
  qc = CRM_FMA(qc, u.hi, crm_inv_fact[8].hi);
  crm_dd cd = crm_make(qc, 0.0);
  cd = crm_dd_mad(cd, u, crm_dd_neg(crm_inv_fact[6]));
  cd = crm_dd_mad(cd, u, crm_inv_fact[4]);
  cd = crm_dd_mad(cd, u, crm_dd_neg(crm_inv_fact[2]));
  cd = crm_dd_mad(cd, u, crm_inv_fact[0]);
  const crm_dd S = crm_sin_64[j], C = crm_cos_64[j];
  crm_dd sr = crm_dd_add(crm_dd_mul(S, cd), crm_dd_mul(C, sd));
  const crm_dd cr = crm_dd_sub(crm_dd_mul(C, cd), crm_dd_mul(S, sd));
  if (neg) sr = crm_dd_neg(sr);
  double s, c;
  switch (quad) {
    case 0: s = sr.hi; c = cr.hi; break;
    case 1: s = cr.hi; c = -sr.hi; break;
    case 2: s = -sr.hi; c = -cr.hi; break;
    default: s = -cr.hi; c = sr.hi; break;
  }
  *sp = x < 0.0 ? -s : s;
  *cp = c;
}

CRM_FN double crm_sin(double x) {
  double s, c;
  crm_sincos(x, &s, &c);
  return s;
}

CRM_FN double crm_cos(double x) {
  double s, c;
  crm_sincos(x, &s, &c);
  return c;
}

// -------------------------------------------------------------------- acos
// atan(s) for 0 <= s <= 1: atan(j/64) + atan(w), w = (s - c)/(1 + s c)
CRM_FN crm_dd crm_atan01(crm_dd s) {
  const int j = (int)CRM_ADD(CRM_MUL(s.hi, 64.0), 0.5);
  crm_dd w = s;
  if (j > 0) {
    const double c = CRM_MUL((double)j, 0x1p-6);
    const crm_dd num = crm_fast_two_sum(CRM_SUB(s.hi, c), s.lo);  // s.hi - c exact
    const crm_dd den = crm_dd_add_d(crm_dd_mul_d(s, c), 1.0);
    w = crm_dd_div(num, den);
  }
  // atan w = w (1 - v/3 + v^2/5 - ...), v = w^2, |w| <= 2^-7: 1/9 .. 1/15 in double
  const crm_dd v = crm_dd_mul(w, w);
  double q = CRM_FMA(v.hi, -crm_inv_n[15].hi, crm_inv_n[13].hi);
  q = CRM_FMA(q, v.hi, -crm_inv_n[11].hi);
  q = CRM_FMA(q, v.hi, crm_inv_n[9].hi);
  crm_dd acc = crm_make(q, 0.0);
  acc = crm_dd_mad(acc, v, crm_dd_neg(crm_inv_n[7]));
  acc = crm_dd_mad(acc, v, crm_inv_n[5]);
  acc = crm_dd_mad(acc, v, crm_dd_neg(crm_inv_n[3]));
  acc = crm_dd_mad(acc, v, crm_inv_n[1]);
  acc = crm_dd_mul(acc, w);
  return j > 0 ? crm_dd_add(crm_atan_64[j], acc) : acc;
}

// acos|x| = 2 atan(sqrt((1-|x|)/(1+|x|))); acos(-a) = pi - acos(a)
CRM_API double crm_acos(double x) {
  const double ax = CRM_ABS(x);
  if (!(ax <= 1.0)) return crm_from_bits(0x7ff8000000000000ull);  // NaN
  if (x == 1.0) return 0.0;
  if (x == -1.0) return CRM_PI_HI;
  const crm_dd u = crm_dd_div(crm_two_sum(1.0, -ax), crm_two_sum(1.0, ax));
  crm_dd a = crm_atan01(crm_dd_sqrt(u));
  a = crm_make(CRM_MUL(a.hi, 2.0), CRM_MUL(a.lo, 2.0));
  if (x >= 0.0) return a.hi;
  return crm_dd_sub(crm_make(CRM_PI_HI, CRM_PI_LO), a).hi;
}
