// Double-float ("float-float") arithmetic: a value is an unevaluated sum
// hi + lo of two FP32 numbers with |lo| <= ulp(hi)/2, about 44 significant
// bits.  Built from the error-free transformations of Knuth (TwoSum) and
// Dekker (FastTwoSum, and TwoProduct through a fused multiply-add), as in
// the double-double literature (Hida, Li & Bailey 2001), here on FP32 words.
// On sm_103a the FP64 pipe runs at 1/64 of the FP32 rate, so a double-float
// Hamilton product (~170 FP32 operations) costs about a sixth of an FP64 one.
//
// Used for the first iterations of voxels whose FP32 orbit is too
// ill-conditioned for the requested relative error: rounding errors of the
// early iterations are amplified the most, so a double-float head followed by
// FP32 removes most of the error at a fraction of the FP64 cost.
#pragma once
#include <cuda_runtime.h>

#include "qj_device.cuh"

namespace qj {
namespace qff {

struct F {
  float hi, lo;
};

// s + e = a + b exactly (Knuth TwoSum, 6 operations, no ordering needed)
__device__ __forceinline__ F two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return F{s, e};
}

// s + e = a + b exactly when |a| >= |b| (Dekker FastTwoSum)
__device__ __forceinline__ F fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return F{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// p + e = a * b exactly (the FMA gives the low part)
__device__ __forceinline__ F two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return F{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ F from_double(double v) {
  const float hi = __double2float_rn(v);
  return F{hi, __double2float_rn(v - (double)hi)};
}

__device__ __forceinline__ F neg(F a) { return F{-a.hi, -a.lo}; }

__device__ __forceinline__ F add(F a, F b) {
  const F s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ F mul(F a, F b) {
  const F p = two_prod(a.hi, b.hi);
  return fast_two_sum(p.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo)));
}

__device__ __forceinline__ F mul(F a, float b) {
  const F p = two_prod(a.hi, b);
  return fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}

// a0*b0 + a1*b1 + a2*b2 + a3*b3: four exact products, the high parts summed
// with TwoSum, every low part and rounding error gathered in one FP32 sum
__device__ __forceinline__ F dot4(F a0, F b0, F a1, F b1, F a2, F b2, F a3, F b3) {
  const F p0 = two_prod(a0.hi, b0.hi), p1 = two_prod(a1.hi, b1.hi);
  const F p2 = two_prod(a2.hi, b2.hi), p3 = two_prod(a3.hi, b3.hi);
  float e = __fmaf_rn(a0.hi, b0.lo, __fmaf_rn(a0.lo, b0.hi, p0.lo));
  e = __fadd_rn(e, __fmaf_rn(a1.hi, b1.lo, __fmaf_rn(a1.lo, b1.hi, p1.lo)));
  e = __fadd_rn(e, __fmaf_rn(a2.hi, b2.lo, __fmaf_rn(a2.lo, b2.hi, p2.lo)));
  e = __fadd_rn(e, __fmaf_rn(a3.hi, b3.lo, __fmaf_rn(a3.lo, b3.hi, p3.lo)));
  F s = two_sum(p0.hi, p1.hi);
  e = __fadd_rn(e, s.lo);
  s = two_sum(s.hi, p2.hi);
  e = __fadd_rn(e, s.lo);
  s = two_sum(s.hi, p3.hi);
  e = __fadd_rn(e, s.lo);
  return fast_two_sum(s.hi, e);
}

struct Q {
  F w, x, y, z;
};

__device__ __forceinline__ Q qmul(const Q& a, const Q& b) {
  Q o;
  o.w = dot4(a.w, b.w, a.x, neg(b.x), a.y, neg(b.y), a.z, neg(b.z));
  o.x = dot4(a.w, b.x, a.x, b.w, a.y, b.z, a.z, neg(b.y));
  o.y = dot4(a.w, b.y, a.x, neg(b.z), a.y, b.w, a.z, b.x);
  o.z = dot4(a.w, b.z, a.x, b.y, a.y, neg(b.x), a.z, b.w);
  return o;
}

// a * conj(b)
__device__ __forceinline__ Q qmul_conj(const Q& a, const Q& b) {
  Q o;
  o.w = dot4(a.w, b.w, a.x, b.x, a.y, b.y, a.z, b.z);
  o.x = dot4(a.w, neg(b.x), a.x, b.w, a.y, neg(b.z), a.z, b.y);
  o.y = dot4(a.w, neg(b.y), a.x, b.z, a.y, b.w, a.z, neg(b.x));
  o.z = dot4(a.w, neg(b.z), a.x, neg(b.y), a.y, b.x, a.z, b.w);
  return o;
}

__device__ __forceinline__ Q qsq(const Q& a) {
  Q o;
  o.w = dot4(a.w, a.w, a.x, neg(a.x), a.y, neg(a.y), a.z, neg(a.z));
  const F w2 = F{2.f * a.w.hi, 2.f * a.w.lo};  // exact
  o.x = mul(w2, a.x);
  o.y = mul(w2, a.y);
  o.z = mul(w2, a.z);
  return o;
}

__device__ __forceinline__ F norm2(const Q& q) {
  return dot4(q.w, q.w, q.x, q.x, q.y, q.y, q.z, q.z);
}

__device__ __forceinline__ q32::Q hi(const Q& q) { return q32::Q{q.w.hi, q.x.hi, q.y.hi, q.z.hi}; }

// 1 / a: the FP32 reciprocal refined by one Newton step in double-float
__device__ __forceinline__ F recip(F a) {
  const float r = q32::rcp_approx(a.hi);
  // r + r * (1 - a * r)
  const F ar = mul(a, r);
  const F resid = add(F{1.f, 0.f}, neg(ar));
  return add(F{r, 0.f}, mul(resid, r));
}

// Integer power 1..QJ_MAX_INT_EXP by square-and-multiply.
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

// The cell centre (x, y, z) of g as double-float, from the affine
// coefficients of GridParams: within ~2^-44 of the exact centre, like a
// double rounded to a pair, without FP64 instructions.
__device__ __forceinline__ Q cell_center_ff(const GridParams& g, int x, int y, int z) {
  const float idx[3] = {(float)x, (float)y, (float)z};  // exact (< 2^24)
  F p[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    F s = {g.ffa[c][0], g.ffa[c][1]};
#pragma unroll
    for (int k = 0; k < 3; k++) s = add(s, mul(F{g.ffb[c][k][0], g.ffb[c][k][1]}, idx[k]));
    p[c] = s;
  }
  return Q{p[0], p[1], p[2], F{g.ffslice[0], g.ffslice[1]}};
}

// The FP32 start point of the bulk kernels: the cell centre rounded to FP32
// from its double-float value (the FP32 rounding of the exact centre, as a
// double centre rounded to FP32 gives but for ties within 2^-44)
__device__ __forceinline__ q32::Q cell_center_f32(const GridParams& g, int x, int y, int z) {
  return hi(cell_center_ff(g, x, y, z));
}

}  // namespace qff

// Relative rounding of double-float arithmetic (sloppy add: ~2^-44 under
// cancellation) and its per-application step, scaled as the FP32 model's
// (q32::ERR_STEP = 64 ulp).
constexpr float EPS_FF = 5.684342e-14f;  // 2^-44
constexpr float ERR_STEP_FF = 64.f * EPS_FF;

// One root term (q - r_i)^(e_i) in double-float (integer exponents only);
// with DE, adds (+-e_i) d/|d|^2 to g from the high parts, as the FP32 form.
template <bool DE>
__device__ __forceinline__ qff::Q root_term_ff(const MapParams& m, const qff::Q& q, int i,
                                               q32::Q& g) {
  using namespace qff;
  const Q d = {add(q.w, neg(F{m.rff[i][0][0], m.rff[i][0][1]})),
               add(q.x, neg(F{m.rff[i][1][0], m.rff[i][1][1]})),
               add(q.y, neg(F{m.rff[i][2][0], m.rff[i][2][1]})),
               add(q.z, neg(F{m.rff[i][3][0], m.rff[i][3][1]}))};
  if (DE) {
    const q32::Q dh = hi(d);
    const float k = m.x32[i][0] * q32::rcp_approx(q32::norm2(dh));
    g.w = fmaf(k, dh.w, g.w);
    g.x = fmaf(k, dh.x, g.x);
    g.y = fmaf(k, dh.y, g.y);
    g.z = fmaf(k, dh.z, g.z);
  }
  return qpow_int(d, m.ie[i]);
}

template <bool DE>
__device__ __forceinline__ qff::Q product_ff(const MapParams& m, const qff::Q& q, int lo, int hi,
                                             q32::Q& g) {
  qff::Q r = root_term_ff<DE>(m, q, lo, g);
#pragma unroll 1
  for (int i = lo + 1; i < hi; i++) r = qff::qmul(r, root_term_ff<DE>(m, q, i, g));
  return r;
}

// The Lagrange order (lagrange32) in double-float.
template <bool DE>
__device__ __forceinline__ qff::Q lagrange_ff(const MapParams& m, const qff::Q& q, q32::Q& g) {
  using namespace qff;
  const int same = m.nt < m.nb ? m.nt : m.nb;
  auto divide = [&](const Q& r, int i) {
    const Q b = root_term_ff<DE>(m, q, i, g);
    const F inv = recip(norm2(b));
    Q o = qmul_conj(r, b);
    o.w = mul(o.w, inv);
    o.x = mul(o.x, inv);
    o.y = mul(o.y, inv);
    o.z = mul(o.z, inv);
    return o;
  };
  Q r = root_term_ff<DE>(m, q, 0, g);
  r = divide(r, m.nt);
#pragma unroll 1
  for (int k = 1; k < same; k++) r = divide(qmul(r, root_term_ff<DE>(m, q, k, g)), m.nt + k);
#pragma unroll 1
  for (int k = same; k < m.nt; k++) r = qmul(r, root_term_ff<DE>(m, q, k, g));
#pragma unroll 1
  for (int k = same; k < m.nb; k++) r = divide(r, m.nt + k);
  return r;
}

// One map application in double-float; *g2 = |grad log|R||^2 in FP32.
// Requires m.all_int (integer effective exponents).
template <bool DE>
__device__ __forceinline__ qff::Q apply_ff(const MapParams& m, const qff::Q& q, float* g2) {
  using namespace qff;
  q32::Q g = {0.f, 0.f, 0.f, 0.f};
  if (m.lagrange && m.nb > 0) {
    Q out = lagrange_ff<DE>(m, q, g);
    const F s = {m.scale_ff[0], m.scale_ff[1]};
    out.w = mul(out.w, s);
    out.x = mul(out.x, s);
    out.y = mul(out.y, s);
    out.z = mul(out.z, s);
    if (DE) *g2 = q32::norm2(g);
    return out;
  }
  const Q top = product_ff<DE>(m, q, 0, m.nt, g);
  Q out;
  if (m.nb > 0) {
    const Q bot = product_ff<DE>(m, q, m.nt, m.nt + m.nb, g);
    const F inv = mul(recip(norm2(bot)), F{m.scale_ff[0], m.scale_ff[1]});
    out = qmul_conj(top, bot);
    out.w = mul(out.w, inv);
    out.x = mul(out.x, inv);
    out.y = mul(out.y, inv);
    out.z = mul(out.z, inv);
  } else {
    const F s = {m.scale_ff[0], m.scale_ff[1]};
    out.w = mul(top.w, s);
    out.x = mul(top.x, s);
    out.y = mul(top.y, s);
    out.z = mul(top.z, s);
  }
  if (DE) *g2 = q32::norm2(g);
  return out;
}

// The escape loop in double-float at an arbitrary point (integer exponents):
// returns log|q_N| and, through *err, a first-order bound on its absolute
// error, propagated as the FP32 model's (relative error of q_n scaled by
// |grad log|R|| |q_n| and ERR_STEP_FF added per application).  *err is
// infinite where no bound holds: an iterate within its error of the escape
// radius (FP64 may stop at another iterate), |q| near the bottom of the FP32
// exponent range the pairs live in, or a non-finite value.
__device__ __forceinline__ double escape_ff(const MapParams& m, const IterParams& it,
                                            const double p[3], double slice, float* err) {
  using namespace qff;
  Q q = {from_double(p[0]), from_double(p[1]), from_double(p[2]), from_double(slice)};
  const double esc2 = it.escape * it.escape;
  auto m2_of = [](const Q& v) {
    const F n = norm2(v);
    return (double)n.hi + (double)n.lo;
  };
  double m2 = m2_of(q);
  float e = EPS_FF;
  int n = 0;
  bool bad = false, near = false;
  // the escape test compares |q|^2 with esc^2 in FP64 here and |q| with esc
  // in the reference: a relative margin of 1e-14 covers the difference
  auto near_esc = [&](double v) {
    return fabs(v - esc2) < 2.0 * fmax((double)e, 1e-14) * esc2;
  };
  while (m2 < esc2 && n < it.max_it) {
    float gg = 0.f;
    q = apply_ff<true>(m, q, &gg);
    near = near || near_esc(m2);
    e = q32::propagate_err_step(e, gg, (float)m2, ERR_STEP_FF);
    m2 = m2_of(q);
    n++;
    if (m2 < 1e-28) {
      bad = true;
      break;
    }
  }
  bad = bad || near || (m2 >= esc2 && n < it.max_it && near_esc(m2));
  const double f = 0.5 * log(m2);
  *err = (bad || !isfinite(f) || !(e < 1e-3f)) ? __int_as_float(0x7f800000) : e;
  return f;
}

// ---- two voxels per lane -------------------------------------------------
// The same double-float arithmetic on packed f32x2 operands (voxel a in .x,
// voxel b in .y).  Every packed operation rounds each half as its scalar
// form does, so each voxel gets the bits of the one-voxel code.
namespace qff2 {

using q32x2::add2;
using q32x2::fma2;
using q32x2::mul2;
using q32x2::neg2;
using q32x2::pair;

struct F2 {
  float2 hi, lo;
};

__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return add2(a, neg2(b)); }

__device__ __forceinline__ F2 two_sum(float2 a, float2 b) {
  const float2 s = add2(a, b);
  const float2 bb = sub2(s, a);
  const float2 e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
  return F2{s, e};
}

__device__ __forceinline__ F2 fast_two_sum(float2 a, float2 b) {
  const float2 s = add2(a, b);
  return F2{s, sub2(b, sub2(s, a))};
}

__device__ __forceinline__ F2 two_prod(float2 a, float2 b) {
  const float2 p = mul2(a, b);
  return F2{p, fma2(a, b, neg2(p))};
}

__device__ __forceinline__ F2 neg(F2 a) { return F2{neg2(a.hi), neg2(a.lo)}; }

__device__ __forceinline__ F2 add(F2 a, F2 b) {
  const F2 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, add2(s.lo, add2(a.lo, b.lo)));
}

__device__ __forceinline__ F2 mul(F2 a, F2 b) {
  const F2 p = two_prod(a.hi, b.hi);
  return fast_two_sum(p.hi, fma2(a.hi, b.lo, fma2(a.lo, b.hi, p.lo)));
}

__device__ __forceinline__ F2 mul(F2 a, float2 b) {
  const F2 p = two_prod(a.hi, b);
  return fast_two_sum(p.hi, fma2(a.lo, b, p.lo));
}

__device__ __forceinline__ F2 dot4(F2 a0, F2 b0, F2 a1, F2 b1, F2 a2, F2 b2, F2 a3, F2 b3) {
  const F2 p0 = two_prod(a0.hi, b0.hi), p1 = two_prod(a1.hi, b1.hi);
  const F2 p2 = two_prod(a2.hi, b2.hi), p3 = two_prod(a3.hi, b3.hi);
  float2 e = fma2(a0.hi, b0.lo, fma2(a0.lo, b0.hi, p0.lo));
  e = add2(e, fma2(a1.hi, b1.lo, fma2(a1.lo, b1.hi, p1.lo)));
  e = add2(e, fma2(a2.hi, b2.lo, fma2(a2.lo, b2.hi, p2.lo)));
  e = add2(e, fma2(a3.hi, b3.lo, fma2(a3.lo, b3.hi, p3.lo)));
  F2 t = two_sum(p0.hi, p1.hi);
  e = add2(e, t.lo);
  t = two_sum(t.hi, p2.hi);
  e = add2(e, t.lo);
  t = two_sum(t.hi, p3.hi);
  e = add2(e, t.lo);
  return fast_two_sum(t.hi, e);
}

struct Q {
  F2 w, x, y, z;
};

__device__ __forceinline__ Q qmul(const Q& a, const Q& b) {
  Q o;
  o.w = dot4(a.w, b.w, a.x, neg(b.x), a.y, neg(b.y), a.z, neg(b.z));
  o.x = dot4(a.w, b.x, a.x, b.w, a.y, b.z, a.z, neg(b.y));
  o.y = dot4(a.w, b.y, a.x, neg(b.z), a.y, b.w, a.z, b.x);
  o.z = dot4(a.w, b.z, a.x, b.y, a.y, neg(b.x), a.z, b.w);
  return o;
}

__device__ __forceinline__ Q qmul_conj(const Q& a, const Q& b) {
  Q o;
  o.w = dot4(a.w, b.w, a.x, b.x, a.y, b.y, a.z, b.z);
  o.x = dot4(a.w, neg(b.x), a.x, b.w, a.y, neg(b.z), a.z, b.y);
  o.y = dot4(a.w, neg(b.y), a.x, b.z, a.y, b.w, a.z, neg(b.x));
  o.z = dot4(a.w, neg(b.z), a.x, neg(b.y), a.y, b.x, a.z, b.w);
  return o;
}

__device__ __forceinline__ Q qsq(const Q& a) {
  Q o;
  o.w = dot4(a.w, a.w, a.x, neg(a.x), a.y, neg(a.y), a.z, neg(a.z));
  const F2 w2 = F2{mul2(pair(2.f), a.w.hi), mul2(pair(2.f), a.w.lo)};  // exact
  o.x = mul(w2, a.x);
  o.y = mul(w2, a.y);
  o.z = mul(w2, a.z);
  return o;
}

__device__ __forceinline__ F2 norm2(const Q& q) {
  return dot4(q.w, q.w, q.x, q.x, q.y, q.y, q.z, q.z);
}

__device__ __forceinline__ q32x2::Q2 hi(const Q& q) {
  return q32x2::Q2{q.w.hi, q.x.hi, q.y.hi, q.z.hi};
}

__device__ __forceinline__ float2 rcp2(float2 x) {
  return make_float2(q32::rcp_approx(x.x), q32::rcp_approx(x.y));
}

__device__ __forceinline__ F2 recip(F2 a) {
  const float2 r = rcp2(a.hi);
  const F2 ar = mul(a, r);
  const F2 resid = add(F2{pair(1.f), pair(0.f)}, neg(ar));
  return add(F2{r, pair(0.f)}, mul(resid, r));
}

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

__device__ __forceinline__ F2 join(const qff::F& a, const qff::F& b) {
  return F2{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)};
}

__device__ __forceinline__ Q join(const qff::Q& a, const qff::Q& b) {
  return Q{join(a.w, b.w), join(a.x, b.x), join(a.y, b.y), join(a.z, b.z)};
}

}  // namespace qff2

// root_term_ff for two voxels
template <bool DE>
__device__ __forceinline__ qff2::Q root_term_ff2(const MapParams& m, const qff2::Q& q, int i,
                                                 q32x2::Q2& g) {
  using namespace qff2;
  auto rootc = [&](int c) {
    return F2{pair(m.rff[i][c][0]), pair(m.rff[i][c][1])};
  };
  const Q d = {add(q.w, neg(rootc(0))), add(q.x, neg(rootc(1))), add(q.y, neg(rootc(2))),
               add(q.z, neg(rootc(3)))};
  if (DE) {
    const q32x2::Q2 dh = hi(d);
    const float2 k = mul2(pair(m.x32[i][0]), rcp2(q32x2::norm2(dh)));
    g.w = fma2(k, dh.w, g.w);
    g.x = fma2(k, dh.x, g.x);
    g.y = fma2(k, dh.y, g.y);
    g.z = fma2(k, dh.z, g.z);
  }
  return qpow_int(d, m.ie[i]);
}

template <bool DE>
__device__ __forceinline__ qff2::Q product_ff2(const MapParams& m, const qff2::Q& q, int lo,
                                               int hi, q32x2::Q2& g) {
  qff2::Q r = root_term_ff2<DE>(m, q, lo, g);
#pragma unroll 1
  for (int i = lo + 1; i < hi; i++) r = qff2::qmul(r, root_term_ff2<DE>(m, q, i, g));
  return r;
}

// lagrange_ff for two voxels
template <bool DE>
__device__ __forceinline__ qff2::Q lagrange_ff2(const MapParams& m, const qff2::Q& q,
                                                q32x2::Q2& g) {
  using namespace qff2;
  const int same = m.nt < m.nb ? m.nt : m.nb;
  auto divide = [&](const Q& r, int i) {
    const Q b = root_term_ff2<DE>(m, q, i, g);
    const F2 inv = recip(norm2(b));
    Q o = qmul_conj(r, b);
    o.w = mul(o.w, inv);
    o.x = mul(o.x, inv);
    o.y = mul(o.y, inv);
    o.z = mul(o.z, inv);
    return o;
  };
  Q r = root_term_ff2<DE>(m, q, 0, g);
  r = divide(r, m.nt);
#pragma unroll 1
  for (int k = 1; k < same; k++) r = divide(qmul(r, root_term_ff2<DE>(m, q, k, g)), m.nt + k);
#pragma unroll 1
  for (int k = same; k < m.nt; k++) r = qmul(r, root_term_ff2<DE>(m, q, k, g));
#pragma unroll 1
  for (int k = same; k < m.nb; k++) r = divide(r, m.nt + k);
  return r;
}

// apply_ff for two voxels; *g2 = each one's |grad log|R||^2 in FP32
template <bool DE>
__device__ __forceinline__ qff2::Q apply_ff2(const MapParams& m, const qff2::Q& q, float2* g2) {
  using namespace qff2;
  q32x2::Q2 g = {pair(0.f), pair(0.f), pair(0.f), pair(0.f)};
  const F2 s = {pair(m.scale_ff[0]), pair(m.scale_ff[1])};
  if (m.lagrange && m.nb > 0) {
    Q out = lagrange_ff2<DE>(m, q, g);
    out.w = mul(out.w, s);
    out.x = mul(out.x, s);
    out.y = mul(out.y, s);
    out.z = mul(out.z, s);
    if (DE) *g2 = q32x2::norm2(g);
    return out;
  }
  const Q top = product_ff2<DE>(m, q, 0, m.nt, g);
  Q out;
  if (m.nb > 0) {
    const Q bot = product_ff2<DE>(m, q, m.nt, m.nt + m.nb, g);
    const F2 inv = mul(recip(norm2(bot)), s);
    out = qmul_conj(top, bot);
    out.w = mul(out.w, inv);
    out.x = mul(out.x, inv);
    out.y = mul(out.y, inv);
    out.z = mul(out.z, inv);
  } else {
    out.w = mul(top.w, s);
    out.x = mul(top.x, s);
    out.y = mul(top.y, s);
    out.z = mul(top.z, s);
  }
  if (DE) *g2 = q32x2::norm2(g);
  return out;
}

}  // namespace qj
