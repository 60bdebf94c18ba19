// Fitting energies and their gradients.
//
// tanh_grad_kernel: the reference's tanh-weighted score and its analytic
// one-application gradients in one pass per voxel, FP64 in reference
// operation order:
//   score  = sum -tanh(alpha F) w                 weightScore, OPTIMIZE_3D.cpp:4502-4517
//   F      = the adaptive-precision map           computeRationalMapAP, :1374-1567
//            (voxels whose FP64 map overflows: recomputed in extended range,
//            field, score and gradients, where the reference uses long double)
//   g[0]   = d/d log s                            computeExpGradientAP, :3589-3625
//   g[1+j] = d/d bottom exponent j                computeBottomGradientAP, :10012-10116
//   g[1+nb+i] = d/d top exponent i                computeTopGradientAP, :8905-9006
//   g[1+nb+nt], g[2+nb+nt] = d/d sigma_t, sigma_b compute{Top,Bottom}BulkScalarGradientAP
// (layout of toothOptimizer's FormScaledFunctionGradient,
// projects/toothOptimizer/toothOptimizer.cpp:65-109).  The reference runs
// one full-grid pass per parameter; here one voxel's thread produces every
// parameter's term from the last iteration's factors, kept in local memory.
// Sums are deterministic: warp shuffle trees, warps in order, blocks in
// order with compensated (Neumaier) summation.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <vector>
#include <type_traits>

#include "qj_device.cuh"
#include "qj_energy.h"

namespace qj {

namespace {

using namespace q64;

constexpr int EN_T = 128;  // threads per block

// QUATERNION::log, QUATERNION.cpp:352-365.
__device__ __forceinline__ Q qlog(const Q& q) {
  const double qm = mag(q);
  const double vm = __dsqrt_rn(add(add(mul(q.x, q.x), mul(q.y, q.y)), mul(q.z, q.z)));
  double vx = 0, vy = 0, vz = 0;
  if (vm > 0) {
    vx = __ddiv_rn(q.x, vm);
    vy = __ddiv_rn(q.y, vm);
    vz = __ddiv_rn(q.z, vm);
  }
  const double a = acos(__ddiv_rn(q.w, qm));
  return Q{log(qm), mul(vx, a), mul(vy, a), mul(vz, a)};
}

// QUATERNION::inverse, QUATERNION.cpp:167-172 (conjugate / |q|^2).
__device__ __forceinline__ Q qinv(const Q& q) {
  const double inv = __ddiv_rn(1.0, norm2(q));
  return Q{mul(q.w, inv), mul(-q.x, inv), mul(-q.y, inv), mul(-q.z, inv)};
}

// QUATERNION::dot, QUATERNION.h
__device__ __forceinline__ double qdot(const Q& a, const Q& b) {
  return add(add(add(mul(a.w, b.w), mul(a.x, b.x)), mul(a.y, b.y)), mul(a.z, b.z));
}

__device__ __forceinline__ Q qscale(const Q& q, double k) {
  return Q{mul(q.w, k), mul(q.x, k), mul(q.y, k), mul(q.z, k)};
}

// Per-warp accumulation of one slot (lane values summed by a shuffle tree).
__device__ __forceinline__ void warp_accum(double* acc, int slot, double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) acc[slot] += v;
}

// ---- extended range -------------------------------------------------------
// Voxels whose FP64 map overflows are recomputed by the reference in long
// double (computeRationalMapAP's second pass, OPTIMIZE_3D.cpp:1490-1567, and
// the "overflow pass" of every gradient, e.g. :9007-9106).  Here a quaternion
// is a mantissa m (largest component in [0.5, 1)) times 2^e: the same
// formulas, with the range of the exponent instead of more mantissa bits.
struct QX {
  Q m;
  int e;
};

constexpr double LN2 = 0.6931471805599453;

__device__ __forceinline__ QX xnorm(const Q& m, int e) {
  const double a = fmax(fmax(fabs(m.w), fabs(m.x)), fmax(fabs(m.y), fabs(m.z)));
  if (!(a > 0.0) || isinf(a)) return QX{m, e};
  int k;
  frexp(a, &k);
  return QX{Q{ldexp(m.w, -k), ldexp(m.x, -k), ldexp(m.y, -k), ldexp(m.z, -k)}, e + k};
}

__device__ __forceinline__ QX xof(const Q& q) { return xnorm(q, 0); }

__device__ __forceinline__ QX xmul(const QX& a, const QX& b) {
  return xnorm(qmul(a.m, b.m), a.e + b.e);
}

// l * (conj(r) / |r|^2), as operator/(q,q)
__device__ __forceinline__ QX xdiv(const QX& l, const QX& r) {
  const double inv = __ddiv_rn(1.0, norm2(r.m));
  const QX ri = xnorm(Q{mul(r.m.w, inv), mul(-r.m.x, inv), mul(-r.m.y, inv), mul(-r.m.z, inv)},
                      -r.e);
  return xmul(l, ri);
}

// times a finite scalar of any size
__device__ __forceinline__ QX xscale(const QX& a, double k) {
  int ke = 0;
  const double km = frexp(k, &ke);
  return xnorm(qscale(a.m, km), a.e + ke);
}

__device__ __forceinline__ double xlogmag(const QX& a) {
  return add(log(mag(a.m)), mul((double)a.e, LN2));
}

// (a . b) / (a . a), both scaled
__device__ __forceinline__ double xdot_ratio(const QX& a, const QX& b) {
  return ldexp(__ddiv_rn(qdot(a.m, b.m), qdot(a.m, a.m)), b.e - a.e);
}

// QUATERNION::pow (QUATERNION.cpp:375-393) with |q|^e = 2^k 2^f
__device__ __forceinline__ QX xpow(const Q& q, double e) {
  const double partial = add(add(mul(q.x, q.x), mul(q.y, q.y)), mul(q.z, q.z));
  const double qm = __dsqrt_rn(add(partial, mul(q.w, q.w)));
  if (!(qm > 0.0)) {
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    return QX{Q{nan, nan, nan, nan}, 0};
  }
  const double vm = __dsqrt_rn(partial);
  const double vminv = (vm > 0.0) ? __ddiv_rn(1.0, vm) : 0.0;
  const double scale = mul(mul(e, acos(__ddiv_rn(q.w, qm))), vminv);
  const double mm = mul(scale, vm);
  const double minv = (mm > 0.0) ? __ddiv_rn(1.0, mm) : 0.0;
  const double l2 = mul(e, log2(qm));
  const double k = floor(l2);
  const double em = exp2(sub(l2, k));
  double s, c;
  sincos(mm, &s, &c);
  const double scale2 = mul(mul(mul(scale, em), minv), s);
  return xnorm(Q{mul(em, c), mul(scale2, q.x), mul(scale2, q.y), mul(scale2, q.z)}, (int)k);
}

__device__ __forceinline__ QX xpow_int(const Q& d, int n) {
  const QX b = xof(d);
  QX r = b;
  for (int k = 1; k < n; k++) r = xmul(r, b);
  return r;
}

// The map iterated in extended range from q0 (an FP64 overflow detected):
// returns log|q_N| (0 where it is still not a number, as the reference's
// stillNans); the last application's factors go to (Pf, Pe) and its top and
// bottom products to *T, *B.
template <bool POW_REF>
__device__ __noinline__ double ext_map(const MapParams& m, const Q q0, int max_it, Q* Pf, int* Pe,
                                       QX* Tout, QX* Bout) {
  const int nt = m.nt, nb = m.nb;
  Q q = q0;
  double mg = mag(q0), logm = log(mg);
  QX T = {Q{1, 0, 0, 0}, 0}, B = T;
  int it = 0;
  while (mg < 20.0 && it < max_it) {
#pragma unroll 1
    for (int side = 0; side < 2; side++) {
      const int lo = side ? nt : 0, hi = side ? nt + nb : nt;
      QX acc = {Q{1, 0, 0, 0}, 0};
#pragma unroll 1
      for (int i = lo; i < hi; i++) {
        const Q d{sub(q.w, m.r64[i][0]), sub(q.x, m.r64[i][1]), sub(q.y, m.r64[i][2]),
                  sub(q.z, m.r64[i][3])};
        const QX f = POW_REF ? xpow(d, m.e64[i]) : xpow_int(d, m.ie[i]);
        Pf[i] = f.m;
        Pe[i] = f.e;
        acc = (i == lo) ? f : xmul(acc, f);
      }
      if (side == 0)
        T = acc;
      else if (nb > 0)
        B = acc;
    }
    const QX R = xscale(nb > 0 ? xdiv(T, B) : T, m.scale);
    logm = xlogmag(R);
    mg = exp(logm);
    if (mg < 20.0) q = Q{ldexp(R.m.w, R.e), ldexp(R.m.x, R.e), ldexp(R.m.y, R.e), ldexp(R.m.z, R.e)};
    it++;
  }
  *Tout = T;
  *Bout = B;
  return isnan(logm) ? 0.0 : logm;
}

// Exponent of a finite positive double (its bits), -1023 for zero and
// denormals, 1024 for infinities and not-a-number.
__device__ __forceinline__ int ilog2_bits(double v) {
  return (int)((__double_as_longlong(v) >> 52) & 0x7ff) - 1023;
}

// One voxel's map (computeRationalMapAP's first pass, OPTIMIZE_3D.cpp:1408-1488):
// the last application's factors Pf and the suffix products Sf the reference
// caches with them, T and B, the overflow flag as FE_OVERFLOW would raise it.
// With BOUNDS, also what decides whether a voxel's gradient terms can be
// skipped as exact zeros: the spread of the factors' magnitudes and whether
// every q0 - root is of moderate size and away from 1.
struct Voxel {
  Q q0, T, B;
  double mg;
  int its;
  bool over, iterated;
  int spread;      // sum over factors of |log2 |factor|^2|
  bool bases_ok;
};

template <bool POW_REF, bool BOUNDS>
__device__ __forceinline__ void eval_voxel(const MapParams& m, const Q& q0, int max_it, Q* Pf,
                                           Q* Sf, Voxel& v) {
  const int nt = m.nt, nb = m.nb;
  v.q0 = q0;
  v.T = Q{1, 0, 0, 0};
  v.B = Q{1, 0, 0, 0};
  v.its = 0;
  v.over = false;
  v.iterated = false;
  v.spread = 0;
  v.bases_ok = true;
  Q q = q0;
  double mg = mag(q);
  if (!(mg < 1e-8)) {  // "if we hit the origin, move on"
    while (mg < 20.0 && v.its < max_it) {  // computeRationalMapAP's escape radius 20
      v.iterated = true;
      if (BOUNDS) {
        v.spread = 0;
        v.bases_ok = true;
      }
#pragma unroll 1
      for (int side = 0; side < 2; side++) {
        const int lo = side ? nt : 0, hi = side ? nt + nb : nt;
        Q acc_q = {1, 0, 0, 0};
#pragma unroll 1
        for (int i = lo; i < hi; i++) {
          const Q d{sub(q.w, m.r64[i][0]), sub(q.x, m.r64[i][1]), sub(q.y, m.r64[i][2]),
                    sub(q.z, m.r64[i][3])};
          Pf[i] = POW_REF ? qpow(d, m.e64[i]) : qpow_int(d, m.ie[i]);
          acc_q = (i == lo) ? Pf[i] : qmul(acc_q, Pf[i]);
          if (BOUNDS) {
            v.spread += abs(ilog2_bits(norm2(Pf[i])));
            const double b2 = norm2(d);
            const Q d1{sub(d.w, 1.0), d.x, d.y, d.z};
            v.bases_ok = v.bases_ok && b2 > 1e-40 && b2 < 1e40 && norm2(d1) > 1e-20;
          }
        }
        if (side == 0)
          v.T = acc_q;
        else if (nb > 0)
          v.B = acc_q;
      }
      // the suffix products evaluateScaledPowerFactored caches in the same
      // evaluation (POLYNOMIAL_4D.cpp:1066-1072); an overflow there flags
      // the voxel like one in the forward product (a non-finite
      // intermediate leaves the full suffix product non-finite)
      bool suffix_ok = true;
#pragma unroll 1
      for (int side = 0; side < 2; side++) {
        const int lo = side ? nt : 0, hi = side ? nt + nb : nt;
        if (hi == lo) continue;
        Sf[hi - 1] = Pf[hi - 1];
#pragma unroll 1
        for (int i = hi - 2; i >= lo; i--) Sf[i] = qmul(Pf[i], Sf[i + 1]);
        suffix_ok = suffix_ok && isfinite(Sf[lo].w) && isfinite(Sf[lo].x) &&
                    isfinite(Sf[lo].y) && isfinite(Sf[lo].z);
      }
      const Q& T = v.T;
      const Q& B = v.B;
      q = nb > 0 ? qdiv(T, B) : T;
      // what raises FE_OVERFLOW in the reference: a non-finite factor
      // product, |B|^2 beyond range inside the division, or the quotient
      v.over = v.over || !suffix_ok || !isfinite(T.w) || !isfinite(T.x) || !isfinite(T.y) ||
               !isfinite(T.z) ||
               (nb > 0 && (!isfinite(B.w) || !isfinite(B.x) || !isfinite(B.y) ||
                           !isfinite(B.z) || isinf(norm2(B)))) ||
               !isfinite(q.w) || !isfinite(q.x) || !isfinite(q.y) || !isfinite(q.z);
      q = qscale(q, m.scale);
      mg = mag(q);
      if (isinf(mg) || isnan(mg)) v.over = true;
      v.its++;
    }
  }
  v.mg = mg;
}

// R = T / B and dS/dF of a voxel whose map did not overflow; false when R is
// zero or infinite (the reference skips such voxels in every gradient).
__device__ __forceinline__ bool grad_setup(const Voxel& v, double logs, double alpha, double thr,
                                           double w, Q& R, double& dSdF, double& RR) {
  R = qdiv(v.T, v.B);
  const double Rm = mag(R);
  if (Rm <= 0.0 || isinf(Rm)) return false;
  const double F = add(log(Rm), logs);
  const double th = tanh(mul(alpha, sub(F, thr)));
  dSdF = mul(mul(-alpha, w), sub(1.0, mul(th, th)));
  RR = __ddiv_rn(1.0, qdot(R, R));
  return true;
}

// The per-parameter gradient terms of one voxel (FP64 path) and their warp
// sums; every lane of the warp calls it (inactive lanes with ok = false).
template <bool POW_REF>
__device__ __forceinline__ void grad_terms(const MapParams& m, const Voxel& v, bool ok,
                                           const Q& R, double dSdF, double RR, const Q* Pf,
                                           const Q* Sf, double* acc, int s_bad) {
  const int nt = m.nt, nb = m.nb;
  const Q& q0 = v.q0;
  const Q& T = v.T;
  const Q& B = v.B;
  // one application from q0: the map's factor is the gradient's power, bit for bit
  const bool reuse = POW_REF && v.its == 1;
  // x / B = x * (conj(B) / |B|^2) (operator/): B's factor once, not per term
  Q Bi = {0, 0, 0, 0};
  if (ok) {
    const double inv = __ddiv_rn(1.0, norm2(B));
    Bi = Q{mul(B.w, inv), mul(-B.x, inv), mul(-B.y, inv), mul(-B.z, inv)};
  }
  double c_bulk_t = 0, c_bulk_b = 0, c_bad = 0;
  // top roots: left = forward[i-1], right = backward[i+1]
  Q left = {1, 0, 0, 0};
#pragma unroll 1
  for (int i = 0; i < nt; i++) {
    double c_i = 0;
    if (ok) {
      const Q right = (nt > 1 && i < nt - 1) ? Sf[i + 1] : Q{1, 0, 0, 0};
      const Q base{sub(q0.w, m.r64[i][0]), sub(q0.x, m.r64[i][1]), sub(q0.y, m.r64[i][2]),
                   sub(q0.z, m.r64[i][3])};
      const Q pw = reuse ? Pf[i] : qpow(base, m.e64[i]);
      const Q lg = qlog(base);
#pragma unroll 1
      for (int pass = 0; pass < 2; pass++) {
        const double k = pass == 0 ? m.sigma[0] : m.ep[i];
        const Q dT = qmul(qmul(left, qmul(qscale(pw, k), lg)), right);
        const double dSdt = mul(dSdF, mul(RR, qdot(R, qmul(dT, Bi))));
        if (isnan(dSdt) || isinf(dSdt)) {
          c_bad += 1;
          continue;
        }
        if (pass == 0)
          c_i = dSdt;
        else
          c_bulk_t += dSdt;
      }
      left = (i == 0) ? Pf[0] : qmul(left, Pf[i]);
    }
    warp_accum(acc, 1 + nb + i, c_i);
  }
  // bottom roots: the reference's formula, R' = T / (-left * middle * right)
  Q lb = {1, 0, 0, 0};
#pragma unroll 1
  for (int j = 0; j < nb; j++) {
    double c_j = 0;
    if (ok) {
      const Q right = (nb > 1 && j < nb - 1) ? Sf[nt + j + 1] : Q{1, 0, 0, 0};
      const Q base{sub(q0.w, m.r64[nt + j][0]), sub(q0.x, m.r64[nt + j][1]),
                   sub(q0.y, m.r64[nt + j][2]), sub(q0.z, m.r64[nt + j][3])};
      const Q pw = reuse ? Pf[nt + j] : qpow(base, m.e64[nt + j]);
      const Q li = qinv(qlog(base));
      const Q minus1 = {-1, 0, 0, 0};
#pragma unroll 1
      for (int pass = 0; pass < 2; pass++) {
        if (pass == 0 && !(m.sigma[1] > 0.0)) continue;
        if (pass == 1 && m.ep[nt + j] < 1e-8) continue;
        const double k = __ddiv_rn(1.0, pass == 0 ? m.sigma[1] : m.ep[nt + j]);
        const Q dB = qmul(qmul(qmul(minus1, lb), qmul(qscale(pw, k), li)), right);
        const double dSdt = mul(dSdF, mul(RR, qdot(R, qdiv(T, dB))));
        if (isnan(dSdt) || isinf(dSdt)) {
          c_bad += 1;
          continue;
        }
        if (pass == 0)
          c_j = dSdt;
        else
          c_bulk_b += dSdt;
      }
      lb = (j == 0) ? Pf[nt] : qmul(lb, Pf[nt + j]);
    }
    warp_accum(acc, 1 + j, c_j);
  }
  warp_accum(acc, 1 + nb + nt, c_bulk_t);
  warp_accum(acc, 2 + nb + nt, c_bulk_b);
  warp_accum(acc, s_bad, c_bad);
}

// The same terms on the extended factors of an overflowed voxel (the
// gradients' overflow passes: every term added, not-a-number included; the
// sigma_b terms summed apart).
__device__ __noinline__ void grad_terms_ext(const MapParams& m, const Q q0, bool ok, const QX Rx,
                                            const QX Tx, const QX Bx, double dSdF, const Q* Pf,
                                            const int* Pe, const Q* Sf, const int* Se,
                                            double* acc, int s_bulkb_x) {
  const int nt = m.nt, nb = m.nb;
  double c_bulk_t = 0, c_bulk_bx = 0;
  QX lx = {Q{1, 0, 0, 0}, 0};
#pragma unroll 1
  for (int i = 0; i < nt; i++) {
    double c_i = 0;
    if (ok) {
      const QX right = (nt > 1 && i < nt - 1) ? QX{Sf[i + 1], Se[i + 1]} : QX{Q{1, 0, 0, 0}, 0};
      const Q base{sub(q0.w, m.r64[i][0]), sub(q0.x, m.r64[i][1]), sub(q0.y, m.r64[i][2]),
                   sub(q0.z, m.r64[i][3])};
      const QX pw = xpow(base, m.e64[i]);
      const QX lg = xof(qlog(base));
#pragma unroll 1
      for (int pass = 0; pass < 2; pass++) {
        const double k = pass == 0 ? m.sigma[0] : m.ep[i];
        const QX dT = xmul(xmul(lx, xmul(xscale(pw, k), lg)), right);
        const double dSdt = mul(dSdF, xdot_ratio(Rx, xdiv(dT, Bx)));
        if (pass == 0)
          c_i = dSdt;
        else
          c_bulk_t += dSdt;
      }
      lx = (i == 0) ? QX{Pf[0], Pe[0]} : xmul(lx, QX{Pf[i], Pe[i]});
    }
    warp_accum(acc, 1 + nb + i, c_i);
  }
  QX lbx = {Q{1, 0, 0, 0}, 0};
#pragma unroll 1
  for (int j = 0; j < nb; j++) {
    double c_j = 0;
    if (ok) {
      const QX right = (nb > 1 && j < nb - 1) ? QX{Sf[nt + j + 1], Se[nt + j + 1]}
                                              : QX{Q{1, 0, 0, 0}, 0};
      const Q base{sub(q0.w, m.r64[nt + j][0]), sub(q0.x, m.r64[nt + j][1]),
                   sub(q0.y, m.r64[nt + j][2]), sub(q0.z, m.r64[nt + j][3])};
      const QX pw = xpow(base, m.e64[nt + j]);
      const QX li = xof(qinv(qlog(base)));
      const QX minus1 = {Q{-0.5, 0, 0, 0}, 1};
      // (the overflow pass of computeBottomGradientAP has no power-scalar
      // guard: with sigma_b = 0 its terms are not numbers, :10130-10216)
#pragma unroll 1
      for (int pass = 0; pass < 2; pass++) {
        if (pass == 1 && m.ep[nt + j] < 1e-8) continue;
        const double k = __ddiv_rn(1.0, pass == 0 ? m.sigma[1] : m.ep[nt + j]);
        const QX dB = xmul(xmul(xmul(minus1, lbx), xmul(xscale(pw, k), li)), right);
        const double dSdt = mul(dSdF, xdot_ratio(Rx, xdiv(Tx, dB)));
        if (pass == 0)
          c_j = dSdt;
        else
          c_bulk_bx += dSdt;
      }
      lbx = (j == 0) ? QX{Pf[nt], Pe[nt]} : xmul(lbx, QX{Pf[nt + j], Pe[nt + j]});
    }
    warp_accum(acc, 1 + j, c_j);
  }
  warp_accum(acc, 1 + nb + nt, c_bulk_t);
  warp_accum(acc, s_bulkb_x, c_bulk_bx);
}

// Block b takes a contiguous range of voxels, EN_T at a time.  Every voxel's
// map, field, score and d/d log s term are computed in the first step.  The
// per-parameter terms are skipped where they are exact zeros (saturated tanh
// or zero weight, with every intermediate provably in range); a warp with at
// least 24 voxels needing them computes them at once from the factors it
// holds (16.2 / 15.0 / 14.5 ms per pass at 8 / 16 / 24 on the 97^3
// objective benchmark), sparser ones queue their voxels in shared memory, in
// voxel order, to be re-evaluated and computed EN_T at a time in full warps.
template <bool POW_REF>
__global__ void __launch_bounds__(EN_T, 4) tanh_grad_kernel(const __grid_constant__ MapParams m,
                                                         const GridParams g, const WeightGrid wg,
                                                         const double* __restrict__ weights,
                                                         int max_it, double alpha, double thr,
                                                         double* __restrict__ field,
                                                         double* __restrict__ partials, int slots) {
  extern __shared__ double acc_sh[];  // [EN_T / 32][slots]
  __shared__ long long queue[2 * EN_T];
  __shared__ int queued, wcount[EN_T / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* acc = acc_sh + warp * slots;
  for (int k = threadIdx.x; k < (EN_T / 32) * slots; k += EN_T) acc_sh[k] = 0.0;
  if (threadIdx.x == 0) queued = 0;
  __syncthreads();
  Q Pf[QJ_MAX_ROOTS];  // last application's factors (local memory)
  Q Sf[QJ_MAX_ROOTS];  // their suffix products
  int Pe[QJ_MAX_ROOTS], Se[QJ_MAX_ROOTS];  // their exponents on the extended path
  const int nt = m.nt, nb = m.nb;
  const long long N = (long long)g.X * g.Y * g.Z;
  const double logs = log(m.scale);
  const int s_score = 3 + nt + nb, s_over = s_score + 1, s_bad = s_score + 2;
  const int s_bulkb_x = s_score + 3, s_band = s_score + 4;
  // every k a gradient term scales by (sigma_t, e_i; 1/sigma_b, 1/e_j) within
  // [1e-10, 1e10] (or zero where a term is identically zero)
  bool k_ok = (m.sigma[0] == 0.0 || (fabs(m.sigma[0]) >= 1e-10 && fabs(m.sigma[0]) <= 1e10)) &&
              (!(m.sigma[1] > 0.0) || (m.sigma[1] >= 1e-10 && m.sigma[1] <= 1e10));
  for (int i = 0; i < nt + nb; i++) {
    const double e = fabs(m.ep[i]);
    k_ok = k_ok && (e == 0.0 || (e >= 1e-10 && e <= 1e10));
  }
  const long long per = (N + gridDim.x - 1) / gridDim.x;
  const long long lo_b = (long long)blockIdx.x * per;
  const long long hi_b = lo_b + per < N ? lo_b + per : N;
  auto cell = [&](long long idx, double* p) {
    const int x = (int)(idx % g.X), y = (int)((idx / g.X) % g.Y);
    const int z = (int)(idx / ((long long)g.X * g.Y));
    cell_center(g, x, y, z, p);
  };
  // the queued voxels' terms: each thread re-evaluates one voxel's map
  auto drain = [&](int count) {
    const bool ok = threadIdx.x < count;
    Voxel v;
    Q R = {0, 0, 0, 0};
    double dSdF = 0, RR = 0;
    bool good = false;
    if (ok) {
      double p[3];
      cell(queue[threadIdx.x], p);
      eval_voxel<POW_REF, false>(m, Q{p[0], p[1], p[2], g.slice}, max_it, Pf, Sf, v);
      good = grad_setup(v, logs, alpha, thr, trilinear(wg, weights, p), R, dSdF, RR);
    } else {
      v.its = 0;
    }
    grad_terms<POW_REF>(m, v, good, R, dSdF, RR, Pf, Sf, acc, s_bad);
  };
  for (long long base = lo_b; base < hi_b; base += EN_T) {
    const long long idx = base + threadIdx.x;
    const bool live = idx < hi_b;
    double c_exp = 0, c_score = 0, c_over = 0, c_band = 0;
    bool want = false, ext = false;
    Voxel v;
    v.over = false;
    v.iterated = false;
    v.its = 0;
    double dSdF = 0;
    QX Tx = {Q{1, 0, 0, 0}, 0}, Bx = Tx, Rx = Tx;
    Q q0 = {0, 0, 0, 0};
    Q Rg = {0, 0, 0, 0};
    double RRg = 0;
    if (live) {
      double p[3];
      cell(idx, p);
      q0 = Q{p[0], p[1], p[2], g.slice};
      eval_voxel<POW_REF, true>(m, q0, max_it, Pf, Sf, v);
      double fval = 0.0;
      if (v.iterated || v.mg >= 1e-8) fval = log(v.mg);
      if (!(mag(q0) < 1e-8) && v.over)
        fval = ext_map<POW_REF>(m, q0, max_it, Pf, Pe, &Tx, &Bx);
      if (field) field[idx] = fval;
      const double w = trilinear(wg, weights, p);
      c_score = mul(-tanh(mul(alpha, fval)), w);
      {
        const double S = tanh(mul(alpha, sub(fval, thr)));
        c_exp = mul(mul(-alpha, w), sub(1.0, mul(S, S)));
      }
      c_over = v.over ? 1.0 : 0.0;
      if (v.iterated && !v.over) {
        Q& R = Rg;
        double& RR = RRg;
        if (grad_setup(v, logs, alpha, thr, w, R, dSdF, RR)) {
          // dSdF = 0 makes every term dSdF * y an exact zero; y stays finite
          // when the factors' magnitudes spread over at most 2^300, every
          // q0 - root is moderate and away from 1 and every k is moderate
          const double r2 = qdot(R, R), b2 = norm2(v.B);
          const bool zero_terms = dSdF == 0.0 && k_ok && v.bases_ok && v.spread <= 300 &&
                                  r2 > 1e-260 && r2 < 1e260 && b2 > 1e-130 && b2 < 1e130;
          want = !zero_terms;
        }
      } else if (v.iterated) {
        // the gradients' overflow pass, on the extended factors
        Rx = xdiv(Tx, Bx);
        if (qdot(Rx.m, Rx.m) > 0.0 && isfinite(Rx.m.w)) {
          const double F = add(xlogmag(Rx), logs);
          const double th = tanh(mul(alpha, sub(F, thr)));
          dSdF = mul(mul(-alpha, w), sub(1.0, mul(th, th)));
          ext = true;
#pragma unroll 1
          for (int side = 0; side < 2; side++) {
            const int lo = side ? nt : 0, hi = side ? nt + nb : nt;
            if (hi == lo) continue;
            Sf[hi - 1] = Pf[hi - 1];
            Se[hi - 1] = Pe[hi - 1];
#pragma unroll 1
            for (int i = hi - 2; i >= lo; i--) {
              const QX sx = xmul(QX{Pf[i], Pe[i]}, QX{Sf[i + 1], Se[i + 1]});
              Sf[i] = sx.m;
              Se[i] = sx.e;
            }
          }
        }
      }
      c_band = want ? 1.0 : 0.0;
    }
    warp_accum(acc, 0, c_exp);
    warp_accum(acc, s_score, c_score);
    warp_accum(acc, s_over, c_over);
    warp_accum(acc, s_band, c_band);
    if (__any_sync(0xffffffffu, ext))
      grad_terms_ext(m, q0, ext, Rx, Tx, Bx, dSdF, Pf, Pe, Sf, Se, acc, s_bulkb_x);
    // a warp with many voxels needing their terms computes them now, from
    // the factors it holds; the others append theirs to the queue, in voxel
    // order, to be computed in full warps
    unsigned bal = __ballot_sync(0xffffffffu, want);
    if (__popc(bal) >= 24) {
      grad_terms<POW_REF>(m, v, want, Rg, dSdF, RRg, Pf, Sf, acc, s_bad);
      bal = 0;
      want = false;
    }
    if (lane == 0) wcount[warp] = __popc(bal);
    __syncthreads();
    int off = queued;
    for (int k = 0; k < warp; k++) off += wcount[k];
    if (want) queue[off + __popc(bal & ((1u << lane) - 1u))] = idx;
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int k = 0; k < EN_T / 32; k++) tot += wcount[k];
      queued += tot;
    }
    __syncthreads();
    if (queued >= EN_T) {
      drain(EN_T);
      __syncthreads();
      const int rest = queued - EN_T;
      if (threadIdx.x < rest) queue[threadIdx.x] = queue[EN_T + threadIdx.x];
      __syncthreads();
      if (threadIdx.x == 0) queued = rest;
      __syncthreads();
    }
  }
  if (queued > 0) drain(queued);
  __syncthreads();
  for (int k = threadIdx.x; k < slots; k += EN_T) {
    double s = 0;
    for (int wv = 0; wv < EN_T / 32; wv++) s += acc_sh[wv * slots + k];
    partials[(long long)blockIdx.x * slots + k] = s;
  }
}

// Neumaier-compensated sum of partials[b][k] over blocks b, in block order.
// The loads of 16 rows are issued before their additions (same additions in
// the same order), so the loop waits on memory once per 16 rows.
__global__ void reduce_partials_kernel(const double* __restrict__ partials, int nblocks,
                                       int slots, double* __restrict__ out) {
  constexpr int U = 16;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < slots; k += gridDim.x * blockDim.x) {
    double s = 0, c = 0;
    for (int b0 = 0; b0 < nblocks; b0 += U) {
      double v[U];
#pragma unroll
      for (int u = 0; u < U; u++)
        v[u] = b0 + u < nblocks ? partials[(long long)(b0 + u) * slots + k] : 0.0;
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (b0 + u >= nblocks) break;
        const double t = s + v[u];
        c += (fabs(s) >= fabs(v[u])) ? (s - t) + v[u] : (v[u] - t) + s;
        s = t;
      }
    }
    out[k] = s + c;
  }
}

// computeBottomBulkScalarGradientAP starts its overflow pass from zeroed
// per-slice sums (OPTIMIZE_3D.cpp:10466-10471) where
// computeTopBulkScalarGradientAP keeps them: once any voxel overflowed or gave
// a non-finite term, the sigma_b gradient is the overflow pass's sum alone.
__global__ void bottom_bulk_fix_kernel(double* __restrict__ out, int nt, int nb) {
  const int s_score = 3 + nt + nb;
  if (out[s_score + 1] + out[s_score + 2] > 0.0) out[2 + nb + nt] = out[s_score + 3];
}

}  // namespace

int tanh_slots(int nt, int nb) { return 8 + nt + nb; }

int tanh_blocks() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms * 4;
}

cudaError_t launch_tanh_grad(const MapParams& m, const GridParams& g, const WeightGrid& wg,
                             const double* weights, int max_it, double alpha, double thr,
                             bool pow_ref, double* field, double* partials, int nblocks,
                             double* out, cudaStream_t s) {
  const int slots = tanh_slots(m.nt, m.nb);
  const size_t sh = sizeof(double) * (EN_T / 32) * slots;
  if (pow_ref)
    tanh_grad_kernel<true><<<nblocks, EN_T, sh, s>>>(m, g, wg, weights, max_it, alpha, thr, field,
                                                     partials, slots);
  else
    tanh_grad_kernel<false><<<nblocks, EN_T, sh, s>>>(m, g, wg, weights, max_it, alpha, thr,
                                                      field, partials, slots);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  reduce_partials_kernel<<<1, 256, 0, s>>>(partials, nblocks, slots, out);
  bottom_bulk_fix_kernel<<<1, 1, 0, s>>>(out, m.nt, m.nb);
  return cudaGetLastError();
}

// ===========================================================================
// Squared-error fitting energy on the distance estimate and its adjoint.
//
// No reference counterpart (the reference tracks no derivative of this map
// and fits only exponents and scales).  Per sample x_k with target t_k
// (the fitted value is D tanh(d / D) with D = d_sat, so that samples deep
// inside, whose |q'| contracts towards zero and whose d grows without bound,
// saturate instead of dominating the sum):
//   q_0 = (x, y, z, slice); for n < N (escape test as the field):
//     d_i = q_n - r_i, P_i = d_i^{e_i} (polar power), T = prod top P_i,
//     B = prod bottom P_i, q_{n+1} = s T B^-1,
//     g_n = sum_top e_i d_i/|d_i|^2 - sum_bot e_j d_j/|d_j|^2,
//     L_{n+1} = L_n + log|g_n| + log|q_{n+1}|          (L = log|q'|)
//   d = |q_N| log|q_N| exp(-L_N),  E = sum_k (D tanh(d_k / D) - t_k)^2.
// Parameters: root positions (4 each), effective exponents, log s, laid out
// [top roots 4nt | bottom roots 4nb | top exps nt | bottom exps nb | log s].
// The forward pass keeps q at every SQ_CK-th iteration of the samples whose
// gradient is wanted (every iteration: SQ_CK = 1); the backward pass
// recomputes each segment forward from its first kept point before
// reversing it (nothing to recompute at SQ_CK = 1).
// ===========================================================================
namespace {

constexpr int SQ_T = 64;    // threads per block of the backward pass
constexpr int SQ_BWD_PER_SM = 8;  // backward blocks per SM
constexpr int SQF_T = 128;  // threads per block of the forward pass
constexpr int SQC_T = 256;  // threads per chunk block
constexpr int SQ_CH = 2048; // samples per chunk (sums and sort)
// Spacing of the kept orbit points (iterations).  1: the adjoint evaluates
// every Jacobian at the forward pass's own orbit.  A wider spacing saves
// memory, but its recomputed segments must reproduce the forward's rounding
// bit for bit: with the roots of a step spread over lanes (products in
// another order) a recomputed orbit drifts from the forward's and the FP32
// gradient lost a factor of 10-40 in accuracy at spacing 8.
constexpr int SQ_CK = 1;
constexpr int SQ_MAXIT = 256;

template <class T>
struct V4 {
  T w, x, y, z;
};

template <class T>
__device__ __forceinline__ V4<T> v4mul(const V4<T>& a, const V4<T>& b) {
  return V4<T>{a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z,
               a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
               a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
               a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w};
}
template <class T>
__device__ __forceinline__ V4<T> v4conj(const V4<T>& a) { return V4<T>{a.w, -a.x, -a.y, -a.z}; }
template <class T>
__device__ __forceinline__ T v4dot(const V4<T>& a, const V4<T>& b) {
  return a.w * b.w + a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class T>
__device__ __forceinline__ V4<T> v4scale(const V4<T>& a, T k) {
  return V4<T>{a.w * k, a.x * k, a.y * k, a.z * k};
}
template <class T>
__device__ __forceinline__ V4<T> v4add(const V4<T>& a, const V4<T>& b) {
  return V4<T>{a.w + b.w, a.x + b.x, a.y + b.y, a.z + b.z};
}

// polar power (the form of QUATERNION::pow) and its vector-Jacobian product
template <class T>
struct PowParts {
  T rho, vm, theta, A, c, s;
};

// The FP32 polar power's fast form (the default; qjg_set_energy_fast(0)
// selects the accurate device functions): the angle from a polynomial atan
// and the PTX approximations of log2, exp2, sin/cos, the reciprocal (every
// division) and the reciprocal square root, with denormals flushed.  On the
// differentiation workload (200k samples, 64/16 roots, 30 iterations) it
// moves the FP32 energy from 3e-9 to 8e-8 of the FP64 form's; the FP32
// gradient stays within 1e-5 of the FP64 form's (about 1e-6 measured).
__constant__ int c_sq_fast = 1;

// How a device function picks the FP32 form: SQM_RT reads the switch
// (c_sq_fast) where it is used; SQM_FAST and SQM_ACC fix the form at compile
// time, so that a kernel instantiated for one form runs its root loop as
// straight-line code (the forward kernel tests the switch once, at entry).
// The FP64 form ignores the mode.
constexpr int SQM_RT = 0, SQM_FAST = 1, SQM_ACC = 2;

template <int M>
__device__ __forceinline__ bool sq_fast() {
  if constexpr (M == SQM_FAST) return true;
  if constexpr (M == SQM_ACC) return false;
  return c_sq_fast != 0;
}

// The fast form's transcendentals: the PTX approximations with denormal
// inputs and results flushed to zero, one special-function instruction each
// (the device library's __log2f, rsqrtf and exp2f add a denormal range fix-up
// around the same approximation).  Accuracy as documented for the PTX
// instructions: ex2 and lg2 about 2^-22 relative / absolute, rsqrt and rcp
// about 1 ulp, sin and cos 2^-20.5 absolute for arguments within [-pi, pi]
// (|e theta| stays within a few pi here).
__device__ __forceinline__ float lg2_ftz(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float ex2_ftz(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sin_ftz(float x) {
  float y;
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float cos_ftz(float x) {
  float y;
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// smallest normal FP32 value: below it the flushed approximations read 0
constexpr float SQ_FLT_MIN = 1.17549435e-38f;

// atan(t) for 0 <= t <= 1 as t P(t^2), P of degree 7 fitted for this
// library (weighted least squares on Chebyshev nodes of t^2 in [0, 1]; max
// relative error 2.3e-7 evaluated in FP32)
__device__ __forceinline__ float atan01_fast(float t) {
  const float u = t * t;
  float p = -0.004780514165759087f;
  p = fmaf(p, u, 0.024557340890169144f);
  p = fmaf(p, u, -0.0599050298333168f);
  p = fmaf(p, u, 0.09942781925201416f);
  p = fmaf(p, u, -0.14029428362846375f);
  p = fmaf(p, u, 0.19971376657485962f);
  p = fmaf(p, u, -0.3333209455013275f);
  p = fmaf(p, u, 0.9999999403953552f);
  return p * t;
}

// atan2(y, x) for y >= 0, in [0, pi]
__device__ __forceinline__ float atan2_pos_fast(float y, float x) {
  const float ax = fabsf(x);
  const float mx = fmaxf(ax, y), mn = fminf(ax, y);
  float a = mx > SQ_FLT_MIN ? atan01_fast(mn * rcp_ftz(mx)) : 0.f;
  if (y > ax) a = 1.57079632679489662f - a;
  return x < 0.f ? 3.14159265358979324f - a : a;
}

// a / b: FP64 and the accurate FP32 form divide (IEEE); the fast FP32 form
// multiplies by the hardware reciprocal, whose IEEE division sequence was a
// tenth of the adjoint's instructions.
template <class T, int M = SQM_RT>
__device__ __forceinline__ T sq_div(T a, T b) {
  if constexpr (std::is_same<T, float>::value) {
    if (sq_fast<M>()) return a * rcp_ftz(b);
  }
  return a / b;
}

// The polar power d^e (the form of QUATERNION::pow).  The fast FP32 form
// also returns |d|^2 through r2out (the log-gradient term divides by it).
template <class T, int M = SQM_RT>
__device__ __forceinline__ V4<T> powv(const V4<T>& d, T e, PowParts<T>* pp,
                                      T* r2out = nullptr) {
  if constexpr (std::is_same<T, float>::value) {
    // FP32: the same polar form through base-2 logarithm and exponential,
    // the angle as atan2(|v|, w), and 1/|v| as one reciprocal square root
    const float v2 = d.x * d.x + d.y * d.y + d.z * d.z;
    const float r2 = v2 + d.w * d.w;
    if (r2out) *r2out = r2;
    float theta, A, s, c, rv;
    if (sq_fast<M>()) {
      rv = v2 > SQ_FLT_MIN ? rsqrt_ftz(v2) : 0.f;
      theta = atan2_pos_fast(v2 * rv, d.w);
      A = ex2_ftz(0.5f * e * lg2_ftz(r2));
      const float ang = e * theta;
      s = sin_ftz(ang);
      c = cos_ftz(ang);
    } else {
      rv = v2 > 0.f ? rsqrtf(v2) : 0.f;
      theta = atan2f(v2 * rv, d.w);
      A = exp2f(0.5f * e * log2f(r2));
      sincospif(e * theta * 0.318309886183790672f, &s, &c);
    }
    const float vm = v2 * rv;
    const float k = A * s * rv;
    if (pp) {
      // rho = sqrt(r2), as r2 rsqrt(r2) in the fast form
      const float rho =
          sq_fast<M>() ? (r2 > SQ_FLT_MIN ? r2 * rsqrt_ftz(r2) : 0.f) : sqrtf(r2);
      *pp = PowParts<T>{rho, vm, theta, A, c, s};
    }
    return V4<T>{A * c, k * d.x, k * d.y, k * d.z};
  }
  const T v2 = d.x * d.x + d.y * d.y + d.z * d.z;
  const T rho = sqrt(v2 + d.w * d.w), vm = sqrt(v2);
  const T theta = acos(d.w / rho);
  const T A = exp(e * log(rho));
  T s, c;
  sincos(e * theta, &s, &c);
  const T k = vm > T(0) ? A * s / vm : T(0);
  if (pp) *pp = PowParts<T>{rho, vm, theta, A, c, s};
  return V4<T>{A * c, k * d.x, k * d.y, k * d.z};
}

// given Pbar, accumulate dbar (returned) and ebar
template <class T, int M = SQM_RT>
__device__ __forceinline__ V4<T> powv_vjp(const V4<T>& d, T e, const PowParts<T>& p,
                                          const V4<T>& Pb, T* ebar) {
  // 1/|v| and 1/rho once (FP64: IEEE divisions)
  const T ivm = p.vm > T(0) ? sq_div<T, M>(T(1), p.vm) : T(0);
  const T irho = sq_div<T, M>(T(1), p.rho);
  const T ux = d.x * ivm, uy = d.y * ivm, uz = d.z * ivm;
  const T pu = Pb.x * ux + Pb.y * uy + Pb.z * uz;
  const T Ab = Pb.w * p.c + pu * p.s;
  const T phib = p.A * (pu * p.c - Pb.w * p.s);
  const T rhob = Ab * e * p.A * irho;
  const T thetab = phib * e;
  T lrho;
  if constexpr (std::is_same<T, float>::value) {
    // log(rho) = ln 2 log2(rho): the fast form's approximation
    lrho = sq_fast<M>() ? 0.693147180559945309f * lg2_ftz(p.rho) : logf(p.rho);
  } else {
    lrho = log(p.rho);
  }
  *ebar += Ab * p.A * lrho + phib * p.theta;
  const T ir2 = irho * irho;
  V4<T> db;
  db.w = rhob * d.w * irho - thetab * p.vm * ir2;
  const T kv = rhob * irho;
  const T kt = thetab * d.w * ir2;
  db.x = kv * d.x + kt * ux;
  db.y = kv * d.y + kt * uy;
  db.z = kv * d.z + kt * uz;
  if (p.vm > T(0)) {
    // u = v / |v|: (I - u u^T) ubar / |v| with ubar = A sin(phi) Pbar_v
    const T ub = p.A * p.s;
    const T ubx = ub * Pb.x, uby = ub * Pb.y, ubz = ub * Pb.z;
    const T proj = ubx * ux + uby * uy + ubz * uz;
    db.x += (ubx - proj * ux) * ivm;
    db.y += (uby - proj * uy) * ivm;
    db.z += (ubz - proj * uz) * ivm;
  }
  return db;
}

// One map application q -> Q with log|g|; fills prefix products F (per
// side) and factors P when given.  The first root of each side starts the
// side's running product (no multiply by one, no select in the loop).
template <class T, int M = SQM_RT>
__device__ __forceinline__ V4<T> sq_apply(const T* __restrict__ rp, const T* __restrict__ ep,
                                          int nt, int nb, T s, const V4<T>& q, T* lg,
                                          V4<T>* F, V4<T>* Pf, V4<T>* Tout, V4<T>* Bout) {
  // acc[0]: top product, acc[1]: bottom product (two loops, so that the
  // running products stay in registers)
  V4<T> acc[2] = {{T(1), T(0), T(0), T(0)}, {T(1), T(0), T(0), T(0)}};
  V4<T> g = {T(0), T(0), T(0), T(0)};
  // root i's factor; its log-gradient term sgn e d / |d|^2 added to g
  auto term = [&](int i, bool bottom) -> V4<T> {
    const V4<T> d{q.w - rp[4 * i], q.x - rp[4 * i + 1], q.y - rp[4 * i + 2], q.z - rp[4 * i + 3]};
    const T e = ep[i];
    const T se = bottom ? -e : e;
    V4<T> P;
    T k;
    bool fast = false;
    if constexpr (std::is_same<T, float>::value) fast = sq_fast<M>();
    if (fast) {
      // |d|^2 from the polar power's own sum
      T r2;
      P = powv<T, M>(d, e, nullptr, &r2);
      k = sq_div<T, M>(se, r2);
    } else {
      k = sq_div<T, M>(se, v4dot(d, d));
      P = powv<T, M>(d, e, nullptr);
    }
    g = v4add(g, v4scale(d, k));
    if (Pf) Pf[i] = P;
    return P;
  };
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const int lo = side ? nt : 0, hi = side ? nt + nb : nt;
    if (lo == hi) continue;
    V4<T> a = term(lo, side != 0);
    if (F) F[lo] = a;
    for (int i = lo + 1; i < hi; i++) {
      a = v4mul(a, term(i, side != 0));
      if (F) F[i] = a;
    }
    acc[side] = a;
  }
  V4<T> Q;
  if (nb > 0) {
    const V4<T> W = v4scale(v4conj(acc[1]), sq_div<T, M>(T(1), v4dot(acc[1], acc[1])));
    Q = v4scale(v4mul(acc[0], W), s);
  } else {
    Q = v4scale(acc[0], s);
  }
  *lg = T(0.5) * log(v4dot(g, g));
  if (Tout) *Tout = acc[0];
  if (Bout) *Bout = acc[1];
  return Q;
}

// The fitted value D tanh(d / D) (d itself when D <= 0) and its derivative;
// a sample whose |d| exceeds 20 D is saturated: value +-D, no gradient.
template <class T>
__device__ __forceinline__ void sq_saturate(T lm, T ld, T dsat, T* val, T* d, T* dval_dd) {
  const T sgn = lm < T(0) ? T(-1) : T(1);
  if (lm == T(0)) {
    *d = T(0);
    *val = T(0);
    *dval_dd = T(1);
    return;
  }
  if (dsat > T(0) && ld > log(T(20) * dsat)) {
    *d = sgn * T(20) * dsat;
    *val = sgn * dsat;
    *dval_dd = T(0);
    return;
  }
  *d = sgn * exp(ld);
  if (dsat > T(0)) {
    const T th = tanh(*d / dsat);
    *val = dsat * th;
    *dval_dd = T(1) - th * th;
  } else {
    *val = *d;
    *dval_dd = T(1);
  }
}

// Per-sample results of the forward pass.  keys[k]: the orbit length N of a
// sample whose gradient the backward pass computes (N >= 1), -1 for a sample
// that adds nothing to the gradient (saturated, or N = 0), -2 for a sample
// left out because its seed is not finite (counted).
template <class T>
struct SqFwdOut {
  double* contrib;  // (D tanh(d/D) - t)^2 per sample
  int* keys;
  int* iters;       // orbit lengths (optional)
  V4<T>* seed_q;    // dE/dq_N per sample (gradient pass)
  T* seed_L;        // dE/dL (constant along the orbit)
  V4<T>* ck;        // q_n at n = 0, SQ_CK, 2 SQ_CK, ...: ck[(n / SQ_CK) * n_samples + k]
};

// Forward pass with lane refill: every lane iterates its own sample and takes
// the next unclaimed one (a warp-aggregated atomic on *claim) as soon as its
// orbit ends, so a warp's lanes stay busy however the orbit lengths differ.
// The per-sample results go to SqFwdOut; the sums are formed afterwards in
// sample order, so they do not depend on which lane took which sample.
template <class T, bool GRAD, int M>
__device__ __forceinline__ void sq_fwd_body(
    const double* __restrict__ params, int nt, int nb, const double* __restrict__ xyz,
    const double* __restrict__ target, long long n_samples, double slice, int max_it,
    double escape, double d_sat, unsigned long long* __restrict__ claim, const SqFwdOut<T>& o) {
  extern __shared__ unsigned char sh_raw[];
  const int nr = nt + nb;
  T* rp = reinterpret_cast<T*>(sh_raw);  // 4 nr
  T* ep = rp + 4 * nr;                   // nr
  for (int k = threadIdx.x; k < 4 * nr; k += SQF_T) rp[k] = (T)params[k];
  for (int k = threadIdx.x; k < nr; k += SQF_T) ep[k] = (T)params[4 * nr + k];
  __syncthreads();
  const T s = (T)exp(params[5 * nr]);
  const T esc = (T)escape, dsat = (T)d_sat;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;

  // the sample's value, residual and (gradient pass) seed
  auto finish = [&](long long k, const V4<T>& q, T L, int n) {
    const T m = sqrt(v4dot(q, q));
    // log|d| first: contracting orbits drive L far below zero, and d itself
    // out of range, long before d matters
    const T lm = log(m);
    const T ld = log(fabs(lm)) + lm - L;
    if (o.iters) o.iters[k] = n;
    T val, dval, dval_dd;
    sq_saturate<T>(lm, ld, dsat, &val, &dval, &dval_dd);
    const T r = val - (T)target[k];
    o.contrib[k] = (double)(r * r);
    if (!GRAD) return;
    int key = -1;
    if (dval_dd != T(0)) {
      // seed: dE/dd = 2 r dval/dd; d = m log m exp(-L):
      // dd/dm = (log m + 1) exp(-L) = d (log m + 1) / (m log m)
      const T db = T(2) * r * dval_dd;
      const T kq = db * (lm + T(1)) * exp(ld - log(m) - log(fabs(lm)));
      if (!isfinite(kq) || !isfinite(db * dval)) {
        key = -2;
      } else if (n > 0) {
        o.seed_q[k] = v4scale(q, kq / m);  // d/dq_N of d: (dd/dm) q_N / m
        o.seed_L[k] = -db * dval;
        key = n;
      }
    }
    o.keys[k] = key;
  };

  long long k = 0;
  bool live = false, done = false;
  V4<T> q{T(0), T(0), T(0), T(0)};
  T L = T(0);
  int n = 0;
  for (;;) {
    // lanes without a sample claim one; a claimed sample whose orbit does
    // not start (|q_0| >= escape or max_it = 0) ends at once and claims again
    unsigned want = __ballot_sync(0xffffffffu, !live && !done);
    while (want) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(claim, (unsigned long long)__popc(want));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (!live && !done) {
        k = (long long)(base + __popc(want & lt));
        if (k >= n_samples) {
          done = true;
        } else {
          q = V4<T>{(T)xyz[3 * k], (T)xyz[3 * k + 1], (T)xyz[3 * k + 2], (T)slice};
          L = T(0);
          n = 0;
          if (sqrt(v4dot(q, q)) < esc && n < max_it)
            live = true;
          else
            finish(k, q, L, n);
        }
      }
      want = __ballot_sync(0xffffffffu, !live && !done);
    }
    if (!__any_sync(0xffffffffu, live)) break;
    if (live) {
      if (GRAD && n % SQ_CK == 0) o.ck[(long long)(n / SQ_CK) * n_samples + k] = q;
      T lg;
      q = sq_apply<T, M>(rp, ep, nt, nb, s, q, &lg, nullptr, nullptr, nullptr, nullptr);
      L += lg + T(0.5) * log(v4dot(q, q));
      n++;
      // 10 * FLT_MIN exit of the field loop
      const T m = sqrt(v4dot(q, q));
      if (!(m < esc && n < max_it) || m < T(1.1754943508e-37)) {
        finish(k, q, L, n);
        live = false;
      }
    }
  }
}

// The FP32 form is chosen once per launch, so that each form's root loop is
// compiled as straight-line code.
template <class T, bool GRAD>
__global__ void __launch_bounds__(SQF_T) sq_fwd_kernel(
    const double* __restrict__ params, int nt, int nb, const double* __restrict__ xyz,
    const double* __restrict__ target, long long n_samples, double slice, int max_it,
    double escape, double d_sat, unsigned long long* __restrict__ claim, SqFwdOut<T> o) {
  if constexpr (std::is_same<T, float>::value) {
    if (c_sq_fast) {
      sq_fwd_body<T, GRAD, SQM_FAST>(params, nt, nb, xyz, target, n_samples, slice, max_it,
                                     escape, d_sat, claim, o);
      return;
    }
  }
  sq_fwd_body<T, GRAD, SQM_ACC>(params, nt, nb, xyz, target, n_samples, slice, max_it, escape,
                                d_sat, claim, o);
}

// Two map applications that share the walk over the roots: the same
// arithmetic as sq_apply for each of qa and qb, so each keeps its bits, with
// the root constants read once and two independent dependency chains.
template <class T, int M = SQM_RT>
__device__ __forceinline__ void sq_apply2(const T* __restrict__ rp, const T* __restrict__ ep,
                                          int nt, int nb, T s, V4<T>& qa, T* lga, V4<T>& qb,
                                          T* lgb) {
  V4<T> acc[2][2] = {{{T(1), T(0), T(0), T(0)}, {T(1), T(0), T(0), T(0)}},
                     {{T(1), T(0), T(0), T(0)}, {T(1), T(0), T(0), T(0)}}};
  V4<T> ga = {T(0), T(0), T(0), T(0)}, gb = ga;
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const int lo = side ? nt : 0, hi = side ? nt + nb : nt;
    V4<T> a = acc[0][side], b = acc[1][side];
    for (int i = lo; i < hi; i++) {
      const T r0 = rp[4 * i], r1 = rp[4 * i + 1], r2 = rp[4 * i + 2], r3 = rp[4 * i + 3];
      const T e = ep[i];
      const V4<T> da{qa.w - r0, qa.x - r1, qa.y - r2, qa.z - r3};
      const V4<T> db{qb.w - r0, qb.x - r1, qb.y - r2, qb.z - r3};
      const T ka = sq_div<T, M>(side ? -e : e, v4dot(da, da));
      const T kb = sq_div<T, M>(side ? -e : e, v4dot(db, db));
      ga = v4add(ga, v4scale(da, ka));
      gb = v4add(gb, v4scale(db, kb));
      const V4<T> Pa = powv<T, M>(da, e, nullptr);
      const V4<T> Pb = powv<T, M>(db, e, nullptr);
      a = i == lo ? Pa : v4mul(a, Pa);
      b = i == lo ? Pb : v4mul(b, Pb);
    }
    acc[0][side] = a;
    acc[1][side] = b;
  }
  if (nb > 0) {
    const V4<T> Wa = v4scale(v4conj(acc[0][1]), sq_div<T, M>(T(1), v4dot(acc[0][1], acc[0][1])));
    const V4<T> Wb = v4scale(v4conj(acc[1][1]), sq_div<T, M>(T(1), v4dot(acc[1][1], acc[1][1])));
    qa = v4scale(v4mul(acc[0][0], Wa), s);
    qb = v4scale(v4mul(acc[1][0], Wb), s);
  } else {
    qa = v4scale(acc[0][0], s);
    qb = v4scale(acc[1][0], s);
  }
  *lga = T(0.5) * log(v4dot(ga, ga));
  *lgb = T(0.5) * log(v4dot(gb, gb));
}

// The forward pass with two samples per lane (slots 0 and 1), each refilled
// as in sq_fwd_kernel; both slots step through one sq_apply2.  A slot without
// a sample steps a dummy point whose results are not used.
template <class T, bool GRAD, int M>
__device__ __forceinline__ void sq_fwd2_body(
    const double* __restrict__ params, int nt, int nb, const double* __restrict__ xyz,
    const double* __restrict__ target, long long n_samples, double slice, int max_it,
    double escape, double d_sat, unsigned long long* __restrict__ claim, SqFwdOut<T> o) {
  extern __shared__ unsigned char sh_raw[];
  const int nr = nt + nb;
  T* rp = reinterpret_cast<T*>(sh_raw);
  T* ep = rp + 4 * nr;
  for (int k = threadIdx.x; k < 4 * nr; k += SQF_T) rp[k] = (T)params[k];
  for (int k = threadIdx.x; k < nr; k += SQF_T) ep[k] = (T)params[4 * nr + k];
  __syncthreads();
  const T s = (T)exp(params[5 * nr]);
  const T esc = (T)escape, dsat = (T)d_sat;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  auto finish = [&](long long k, const V4<T>& q, T L, int n) {
    const T m = sqrt(v4dot(q, q));
    const T lm = log(m);
    const T ld = log(fabs(lm)) + lm - L;
    if (o.iters) o.iters[k] = n;
    T val, dval, dval_dd;
    sq_saturate<T>(lm, ld, dsat, &val, &dval, &dval_dd);
    const T r = val - (T)target[k];
    o.contrib[k] = (double)(r * r);
    if (!GRAD) return;
    int key = -1;
    if (dval_dd != T(0)) {
      const T db = T(2) * r * dval_dd;
      const T kq = db * (lm + T(1)) * exp(ld - log(m) - log(fabs(lm)));
      if (!isfinite(kq) || !isfinite(db * dval)) {
        key = -2;
      } else if (n > 0) {
        o.seed_q[k] = v4scale(q, kq / m);
        o.seed_L[k] = -db * dval;
        key = n;
      }
    }
    o.keys[k] = key;
  };
  long long k[2] = {0, 0};
  bool live[2] = {false, false};
  bool done = false;
  V4<T> q[2] = {{T(0), T(0), T(0), T(0)}, {T(0), T(0), T(0), T(0)}};
  T L[2] = {T(0), T(0)};
  int n[2] = {0, 0};
  for (;;) {
#pragma unroll
    for (int sl = 0; sl < 2; sl++) {
      unsigned want = __ballot_sync(0xffffffffu, !live[sl] && !done);
      while (want) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(claim, (unsigned long long)__popc(want));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (!live[sl] && !done) {
          k[sl] = (long long)(base + __popc(want & lt));
          if (k[sl] >= n_samples) {
            done = true;
          } else {
            const long long kk = k[sl];
            q[sl] = V4<T>{(T)xyz[3 * kk], (T)xyz[3 * kk + 1], (T)xyz[3 * kk + 2], (T)slice};
            L[sl] = T(0);
            n[sl] = 0;
            if (sqrt(v4dot(q[sl], q[sl])) < esc && n[sl] < max_it)
              live[sl] = true;
            else
              finish(kk, q[sl], L[sl], n[sl]);
          }
        }
        want = __ballot_sync(0xffffffffu, !live[sl] && !done);
      }
    }
    if (!__any_sync(0xffffffffu, live[0] || live[1])) break;
#pragma unroll
    for (int sl = 0; sl < 2; sl++)
      if (GRAD && live[sl] && n[sl] % SQ_CK == 0)
        o.ck[(long long)(n[sl] / SQ_CK) * n_samples + k[sl]] = q[sl];
    V4<T> qa = live[0] ? q[0] : V4<T>{T(0.5), T(0.5), T(0.5), T(0.5)};
    V4<T> qb = live[1] ? q[1] : V4<T>{T(0.5), T(0.5), T(0.5), T(0.5)};
    T lga, lgb;
    sq_apply2<T, M>(rp, ep, nt, nb, s, qa, &lga, qb, &lgb);
#pragma unroll
    for (int sl = 0; sl < 2; sl++) {
      if (!live[sl]) continue;
      const V4<T>& qn = sl ? qb : qa;
      q[sl] = qn;
      L[sl] += (sl ? lgb : lga) + T(0.5) * log(v4dot(qn, qn));
      n[sl]++;
      const T m = sqrt(v4dot(qn, qn));
      if (!(m < esc && n[sl] < max_it) || m < T(1.1754943508e-37)) {
        finish(k[sl], qn, L[sl], n[sl]);
        live[sl] = false;
      }
    }
  }
}

// The FP32 form is chosen once per launch (straight-line root loops).
template <class T, bool GRAD>
__global__ void __launch_bounds__(SQF_T) sq_fwd2_kernel(
    const double* __restrict__ params, int nt, int nb, const double* __restrict__ xyz,
    const double* __restrict__ target, long long n_samples, double slice, int max_it,
    double escape, double d_sat, unsigned long long* __restrict__ claim, SqFwdOut<T> o) {
  if constexpr (std::is_same<T, float>::value) {
    if (c_sq_fast) {
      sq_fwd2_body<T, GRAD, SQM_FAST>(params, nt, nb, xyz, target, n_samples, slice, max_it,
                                      escape, d_sat, claim, o);
      return;
    }
  }
  sq_fwd2_body<T, GRAD, SQM_ACC>(params, nt, nb, xyz, target, n_samples, slice, max_it, escape,
                                 d_sat, claim, o);
}

// Per chunk of SQ_CH samples: the energy and the left-out count summed in a
// fixed tree (one partial row per chunk; the backward pass's rows follow, so a
// chunk's row index, and with it the energy's bits, is the same with or
// without the gradient), and
// (gradient pass) the histogram of orbit lengths for the sort, bucket
// max_it - N so that long orbits come first: hist[bucket * nchunks + chunk].
__global__ void __launch_bounds__(SQC_T) sq_chunk_kernel(const double* __restrict__ contrib,
                                                         const int* __restrict__ keys,
                                                         const int* __restrict__ iters,
                                                         long long n, int max_it, int nchunks,
                                                         int* __restrict__ hist,
                                                         double* __restrict__ partials, int slots,
                                                         int row0,
                                                         unsigned long long* __restrict__ work) {
  __shared__ double red_e[SQC_T], red_b[SQC_T];
  __shared__ int h[SQ_MAXIT + 1];
  const int c = blockIdx.x, t = threadIdx.x;
  for (int b = t; b <= max_it; b += SQC_T) h[b] = 0;
  __syncthreads();
  double e = 0.0, bad = 0.0;
  unsigned long long apps = 0, steps = 0;  // map applications (forward), orbit steps (adjoint)
  for (int i = t; i < SQ_CH; i += SQC_T) {
    const long long k = (long long)c * SQ_CH + i;
    if (k >= n) break;
    e += contrib[k];
    apps += (unsigned long long)iters[k];
    if (keys) {
      const int key = keys[k];
      if (key == -2) bad += 1.0;
      else if (key > 0) {
        atomicAdd(&h[max_it - key], 1);
        steps += (unsigned long long)key;
      }
    }
  }
  apps = __reduce_add_sync(0xffffffffu, (unsigned)apps);
  steps = __reduce_add_sync(0xffffffffu, (unsigned)steps);
  if ((t & 31) == 0 && (apps | steps)) {
    atomicAdd(&work[0], apps);
    atomicAdd(&work[1], steps);
  }
  red_e[t] = e;
  red_b[t] = bad;
  __syncthreads();
  for (int w = SQC_T / 2; w; w >>= 1) {
    if (t < w) {
      red_e[t] += red_e[t + w];
      red_b[t] += red_b[t + w];
    }
    __syncthreads();
  }
  double* row = partials + (long long)(row0 + c) * slots;
  for (int j = t; j < slots; j += SQC_T) row[j] = j == 0 ? red_e[0] : j == slots - 1 ? red_b[0] : 0.0;
  if (keys)
    for (int b = t; b <= max_it; b += SQC_T) hist[(long long)b * nchunks + c] = h[b];
}

// Exclusive scan of the histogram in place (one block); *total = entries.
__global__ void __launch_bounds__(1024) sq_scan_kernel(int* __restrict__ hist, long long m,
                                                       int* __restrict__ total) {
  __shared__ int sums[1024];
  const int t = threadIdx.x;
  const long long per = (m + 1023) / 1024, lo = min(m, t * per), hi = min(m, lo + per);
  int own = 0;
  for (long long i = lo; i < hi; i++) own += hist[i];
  sums[t] = own;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int v = t >= off ? sums[t - off] : 0;
    __syncthreads();
    sums[t] += v;
    __syncthreads();
  }
  int run = sums[t] - own;
  for (long long i = lo; i < hi; i++) {
    const int v = hist[i];
    hist[i] = run;
    run += v;
  }
  if (t == 1023) *total = sums[1023];
}

// Stable scatter of the gradient samples into perm, longest orbits first:
// one warp per chunk walks its samples in order; lanes with the same bucket
// take consecutive slots in lane order (__match_any_sync).
__global__ void __launch_bounds__(32) sq_scatter_kernel(const int* __restrict__ keys, long long n,
                                                        int max_it, int nchunks,
                                                        const int* __restrict__ hist,
                                                        unsigned* __restrict__ perm) {
  __shared__ int off[SQ_MAXIT + 1];
  const int c = blockIdx.x, lane = threadIdx.x;
  for (int b = lane; b <= max_it; b += 32) off[b] = hist[(long long)b * nchunks + c];
  __syncwarp();
  const unsigned lt = (1u << lane) - 1u;
  for (int i0 = 0; i0 < SQ_CH; i0 += 32) {
    const long long k = (long long)c * SQ_CH + i0 + lane;
    const int key = k < n ? keys[k] : -1;
    const int b = key > 0 ? max_it - key : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, b);
    const int rank = __popc(grp & lt);
    if (b >= 0) perm[off[b] + rank] = (unsigned)k;
    __syncwarp();
    if (b >= 0 && rank == 0) off[b] += __popc(grp);
    __syncwarp();
  }
}

// Backward pass over the sorted gradient samples: warp w takes groups of 32
// consecutive entries w, w + W, ... (equal orbit lengths within a group but
// at bucket edges, so lanes seldom wait on a longer orbit).  It stores no
// trajectory: from each checkpoint it recomputes the segment forward before
// reversing it.  The steps run warp-uniformly down from the group's longest
// orbit (a lane takes part in the steps below its own length), so that every
// root term's five gradient components are summed over the warp with
// shuffles and added to the warp's double accumulators in shared memory:
// no per-thread gradient array in local memory, and the sums run in a fixed
// order (the gradient is the same on every run).
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <class T, int M>
__device__ __forceinline__ void sq_bwd_body(
    const double* __restrict__ params, int nt, int nb, long long n_samples,
    const unsigned* __restrict__ perm, const int* __restrict__ total,
    const int* __restrict__ keys, const V4<T>* __restrict__ seed_q,
    const T* __restrict__ seed_L, const V4<T>* __restrict__ ck, double* __restrict__ partials,
    int slots) {
  extern __shared__ unsigned char sh_raw[];
  const int nr = nt + nb;
  T* rp = reinterpret_cast<T*>(sh_raw);           // 4 nr
  T* ep = rp + 4 * nr;                            // nr
  double* acc_sh = reinterpret_cast<double*>(sh_raw + ((sizeof(T) * 5 * nr + 15) / 16) * 16);
  for (int k = threadIdx.x; k < 4 * nr; k += SQ_T) rp[k] = (T)params[k];
  for (int k = threadIdx.x; k < nr; k += SQ_T) ep[k] = (T)params[4 * nr + k];
  for (int k = threadIdx.x; k < (SQ_T / 32) * slots; k += SQ_T) acc_sh[k] = 0.0;
  __syncthreads();
  const T s = (T)exp(params[5 * nr]);
  // this warp's sums: acc[1 + 4 i + c] root positions, acc[1 + 4 nr + i]
  // exponents, acc[1 + 5 nr] log s
  double* acc = acc_sh + (threadIdx.x >> 5) * slots;
  // per-thread scratch (local memory)
  V4<T> seg[SQ_CK];
  V4<T> F[QJ_MAX_ROOTS];
  const V4<T> zero{T(0), T(0), T(0), T(0)};
  const int count = *total;
  const int lane = threadIdx.x & 31;
  const long long W = ((long long)gridDim.x * SQ_T) >> 5;
  for (long long grp = ((long long)blockIdx.x * SQ_T + threadIdx.x) >> 5; grp * 32 < count;
       grp += W) {
    const long long j = grp * 32 + lane;
    const bool in = j < count;
    const long long k = in ? (long long)perm[j] : 0;
    const int N = in ? keys[k] : 0;
    V4<T> qb = in ? seed_q[k] : zero;
    const T Lb = in ? seed_L[k] : T(0);
    const int Nmax = __reduce_max_sync(0xffffffffu, N);
    // segments in reverse
    for (int sgi = (Nmax - 1) / SQ_CK; sgi >= 0; sgi--) {
      const int n0 = sgi * SQ_CK, n1 = min(N, n0 + SQ_CK), n1max = min(Nmax, n0 + SQ_CK);
      V4<T> q = n1 > n0 ? ck[(long long)sgi * n_samples + k] : zero;
      for (int n = n0; n < n1; n++) {
        seg[n - n0] = q;
        T lg;
        if (n + 1 < n1)
          q = sq_apply<T, M>(rp, ep, nt, nb, s, q, &lg, nullptr, nullptr, nullptr, nullptr);
      }
      for (int n = n1max - 1; n >= n0; n--) {
        const bool on = n < n1;  // this lane's orbit has step n
        V4<T> qn = zero, Tb = zero, Bb = zero, gb = zero;
        T dls = T(0);
        if (on) {
          qn = seg[n - n0];
          T lg;
          V4<T> Tq, Bq;
          const V4<T> Q = sq_apply<T, M>(rp, ep, nt, nb, s, qn, &lg, F, nullptr, &Tq, &Bq);
          // L_{n+1} = L_n + log|g| + log|Q|
          const V4<T> Qb = v4add(qb, v4scale(Q, sq_div<T, M>(Lb, v4dot(Q, Q))));
          // d/d log s: <Qbar, Q>
          dls = v4dot(Qb, Q);
          if (nb > 0) {
            const V4<T> W4 = v4scale(v4conj(Bq), sq_div<T, M>(T(1), v4dot(Bq, Bq)));
            Tb = v4scale(v4mul(Qb, v4conj(W4)), s);
            const V4<T> Wb = v4scale(v4mul(v4conj(Tq), Qb), s);
            Bb = v4scale(v4mul(v4mul(v4conj(W4), Wb), v4conj(W4)), T(-1));
          } else {
            Tb = v4scale(Qb, s);
          }
          // gradient of log|g| w.r.t. g
          V4<T> g = zero;
          for (int i = 0; i < nr; i++) {
            const V4<T> d{qn.w - rp[4 * i], qn.x - rp[4 * i + 1], qn.y - rp[4 * i + 2],
                          qn.z - rp[4 * i + 3]};
            g = v4add(g, v4scale(d, sq_div<T, M>(i >= nt ? -ep[i] : ep[i], v4dot(d, d))));
          }
          gb = v4scale(g, sq_div<T, M>(Lb, v4dot(g, g)));
        }
        dls = warp_sum(dls);
        if (lane == 0) acc[1 + 5 * nr] += (double)dls;
        V4<T> qbn = zero;
        // products: Pbar_i = conj(F_{i-1}) U, U <- U conj(P_i), from the end
        for (int side = 1; side >= 0; side--) {
          const int lo = side ? nt : 0, hi = side ? nr : nt;
          if (hi == lo) continue;
          V4<T> U = side ? Bb : Tb;
          for (int i = hi - 1; i >= lo; i--) {
            T c0 = T(0), c1 = T(0), c2 = T(0), c3 = T(0), c4 = T(0);
            if (on) {
              const V4<T> d{qn.w - rp[4 * i], qn.x - rp[4 * i + 1], qn.y - rp[4 * i + 2],
                            qn.z - rp[4 * i + 3]};
              PowParts<T> pp;
              const V4<T> P = powv<T, M>(d, ep[i], &pp);
              const V4<T> Pb = (i == lo) ? U : v4mul(v4conj(F[i - 1]), U);
              U = v4mul(U, v4conj(P));
              T eb = T(0);
              V4<T> dbar = powv_vjp<T, M>(d, ep[i], pp, Pb, &eb);
              // g term: sgn e d/|d|^2
              const T sgn = side ? T(-1) : T(1);
              const T d2 = v4dot(d, d);
              const T dg = v4dot(d, gb);
              const T id2 = sq_div<T, M>(T(1), d2);
              dbar = v4add(dbar, v4scale(v4add(v4scale(gb, id2), v4scale(d, T(-2) * dg * id2 * id2)),
                                         sgn * ep[i]));
              eb += sgn * dg * id2;
              c0 = -dbar.w;
              c1 = -dbar.x;
              c2 = -dbar.y;
              c3 = -dbar.z;
              c4 = eb;
              qbn = v4add(qbn, dbar);
            }
            c0 = warp_sum(c0);
            c1 = warp_sum(c1);
            c2 = warp_sum(c2);
            c3 = warp_sum(c3);
            c4 = warp_sum(c4);
            if (lane < 5) {
              const T v = lane == 0 ? c0 : lane == 1 ? c1 : lane == 2 ? c2 : lane == 3 ? c3 : c4;
              acc[1 + (lane < 4 ? 4 * i + lane : 4 * nr + i)] += (double)v;
            }
          }
        }
        if (on) qb = qbn;
      }
    }
  }
  __syncthreads();
  // warps in order (the energy and the left-out count are in the chunk rows)
  for (int k = threadIdx.x; k < slots; k += SQ_T) {
    double v = 0;
    for (int w = 0; w < SQ_T / 32; w++) v += acc_sh[w * slots + k];
    partials[(long long)blockIdx.x * slots + k] = v;
  }
}

// The FP32 form is chosen once per launch (straight-line root loops).
template <class T>
__global__ void __launch_bounds__(SQ_T) sq_bwd_kernel(
    const double* __restrict__ params, int nt, int nb, long long n_samples,
    const unsigned* __restrict__ perm, const int* __restrict__ total,
    const int* __restrict__ keys, const V4<T>* __restrict__ seed_q,
    const T* __restrict__ seed_L, const V4<T>* __restrict__ ck, double* __restrict__ partials,
    int slots) {
  if constexpr (std::is_same<T, float>::value) {
    if (c_sq_fast) {
      sq_bwd_body<T, SQM_FAST>(params, nt, nb, n_samples, perm, total, keys, seed_q, seed_L, ck,
                               partials, slots);
      return;
    }
  }
  sq_bwd_body<T, SQM_ACC>(params, nt, nb, n_samples, perm, total, keys, seed_q, seed_L, ck,
                          partials, slots);
}

// ---- the backward pass with the roots spread over lanes ----
//
// sq_bwd_kernel gives each lane a sample and walks the 80 roots of a step in
// series; the gradient samples are few (the others saturate or escape at
// once), so a few hundred warps run long serial chains and most of the GPU
// idles.  Here a group of G lanes takes one sample and lane l of the group
// owns a contiguous run of at most CT top and CB bottom roots.  A map
// application is a per-lane product of the run's polar powers and a scan of
// those products over the group's lanes in lane order (quaternion products
// do not commute).  The adjoint of root i needs the product of the side's
// factors before it and the conjugate of the product after it:
//   Pbar_i = conj(F_{i-1}) Ubar conj(S_{i+1}),
// F from the group's exclusive prefix times the lane's own factors, S from
// the exclusive suffix.  Each lane sums its own roots' five components in
// FP32 registers over the steps of up to SQ_FLUSH samples and then adds them
// to its group's double accumulators in shared memory; the group sums only
// qbar and the log-gradient vector per step (butterflies, so that every lane
// of the group holds the same bits).  The groups of a warp run their steps
// together down from the warp's longest orbit (the samples are sorted by
// orbit length, so a warp's groups seldom differ); a group whose orbit has
// no step n computes alongside and adds nothing.  Each step starts from the
// forward pass's own q_n: a recomputed orbit, its products taken in this
// order, would drift from the forward's in FP32.
template <class T, int G>
__device__ __forceinline__ V4<T> shfl4_up(const V4<T>& v, int o) {
  return V4<T>{__shfl_up_sync(0xffffffffu, v.w, o, G), __shfl_up_sync(0xffffffffu, v.x, o, G),
               __shfl_up_sync(0xffffffffu, v.y, o, G), __shfl_up_sync(0xffffffffu, v.z, o, G)};
}
template <class T, int G>
__device__ __forceinline__ V4<T> shfl4_down(const V4<T>& v, int o) {
  return V4<T>{__shfl_down_sync(0xffffffffu, v.w, o, G), __shfl_down_sync(0xffffffffu, v.x, o, G),
               __shfl_down_sync(0xffffffffu, v.y, o, G), __shfl_down_sync(0xffffffffu, v.z, o, G)};
}
template <class T, int G>
__device__ __forceinline__ V4<T> shfl4_idx(const V4<T>& v, int src) {
  return V4<T>{__shfl_sync(0xffffffffu, v.w, src, G), __shfl_sync(0xffffffffu, v.x, src, G),
               __shfl_sync(0xffffffffu, v.y, src, G), __shfl_sync(0xffffffffu, v.z, src, G)};
}
template <class T, int G>
__device__ __forceinline__ V4<T> group_sum4(V4<T> v) {
#pragma unroll
  for (int o = G / 2; o; o >>= 1)
    v = v4add(v, V4<T>{__shfl_xor_sync(0xffffffffu, v.w, o, G),
                       __shfl_xor_sync(0xffffffffu, v.x, o, G),
                       __shfl_xor_sync(0xffffffffu, v.y, o, G),
                       __shfl_xor_sync(0xffffffffu, v.z, o, G)});
  return v;
}

// A lane's run of one side's roots (first root a, cnt <= C of them; cnt 0
// for lanes past the side), its factors at the current q, the products of
// the factors of the group's lower lanes (E) and higher lanes (X), the
// side's full product, and the run's gradient sums over the current sample
// (four position components and the exponent per root).
template <class T, int C>
struct SideRun {
  int a, cnt;
  V4<T> P[C];
  V4<T> E, X, tot;
  T acc[C][5];
};

template <class T, int G, int C>
__device__ __forceinline__ void side_init(SideRun<T, C>& r, int lo, int ns, int gl) {
  const int c = (ns + G - 1) / G;
  r.a = lo + gl * c;
  r.cnt = max(0, min(c, ns - gl * c));
#pragma unroll
  for (int j = 0; j < C; j++)
#pragma unroll
    for (int m = 0; m < 5; m++) r.acc[j][m] = T(0);
}

// The side's factors at q, the scans over the group's lanes; the side's
// log-gradient terms added to gp.
template <class T, int G, int C, int M>
__device__ __forceinline__ void side_fwd(const T* __restrict__ rp, const T* __restrict__ ep,
                                         T sgn, int gl, const V4<T>& q, SideRun<T, C>& r,
                                         V4<T>& gp) {
  const V4<T> one{T(1), T(0), T(0), T(0)};
  V4<T> Cp = one;
#pragma unroll
  for (int j = 0; j < C; j++) {
    if (j < r.cnt) {
      const int i = r.a + j;
      const V4<T> d{q.w - rp[4 * i], q.x - rp[4 * i + 1], q.y - rp[4 * i + 2],
                    q.z - rp[4 * i + 3]};
      T r2 = T(0);
      const V4<T> P = powv<T, M>(d, ep[i], nullptr, &r2);
      r.P[j] = P;
      Cp = j ? v4mul(Cp, P) : P;
      bool fast = false;
      if constexpr (std::is_same<T, float>::value) fast = sq_fast<M>();
      // the fast form divides by the polar power's own |d|^2
      gp = v4add(gp, v4scale(d, sq_div<T, M>(sgn * ep[i], fast ? r2 : v4dot(d, d))));
    }
  }
  // inclusive prefix over the group's lanes: x_l = C_0 C_1 ... C_l
  V4<T> x = Cp;
#pragma unroll
  for (int o = 1; o < G; o <<= 1) {
    const V4<T> y = shfl4_up<T, G>(x, o);
    if (gl >= o) x = v4mul(y, x);
  }
  r.tot = shfl4_idx<T, G>(x, G - 1);
  const V4<T> e = shfl4_up<T, G>(x, 1);
  r.E = gl ? e : one;
  // inclusive suffix: z_l = C_l C_{l+1} ... C_{G-1}
  V4<T> z = Cp;
#pragma unroll
  for (int o = 1; o < G; o <<= 1) {
    const V4<T> y = shfl4_down<T, G>(z, o);
    if (gl + o < G) z = v4mul(z, y);
  }
  const V4<T> xx = shfl4_down<T, G>(z, 1);
  r.X = gl < G - 1 ? xx : one;
}

// The side's adjoint at qn given Ubar (the adjoint of its full product) and
// gbar (of the log-gradient vector): each root's terms added to the run's
// sums when `on`, and to qbp (this lane's share of qbar).
template <class T, int C, int M>
__device__ __forceinline__ void side_adj(const T* __restrict__ rp, const T* __restrict__ ep,
                                         T sgn, const V4<T>& qn, SideRun<T, C>& r,
                                         const V4<T>& Ub, const V4<T>& gb, bool on, V4<T>& qbp) {
  // Fa[j] = F_{a+j-1}: the side's factors before root a + j
  V4<T> Fa[C];
  Fa[0] = r.E;
#pragma unroll
  for (int j = 1; j < C; j++)
    if (j < r.cnt) Fa[j] = v4mul(Fa[j - 1], r.P[j - 1]);
  // V = Ubar conj(S_{a+j+1}), walked down from the run's end
  V4<T> V = v4mul(Ub, v4conj(r.X));
#pragma unroll
  for (int j = C - 1; j >= 0; j--) {
    if (j < r.cnt) {
      const int i = r.a + j;
      const V4<T> d{qn.w - rp[4 * i], qn.x - rp[4 * i + 1], qn.y - rp[4 * i + 2],
                    qn.z - rp[4 * i + 3]};
      PowParts<T> pp;
      T r2 = T(0);
      powv<T, M>(d, ep[i], &pp, &r2);
      const V4<T> Pb = v4mul(v4conj(Fa[j]), V);
      V = v4mul(V, v4conj(r.P[j]));
      T eb = T(0);
      V4<T> dbar = powv_vjp<T, M>(d, ep[i], pp, Pb, &eb);
      // g term: sgn e d/|d|^2
      bool fast = false;
      if constexpr (std::is_same<T, float>::value) fast = sq_fast<M>();
      const T d2 = fast ? r2 : v4dot(d, d);
      const T dg = v4dot(d, gb);
      const T id2 = sq_div<T, M>(T(1), d2);
      dbar = v4add(dbar, v4scale(v4add(v4scale(gb, id2), v4scale(d, T(-2) * dg * id2 * id2)),
                                 sgn * ep[i]));
      eb += sgn * dg * id2;
      if (on) {
        r.acc[j][0] -= dbar.w;
        r.acc[j][1] -= dbar.x;
        r.acc[j][2] -= dbar.y;
        r.acc[j][3] -= dbar.z;
        r.acc[j][4] += eb;
      }
      qbp = v4add(qbp, dbar);
    }
  }
}

// The run's register sums into the group's accumulators (and reset).
template <class T, int C>
__device__ __forceinline__ void side_flush(SideRun<T, C>& r, double* acc, int nr) {
#pragma unroll
  for (int j = 0; j < C; j++) {
    if (j < r.cnt) {
      const int i = r.a + j;
#pragma unroll
      for (int m = 0; m < 4; m++) acc[1 + 4 * i + m] += (double)r.acc[j][m];
      acc[1 + 4 * nr + i] += (double)r.acc[j][4];
    }
#pragma unroll
    for (int m = 0; m < 5; m++) r.acc[j][m] = T(0);
  }
}

static_assert(SQ_CK == 1, "sq_bwd_roots_kernel reads the forward pass's q at every step");
constexpr int SQ_FLUSH = 16;  // samples a lane sums in FP32 before adding to the double sums

template <class T, int G, int CT, int CB, int M>
__device__ __forceinline__ void sq_bwd_roots_body(
    const double* __restrict__ params, int nt, int nb, long long n_samples,
    const unsigned* __restrict__ perm, const int* __restrict__ total,
    const int* __restrict__ keys, const V4<T>* __restrict__ seed_q,
    const T* __restrict__ seed_L, const V4<T>* __restrict__ ck, double* __restrict__ partials,
    int slots) {
  constexpr int NG = SQ_T / G;  // groups per block
  extern __shared__ unsigned char sh_raw[];
  const int nr = nt + nb;
  T* rp = reinterpret_cast<T*>(sh_raw);  // 4 nr
  T* ep = rp + 4 * nr;                   // nr
  double* acc_sh = reinterpret_cast<double*>(sh_raw + ((sizeof(T) * 5 * nr + 15) / 16) * 16);
  for (int k = threadIdx.x; k < 4 * nr; k += SQ_T) rp[k] = (T)params[k];
  for (int k = threadIdx.x; k < nr; k += SQ_T) ep[k] = (T)params[4 * nr + k];
  for (int k = threadIdx.x; k < NG * slots; k += SQ_T) acc_sh[k] = 0.0;
  __syncthreads();
  const T s = (T)exp(params[5 * nr]);
  const int lane = threadIdx.x & 31, gl = lane & (G - 1);
  // this group's sums: acc[1 + 4 i + c] root positions, acc[1 + 4 nr + i]
  // exponents, acc[1 + 5 nr] log s
  double* acc = acc_sh + (threadIdx.x / G) * slots;
  SideRun<T, CT> top;
  SideRun<T, CB> bot;
  side_init<T, G, CT>(top, 0, nt, gl);
  side_init<T, G, CB>(bot, nt, nb, gl);
  const V4<T> zero{T(0), T(0), T(0), T(0)};
  const int count = *total;
  const long long stride = (long long)gridDim.x * NG;
  T dls = T(0);
  int since = 0;  // samples summed in registers since the last flush
  // the warp's first group in the sorted list; its groups take consecutive entries
  for (long long base = ((long long)blockIdx.x * SQ_T + (threadIdx.x & ~31)) / G; base < count;
       base += stride) {
    const long long j = base + lane / G;
    const bool in = j < count;
    const long long k = in ? (long long)perm[j] : 0;
    const int N = in ? keys[k] : 0;
    V4<T> qb = in ? seed_q[k] : zero;
    const T Lb = in ? seed_L[k] : T(0);
    const int Nmax = __reduce_max_sync(0xffffffffu, N);
    for (int n = Nmax - 1; n >= 0; n--) {
      const bool on = n < N;  // this group's orbit has step n
      // the forward pass's own q_n (SQ_CK = 1)
      const V4<T> qn = on ? ck[(long long)n * n_samples + k] : zero;
      V4<T> gp = zero;
      side_fwd<T, G, CT, M>(rp, ep, T(1), gl, qn, top, gp);
      side_fwd<T, G, CB, M>(rp, ep, T(-1), gl, qn, bot, gp);
      const V4<T> g = group_sum4<T, G>(gp);
      V4<T> Q, Tb, Bb;
      if (nb > 0) {
        const V4<T> W4 = v4scale(v4conj(bot.tot), sq_div<T, M>(T(1), v4dot(bot.tot, bot.tot)));
        Q = v4scale(v4mul(top.tot, W4), s);
        // L_{n+1} = L_n + log|g| + log|Q|
        const V4<T> Qb = v4add(qb, v4scale(Q, sq_div<T, M>(Lb, v4dot(Q, Q))));
        if (on) dls += v4dot(Qb, Q);
        Tb = v4scale(v4mul(Qb, v4conj(W4)), s);
        const V4<T> Wb = v4scale(v4mul(v4conj(top.tot), Qb), s);
        Bb = v4scale(v4mul(v4mul(v4conj(W4), Wb), v4conj(W4)), T(-1));
      } else {
        Q = v4scale(top.tot, s);
        const V4<T> Qb = v4add(qb, v4scale(Q, sq_div<T, M>(Lb, v4dot(Q, Q))));
        if (on) dls += v4dot(Qb, Q);
        Tb = v4scale(Qb, s);
        Bb = zero;
      }
      const V4<T> gb = v4scale(g, sq_div<T, M>(Lb, v4dot(g, g)));
      V4<T> qbp = zero;
      side_adj<T, CT, M>(rp, ep, T(1), qn, top, Tb, gb, on, qbp);
      side_adj<T, CB, M>(rp, ep, T(-1), qn, bot, Bb, gb, on, qbp);
      qbp = group_sum4<T, G>(qbp);
      if (on) qb = qbp;
    }
    // most gradient samples run one or two steps, so a flush per sample (25
    // FP64 additions and conversions per lane) kept the FP64 pipe 41% busy
    // and took 40% of the kernel; sums of at most SQ_FLUSH samples stay in
    // FP32 registers
    if (++since == SQ_FLUSH) {
      side_flush<T, CT>(top, acc, nr);
      side_flush<T, CB>(bot, acc, nr);
      if (gl == 0) acc[1 + 5 * nr] += (double)dls;
      dls = T(0);
      since = 0;
    }
  }
  side_flush<T, CT>(top, acc, nr);
  side_flush<T, CB>(bot, acc, nr);
  if (gl == 0) acc[1 + 5 * nr] += (double)dls;
  __syncthreads();
  // groups in order (the energy and the left-out count are in the chunk rows)
  for (int k = threadIdx.x; k < slots; k += SQ_T) {
    double v = 0;
    for (int w = 0; w < NG; w++) v += acc_sh[w * slots + k];
    partials[(long long)blockIdx.x * slots + k] = v;
  }
}

// The FP32 form is chosen once per launch (straight-line root loops).
template <class T, int G, int CT, int CB, int MINB>
__global__ void __launch_bounds__(SQ_T, MINB) sq_bwd_roots_kernel(
    const double* __restrict__ params, int nt, int nb, long long n_samples,
    const unsigned* __restrict__ perm, const int* __restrict__ total,
    const int* __restrict__ keys, const V4<T>* __restrict__ seed_q,
    const T* __restrict__ seed_L, const V4<T>* __restrict__ ck, double* __restrict__ partials,
    int slots) {
  if (c_sq_fast)
    sq_bwd_roots_body<T, G, CT, CB, SQM_FAST>(params, nt, nb, n_samples, perm, total, keys,
                                              seed_q, seed_L, ck, partials, slots);
  else
    sq_bwd_roots_body<T, G, CT, CB, SQM_ACC>(params, nt, nb, n_samples, perm, total, keys,
                                             seed_q, seed_L, ck, partials, slots);
}

// Compensated sum of partials[b][k] over rows b, one block of SQR_W warps
// per slot k: each thread a Neumaier sum over rows t, t + 32 SQR_W, ...,
// each warp's 32 (sum, compensation) pairs in a fixed tree, then the warps'
// pairs in order, so the result is the same on every run.  The sums are
// FP64-bound, so they are spread over many warps (one warp per slot in
// 256-thread blocks: 30 us for 1 000 rows x 403 slots).
constexpr int SQR_W = 4;

__device__ __forceinline__ void neumaier_add(double& sum, double& c, double v) {
  const double t = sum + v;
  c += (fabs(sum) >= fabs(v)) ? (sum - t) + v : (v - t) + sum;
  sum = t;
}

__device__ __forceinline__ void reduce_slot(const double* __restrict__ partials, int rows,
                                            int slots, int k, double* __restrict__ out) {
  __shared__ double ws[SQR_W], wc[SQR_W];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double sum = 0, c = 0;
  for (int b = threadIdx.x; b < rows; b += 32 * SQR_W)
    neumaier_add(sum, c, partials[(long long)b * slots + k]);
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const double s2 = __shfl_down_sync(0xffffffffu, sum, o);
    const double c2 = __shfl_down_sync(0xffffffffu, c, o);
    c += c2;
    neumaier_add(sum, c, s2);
  }
  if (lane == 0) {
    ws[w] = sum;
    wc[w] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = ws[0], c0 = wc[0];
    for (int i = 1; i < SQR_W; i++) {
      c0 += wc[i];
      neumaier_add(s0, c0, ws[i]);
    }
    out[k] = s0 + c0;
  }
}

__global__ void __launch_bounds__(32 * SQR_W) sq_reduce_kernel(const double* __restrict__ partials,
                                                               int rows, int slots,
                                                               double* __restrict__ out) {
  reduce_slot(partials, rows, slots, blockIdx.x, out);
}

// ---- batches of energy + gradient requests (FP32), one pass for all.
// Items' samples sit in one flat index space, each item's range starting on
// a chunk boundary (SQ_CH), so that a chunk belongs to one item.  The
// forward pass is the refill kernel over the flat space: a lane finds its
// sample's item from the chunk table and reads that item's roots (FP32,
// converted once) from global memory.  Chunk sums, the orbit-length sort and
// the final reduction run per item; the adjoint's warps walk every item's
// sorted groups in turn and write one partial row per group, so each item's
// energy and gradient are sums in a fixed order.
struct SqItem {
  const double* xyz;     // the item's samples (n x 3) and targets
  const double* target;
  const float* rp;       // the item's roots (4 nr) then exponents (nr), FP32
  const double* params;  // the item's parameter vector (for log s)
  int nt, nb, max_it, slots;
  double slice, escape, d_sat;
  long long s0, n;       // first flat sample, samples
  long long c0;          // first chunk
  long long rows0;       // first partial row: the item's chunks, then its groups
  int* total;            // the item's gradient samples (the sort's count)
  unsigned* perm;        // the item's sorted gradient samples (local indices)
  double* partials;      // the item's partial rows
};

__global__ void sq_item_roots_kernel(const SqItem* __restrict__ items, int K) {
  const SqItem& it = items[blockIdx.x];
  const int nr = it.nt + it.nb;
  float* rp = const_cast<float*>(it.rp);
  for (int k = threadIdx.x; k < 5 * nr; k += blockDim.x) rp[k] = (float)it.params[k];
  (void)K;
}

template <int M>
__device__ __forceinline__ void sq_fwd_batch_body(
    const SqItem* __restrict__ items, const int* __restrict__ chunk_item, long long n_flat,
    unsigned long long* __restrict__ claim, SqFwdOut<float> o) {
  using T = float;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  long long k = 0;       // flat sample
  int item = -1;
  bool live = false, done = false;
  V4<T> q{T(0), T(0), T(0), T(0)};
  T L = T(0);
  int n = 0;
  const SqItem* it = nullptr;
  auto finish = [&](long long kf, const V4<T>& qf, T Lf, int nf) {
    const long long kl = kf - it->s0;
    const T m = sqrt(v4dot(qf, qf));
    const T lm = log(m);
    const T ld = log(fabs(lm)) + lm - Lf;
    o.iters[kf] = nf;
    T val, dval, dval_dd;
    sq_saturate<T>(lm, ld, (T)it->d_sat, &val, &dval, &dval_dd);
    const T r = val - (T)it->target[kl];
    o.contrib[kf] = (double)(r * r);
    int key = -1;
    if (dval_dd != T(0)) {
      const T db = T(2) * r * dval_dd;
      const T kq = db * (lm + T(1)) * exp(ld - log(m) - log(fabs(lm)));
      if (!isfinite(kq) || !isfinite(db * dval)) {
        key = -2;
      } else if (nf > 0) {
        o.seed_q[kf] = v4scale(qf, kq / m);
        o.seed_L[kf] = -db * dval;
        key = nf;
      }
    }
    o.keys[kf] = key;
  };
  for (;;) {
    unsigned want = __ballot_sync(0xffffffffu, !live && !done);
    while (want) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(claim, (unsigned long long)__popc(want));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (!live && !done) {
        k = (long long)(base + __popc(want & lt));
        if (k >= n_flat) {
          done = true;
        } else {
          item = chunk_item[k / SQ_CH];
          it = &items[item];
          if (k - it->s0 < it->n) {  // not the padding after the item's samples
            const long long kl = k - it->s0;
            q = V4<T>{(T)it->xyz[3 * kl], (T)it->xyz[3 * kl + 1], (T)it->xyz[3 * kl + 2],
                      (T)it->slice};
            L = T(0);
            n = 0;
            if (sqrt(v4dot(q, q)) < (T)it->escape && n < it->max_it)
              live = true;
            else
              finish(k, q, L, n);
          }
        }
      }
      want = __ballot_sync(0xffffffffu, !live && !done);
    }
    if (!__any_sync(0xffffffffu, live)) break;
    if (live) {
      if (n % SQ_CK == 0) o.ck[(long long)(n / SQ_CK) * n_flat + k] = q;
      const int nr = it->nt + it->nb;
      const T s = (T)exp(it->params[5 * nr]);
      T lg;
      q = sq_apply<T, M>(it->rp, it->rp + 4 * nr, it->nt, it->nb, s, q, &lg, nullptr, nullptr,
                      nullptr, nullptr);
      L += lg + T(0.5) * log(v4dot(q, q));
      n++;
      const T m = sqrt(v4dot(q, q));
      if (!(m < (T)it->escape && n < it->max_it) || m < T(1.1754943508e-37)) {
        finish(k, q, L, n);
        live = false;
      }
    }
  }
}

// The FP32 form is chosen once per launch (straight-line root loops).
__global__ void __launch_bounds__(SQF_T) sq_fwd_batch_kernel(
    const SqItem* __restrict__ items, const int* __restrict__ chunk_item, long long n_flat,
    unsigned long long* __restrict__ claim, SqFwdOut<float> o) {
  if (c_sq_fast)
    sq_fwd_batch_body<SQM_FAST>(items, chunk_item, n_flat, claim, o);
  else
    sq_fwd_batch_body<SQM_ACC>(items, chunk_item, n_flat, claim, o);
}

// The adjoint of a batch: warp w takes groups w, w + W, ... of item 0, then
// of item 1, and so on (the items' sorted gradient samples in groups of 32);
// per group it sums the root terms' gradient components over the warp into
// shared double accumulators as sq_bwd_kernel does and writes them as the
// group's partial row.
template <int M>
__device__ __forceinline__ void sq_bwd_batch_body(
    const SqItem* __restrict__ items, int K, long long n_flat, const int* __restrict__ keys,
    const V4<float>* __restrict__ seed_q, const float* __restrict__ seed_L,
    const V4<float>* __restrict__ ck, int max_slots) {
  using T = float;
  extern __shared__ unsigned char sh_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double* acc = reinterpret_cast<double*>(sh_raw) + (size_t)warp * max_slots;
  V4<T> seg[SQ_CK];
  V4<T> F[QJ_MAX_ROOTS];
  const V4<T> zero{T(0), T(0), T(0), T(0)};
  const long long W = ((long long)gridDim.x * SQ_T) >> 5;
  const long long w0 = ((long long)blockIdx.x * SQ_T + threadIdx.x) >> 5;
  for (int item = 0; item < K; item++) {
    const SqItem& it = items[item];
    const int nt = it.nt, nb = it.nb, nr = nt + nb, slots = it.slots;
    const T* rp = it.rp;
    const T* ep = it.rp + 4 * nr;
    const T s = (T)exp(it.params[5 * nr]);
    const int count = *it.total;
    const long long nchunks = (it.n + SQ_CH - 1) / SQ_CH;
    for (long long grp = w0; grp * 32 < count; grp += W) {
      for (int j = lane; j < slots; j += 32) acc[j] = 0.0;
      __syncwarp();
      const long long j = grp * 32 + lane;
      const bool in = j < count;
      const long long k = in ? it.s0 + (long long)it.perm[j] : 0;  // flat index
      const int N = in ? keys[k] : 0;
      V4<T> qb = in ? seed_q[k] : zero;
      const T Lb = in ? seed_L[k] : T(0);
      const int Nmax = __reduce_max_sync(0xffffffffu, N);
      for (int sgi = (Nmax - 1) / SQ_CK; sgi >= 0; sgi--) {
        const int n0 = sgi * SQ_CK, n1 = min(N, n0 + SQ_CK), n1max = min(Nmax, n0 + SQ_CK);
        V4<T> q = n1 > n0 ? ck[(long long)sgi * n_flat + k] : zero;
        for (int n = n0; n < n1; n++) {
          seg[n - n0] = q;
          T lg;
          if (n + 1 < n1)
            q = sq_apply<T, M>(rp, ep, nt, nb, s, q, &lg, nullptr, nullptr, nullptr, nullptr);
        }
        for (int n = n1max - 1; n >= n0; n--) {
          const bool on = n < n1;
          V4<T> qn = zero, Tb = zero, Bb = zero, gb = zero;
          T dls = T(0);
          if (on) {
            qn = seg[n - n0];
            T lg;
            V4<T> Tq, Bq;
            const V4<T> Q = sq_apply<T, M>(rp, ep, nt, nb, s, qn, &lg, F, nullptr, &Tq, &Bq);
            const V4<T> Qb = v4add(qb, v4scale(Q, sq_div<T, M>(Lb, v4dot(Q, Q))));
            dls = v4dot(Qb, Q);
            if (nb > 0) {
              const V4<T> W4 = v4scale(v4conj(Bq), sq_div<T, M>(T(1), v4dot(Bq, Bq)));
              Tb = v4scale(v4mul(Qb, v4conj(W4)), s);
              const V4<T> Wb = v4scale(v4mul(v4conj(Tq), Qb), s);
              Bb = v4scale(v4mul(v4mul(v4conj(W4), Wb), v4conj(W4)), T(-1));
            } else {
              Tb = v4scale(Qb, s);
            }
            V4<T> g = zero;
            for (int i = 0; i < nr; i++) {
              const V4<T> d{qn.w - rp[4 * i], qn.x - rp[4 * i + 1], qn.y - rp[4 * i + 2],
                            qn.z - rp[4 * i + 3]};
              g = v4add(g, v4scale(d, sq_div<T, M>(i >= nt ? -ep[i] : ep[i], v4dot(d, d))));
            }
            gb = v4scale(g, sq_div<T, M>(Lb, v4dot(g, g)));
          }
          dls = warp_sum(dls);
          if (lane == 0) acc[1 + 5 * nr] += (double)dls;
          V4<T> qbn = zero;
          for (int side = 1; side >= 0; side--) {
            const int lo = side ? nt : 0, hi = side ? nr : nt;
            if (hi == lo) continue;
            V4<T> U = side ? Bb : Tb;
            for (int i = hi - 1; i >= lo; i--) {
              T c0 = T(0), c1 = T(0), c2 = T(0), c3 = T(0), c4 = T(0);
              if (on) {
                const V4<T> d{qn.w - rp[4 * i], qn.x - rp[4 * i + 1], qn.y - rp[4 * i + 2],
                              qn.z - rp[4 * i + 3]};
                PowParts<T> pp;
                const V4<T> P = powv<T, M>(d, ep[i], &pp);
                const V4<T> Pb = (i == lo) ? U : v4mul(v4conj(F[i - 1]), U);
                U = v4mul(U, v4conj(P));
                T eb = T(0);
                V4<T> dbar = powv_vjp<T, M>(d, ep[i], pp, Pb, &eb);
                const T sgn = side ? T(-1) : T(1);
                const T d2 = v4dot(d, d);
                const T dg = v4dot(d, gb);
                const T id2 = sq_div<T, M>(T(1), d2);
                dbar = v4add(dbar, v4scale(v4add(v4scale(gb, id2),
                                                 v4scale(d, T(-2) * dg * id2 * id2)),
                                           sgn * ep[i]));
                eb += sgn * dg * id2;
                c0 = -dbar.w;
                c1 = -dbar.x;
                c2 = -dbar.y;
                c3 = -dbar.z;
                c4 = eb;
                qbn = v4add(qbn, dbar);
              }
              c0 = warp_sum(c0);
              c1 = warp_sum(c1);
              c2 = warp_sum(c2);
              c3 = warp_sum(c3);
              c4 = warp_sum(c4);
              if (lane < 5) {
                const T v = lane == 0 ? c0 : lane == 1 ? c1 : lane == 2 ? c2 : lane == 3 ? c3 : c4;
                acc[1 + (lane < 4 ? 4 * i + lane : 4 * nr + i)] += (double)v;
              }
            }
          }
          if (on) qb = qbn;
        }
      }
      __syncwarp();
      double* row = it.partials + (nchunks + grp) * slots;
      for (int jj = lane; jj < slots; jj += 32) row[jj] = acc[jj];
      __syncwarp();
    }
  }
}

// The FP32 form is chosen once per launch (straight-line root loops).
__global__ void __launch_bounds__(SQ_T) sq_bwd_batch_kernel(
    const SqItem* __restrict__ items, int K, long long n_flat, const int* __restrict__ keys,
    const V4<float>* __restrict__ seed_q, const float* __restrict__ seed_L,
    const V4<float>* __restrict__ ck, int max_slots) {
  if (c_sq_fast)
    sq_bwd_batch_body<SQM_FAST>(items, K, n_flat, keys, seed_q, seed_L, ck, max_slots);
  else
    sq_bwd_batch_body<SQM_ACC>(items, K, n_flat, keys, seed_q, seed_L, ck, max_slots);
}

// The adjoint of a batch with the roots of a step spread over groups of G
// lanes, as sq_bwd_roots_kernel: the blocks take the items one after the
// other; per item each block stages the item's roots in shared memory, its
// groups take the item's sorted gradient samples (flat indices s0 + perm[j])
// and the block writes one partial row after the item's chunk rows (rows
// nchunks + blockIdx.x), so an item's rows are its chunks plus gridDim.x.
constexpr int SQB_ROOT_BYTES = ((5 * QJ_MAX_ROOTS * (int)sizeof(float) + 15) / 16) * 16;

template <int G, int CT, int CB, int M>
__device__ __forceinline__ void sq_bwd_batch_roots_body(
    const SqItem* __restrict__ items, int K, long long n_flat, const int* __restrict__ keys,
    const V4<float>* __restrict__ seed_q, const float* __restrict__ seed_L,
    const V4<float>* __restrict__ ck) {
  using T = float;
  constexpr int NG = SQ_T / G;  // groups per block
  extern __shared__ unsigned char sh_raw[];
  T* rp = reinterpret_cast<T*>(sh_raw);  // 4 nr roots, then nr exponents
  double* acc_sh = reinterpret_cast<double*>(sh_raw + SQB_ROOT_BYTES);
  const int lane = threadIdx.x & 31, gl = lane & (G - 1);
  const V4<T> zero{T(0), T(0), T(0), T(0)};
  const long long stride = (long long)gridDim.x * NG;
  for (int item = 0; item < K; item++) {
    const SqItem& it = items[item];
    const int nt = it.nt, nb = it.nb, nr = nt + nb, slots = it.slots;
    const T* ep = rp + 4 * nr;
    __syncthreads();  // the previous item's roots and sums are read
    for (int k = threadIdx.x; k < 5 * nr; k += SQ_T) rp[k] = it.rp[k];
    for (int k = threadIdx.x; k < NG * slots; k += SQ_T) acc_sh[k] = 0.0;
    __syncthreads();
    const T s = (T)exp(it.params[5 * nr]);
    double* acc = acc_sh + (threadIdx.x / G) * slots;
    SideRun<T, CT> top;
    SideRun<T, CB> bot;
    side_init<T, G, CT>(top, 0, nt, gl);
    side_init<T, G, CB>(bot, nt, nb, gl);
    const int count = *it.total;
    T dls = T(0);
    int since = 0;
    for (long long base = ((long long)blockIdx.x * SQ_T + (threadIdx.x & ~31)) / G; base < count;
         base += stride) {
      const long long j = base + lane / G;
      const bool in = j < count;
      const long long k = in ? it.s0 + (long long)it.perm[j] : 0;  // flat index
      const int N = in ? keys[k] : 0;
      V4<T> qb = in ? seed_q[k] : zero;
      const T Lb = in ? seed_L[k] : T(0);
      const int Nmax = __reduce_max_sync(0xffffffffu, N);
      for (int n = Nmax - 1; n >= 0; n--) {
        const bool on = n < N;
        const V4<T> qn = on ? ck[(long long)n * n_flat + k] : zero;
        V4<T> gp = zero;
        side_fwd<T, G, CT, M>(rp, ep, T(1), gl, qn, top, gp);
        side_fwd<T, G, CB, M>(rp, ep, T(-1), gl, qn, bot, gp);
        const V4<T> g = group_sum4<T, G>(gp);
        V4<T> Tb, Bb;
        if (nb > 0) {
          const V4<T> W4 =
              v4scale(v4conj(bot.tot), sq_div<T, M>(T(1), v4dot(bot.tot, bot.tot)));
          const V4<T> Q = v4scale(v4mul(top.tot, W4), s);
          const V4<T> Qb = v4add(qb, v4scale(Q, sq_div<T, M>(Lb, v4dot(Q, Q))));
          if (on) dls += v4dot(Qb, Q);
          Tb = v4scale(v4mul(Qb, v4conj(W4)), s);
          const V4<T> Wb = v4scale(v4mul(v4conj(top.tot), Qb), s);
          Bb = v4scale(v4mul(v4mul(v4conj(W4), Wb), v4conj(W4)), T(-1));
        } else {
          const V4<T> Q = v4scale(top.tot, s);
          const V4<T> Qb = v4add(qb, v4scale(Q, sq_div<T, M>(Lb, v4dot(Q, Q))));
          if (on) dls += v4dot(Qb, Q);
          Tb = v4scale(Qb, s);
          Bb = zero;
        }
        const V4<T> gb = v4scale(g, sq_div<T, M>(Lb, v4dot(g, g)));
        V4<T> qbp = zero;
        side_adj<T, CT, M>(rp, ep, T(1), qn, top, Tb, gb, on, qbp);
        side_adj<T, CB, M>(rp, ep, T(-1), qn, bot, Bb, gb, on, qbp);
        qbp = group_sum4<T, G>(qbp);
        if (on) qb = qbp;
      }
      if (++since == SQ_FLUSH) {
        side_flush<T, CT>(top, acc, nr);
        side_flush<T, CB>(bot, acc, nr);
        if (gl == 0) acc[1 + 5 * nr] += (double)dls;
        dls = T(0);
        since = 0;
      }
    }
    side_flush<T, CT>(top, acc, nr);
    side_flush<T, CB>(bot, acc, nr);
    if (gl == 0) acc[1 + 5 * nr] += (double)dls;
    __syncthreads();
    const long long nchunks = max(1LL, (it.n + SQ_CH - 1) / SQ_CH);
    double* row = it.partials + (nchunks + blockIdx.x) * slots;
    for (int k = threadIdx.x; k < slots; k += SQ_T) {
      double v = 0;
      for (int w = 0; w < NG; w++) v += acc_sh[w * slots + k];
      row[k] = v;
    }
  }
}

// The FP32 form is chosen once per launch (straight-line root loops).
template <int G, int CT, int CB, int MINB>
__global__ void __launch_bounds__(SQ_T, MINB) sq_bwd_batch_roots_kernel(
    const SqItem* __restrict__ items, int K, long long n_flat, const int* __restrict__ keys,
    const V4<float>* __restrict__ seed_q, const float* __restrict__ seed_L,
    const V4<float>* __restrict__ ck) {
  if (c_sq_fast)
    sq_bwd_batch_roots_body<G, CT, CB, SQM_FAST>(items, K, n_flat, keys, seed_q, seed_L, ck);
  else
    sq_bwd_batch_roots_body<G, CT, CB, SQM_ACC>(items, K, n_flat, keys, seed_q, seed_L, ck);
}

// The final sums of one item: its chunk rows and as many group rows as its
// sort produced (read on the device), as sq_reduce_kernel.
__global__ void __launch_bounds__(32 * SQR_W) sq_reduce_item_kernel(
    const double* __restrict__ partials, int chunk_rows, const int* __restrict__ total, int slots,
    double* __restrict__ out) {
  reduce_slot(partials, chunk_rows + (*total + 31) / 32, slots, blockIdx.x, out);
}

// Forward kernel choice (qjg_set_energy_pairs): two samples per lane or one.
std::atomic<int> g_sq_pairs{0};
// Forward blocks per SM (qjg_set_energy_forward_blocks): 0 the rule in
// sq_launch, else that many (capped by residency), for sweeps.
std::atomic<int> g_sq_fwd_blocks{0};

// FP32 adjoint choice (qjg_set_energy_adjoint_roots): the roots of a step
// spread over a group of lanes (sq_bwd_roots_kernel) or walked by one lane.
std::atomic<int> g_sq_bwd_roots{1};

// Byte layout of the energy scratch (each piece 256-byte aligned).
struct SqLayout {
  size_t claim, work, total, contrib, keys, iters, perm, hist, seed_q, seed_L, ck, partials, out,
      bytes;
  int nchunks, nbwd, nck, slots;
};

SqLayout sq_layout(bool fp64, bool grad, long long n, int max_it, int nt, int nb, int sms) {
  SqLayout L{};
  const size_t el = fp64 ? sizeof(double) : sizeof(float);
  L.slots = 1 + 5 * (nt + nb) + 1 + 1;  // energy, gradient, left-out samples
  L.nchunks = (int)std::max<long long>(1, (n + SQ_CH - 1) / SQ_CH);
  L.nbwd = grad ? sms * SQ_BWD_PER_SM : 0;
  L.nck = max_it > 0 ? (max_it - 1) / SQ_CK + 1 : 0;
  size_t at = 0;
  auto take = [&](size_t b) {
    const size_t o = at;
    at += (b + 255) / 256 * 256;
    return o;
  };
  const size_t nn = (size_t)std::max<long long>(n, 0);
  L.claim = take(sizeof(unsigned long long));
  L.work = take(2 * sizeof(unsigned long long));
  L.total = take(sizeof(int));
  L.contrib = take(sizeof(double) * nn);
  L.keys = take(sizeof(int) * nn);
  L.iters = take(sizeof(int) * nn);
  if (grad) {
    L.perm = take(sizeof(unsigned) * nn);
    L.hist = take(sizeof(int) * (size_t)(max_it + 1) * L.nchunks);
    L.seed_q = take(4 * el * nn);
    L.seed_L = take(el * nn);
    L.ck = take(4 * el * nn * L.nck);
  }
  L.partials = take(sizeof(double) * (size_t)(L.nbwd + L.nchunks) * L.slots);
  L.out = take(sizeof(double) * L.slots);
  L.bytes = at;
  return L;
}

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

// The root-group adjoint on as many blocks as stay resident (at most the
// layout's L.nbwd rows of partials): a second wave of blocks would start its
// long orbits only as blocks of the first wave end.
template <int G, int CT, int CB, int MINB>
cudaError_t launch_bwd_roots(size_t sh_r, const SqLayout& L, int sms, const double* params, int nt,
                             int nb, long long n, const unsigned* perm, const int* total,
                             const SqFwdOut<float>& o, double* rows, int* blocks, cudaStream_t s) {
  const size_t sh = sh_r + sizeof(double) * (SQ_T / G) * L.slots;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, sq_bwd_roots_kernel<float, G, CT, CB, MINB>, SQ_T, sh);
  if (e != cudaSuccess) return e;
  *blocks = std::max(1, std::min(L.nbwd, std::max(per_sm, 1) * sms));
  sq_bwd_roots_kernel<float, G, CT, CB, MINB><<<*blocks, SQ_T, sh, s>>>(
      params, nt, nb, n, perm, total, o.keys, o.seed_q, o.seed_L, o.ck, rows, L.slots);
  return cudaGetLastError();
}

template <class T>
cudaError_t sq_launch(bool grad, const double* params, int nt, int nb, const double* xyz,
                      const double* target, long long n, double slice, int max_it, double escape,
                      double d_sat, unsigned char* scr, const SqLayout& L, int* iters, int sms,
                      cudaStream_t s, int* launches, long long steps_hint) {
  const int nr = nt + nb;
  unsigned long long* claim = reinterpret_cast<unsigned long long*>(scr + L.claim);
  int* total = reinterpret_cast<int*>(scr + L.total);
  double* partials = reinterpret_cast<double*>(scr + L.partials);
  SqFwdOut<T> o{};
  o.contrib = reinterpret_cast<double*>(scr + L.contrib);
  o.keys = reinterpret_cast<int*>(scr + L.keys);
  o.iters = iters ? iters : reinterpret_cast<int*>(scr + L.iters);
  unsigned long long* work = reinterpret_cast<unsigned long long*>(scr + L.work);
  if (grad) {
    o.seed_q = reinterpret_cast<V4<T>*>(scr + L.seed_q);
    o.seed_L = reinterpret_cast<T*>(scr + L.seed_L);
    o.ck = reinterpret_cast<V4<T>*>(scr + L.ck);
  }
  cudaError_t e = cudaMemsetAsync(claim, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(work, 0, 2 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  const size_t sh_roots = sizeof(T) * 5 * nr;
  // persistent forward grid: as many blocks as stay resident
  int per_sm = 0;
  if (grad)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sq_fwd_kernel<T, true>, SQF_T, sh_roots);
  else
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sq_fwd_kernel<T, false>, SQF_T, sh_roots);
  if (e != cudaSuccess) return e;
  // Blocks per SM.  The kernel ends when the lane with the most orbit steps
  // ends, so the grid is sized from the orbit steps of the call: with as
  // many lanes as total steps / max_it, a lane runs about one full-length
  // orbit (or its equivalent in short ones) and no lane is left with two
  // full-length orbits, while each extra warp costs issue slots.  On the
  // differentiation workload (200k samples, 30 iterations, 3.06 M steps,
  // 49% of the orbits at the cap; forward kernel, ms) 2 blocks per SM 1.22,
  // 3 0.96, 4 1.01, 5 0.96, 6 0.83, 8 1.03: 6 is the first count with a lane
  // per full-length orbit.  The steps are those of an earlier call on the
  // same samples (steps_hint), else half the iteration cap per sample (a
  // lane per two samples); at least 3 blocks per SM.  FP64 (bound by the
  // FP64 pipe rather than by the longest lane) keeps about four samples per
  // lane.
  const long long lanes_per_sm = (long long)sms * SQF_T;
  const int fixed = g_sq_fwd_blocks.load(std::memory_order_relaxed);
  long long want = std::max<long long>(3, ((n + 3) / 4 + lanes_per_sm - 1) / lanes_per_sm);
  if (fixed > 0) {
    want = fixed;
  } else if (std::is_same<T, float>::value && max_it > 0) {
    const long long steps = steps_hint > 0 ? steps_hint : (n * max_it + 1) / 2;
    const long long lanes = (steps + max_it - 1) / max_it;
    want = std::max<long long>(3, (lanes + lanes_per_sm - 1) / lanes_per_sm);
  }
  const long long need = (n + SQF_T - 1) / SQF_T;
  const int fblocks = (int)std::max<long long>(
      1, std::min<long long>((long long)sms * std::min<long long>(std::max(per_sm, 1), want), need));
  if (g_sq_pairs.load(std::memory_order_relaxed)) {
    if (grad)
      sq_fwd2_kernel<T, true><<<fblocks, SQF_T, sh_roots, s>>>(params, nt, nb, xyz, target, n,
                                                               slice, max_it, escape, d_sat, claim, o);
    else
      sq_fwd2_kernel<T, false><<<fblocks, SQF_T, sh_roots, s>>>(params, nt, nb, xyz, target, n,
                                                                slice, max_it, escape, d_sat, claim, o);
  } else if (grad) {
    sq_fwd_kernel<T, true><<<fblocks, SQF_T, sh_roots, s>>>(params, nt, nb, xyz, target, n, slice,
                                                            max_it, escape, d_sat, claim, o);
  } else {
    sq_fwd_kernel<T, false><<<fblocks, SQF_T, sh_roots, s>>>(params, nt, nb, xyz, target, n, slice,
                                                             max_it, escape, d_sat, claim, o);
  }
  int* hist = grad ? reinterpret_cast<int*>(scr + L.hist) : nullptr;
  sq_chunk_kernel<<<L.nchunks, SQC_T, 0, s>>>(o.contrib, grad ? o.keys : nullptr, o.iters, n,
                                              max_it, L.nchunks, hist, partials, L.slots, 0, work);
  *launches = 3;
  int bwd_blocks = L.nbwd;  // rows of backward partials written
  if (grad) {
    unsigned* perm = reinterpret_cast<unsigned*>(scr + L.perm);
    sq_scan_kernel<<<1, 1024, 0, s>>>(hist, (long long)(max_it + 1) * L.nchunks, total);
    sq_scatter_kernel<<<L.nchunks, 32, 0, s>>>(o.keys, n, max_it, L.nchunks, hist, perm);
    const size_t sh_r = ((sizeof(T) * 5 * nr + 15) / 16) * 16;
    double* bwd_rows = partials + (size_t)L.nchunks * L.slots;
    bool done = false;
    if constexpr (std::is_same<T, float>::value) {
      // groups of 16 lanes while each side has at most 64 roots (4 per
      // lane); maps with more roots on a side keep one lane per sample,
      // which measured faster there than whole-warp groups (90/10 and 100/28
      // roots, 200k samples: 0.89 vs 0.99 ms, 1.17 vs 1.22 ms)
      const int ct = (nt + 15) / 16, cb = (nb + 15) / 16;
      if (g_sq_bwd_roots.load(std::memory_order_relaxed) && ct <= 4 && cb <= 4) {
        if (cb <= 1)  // at most 16 bottom roots: one per lane, 8 blocks per SM
          e = launch_bwd_roots<16, 4, 1, 8>(sh_r, L, sms, params, nt, nb, n, perm, total, o,
                                            bwd_rows, &bwd_blocks, s);
        else
          e = launch_bwd_roots<16, 4, 4, 1>(sh_r, L, sms, params, nt, nb, n, perm, total, o,
                                            bwd_rows, &bwd_blocks, s);
        if (e != cudaSuccess) return e;
        done = true;
      }
    }
    if (!done)
      sq_bwd_kernel<T><<<L.nbwd, SQ_T, sh_r + sizeof(double) * (SQ_T / 32) * L.slots, s>>>(
          params, nt, nb, n, perm, total, o.keys, o.seed_q, o.seed_L, o.ck, bwd_rows, L.slots);
    *launches += 3;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sq_reduce_kernel<<<L.slots, 32 * SQR_W, 0, s>>>(partials, bwd_blocks + L.nchunks, L.slots,
                                                  reinterpret_cast<double*>(scr + L.out));
  return cudaGetLastError();
}

// Byte layout of a batch's scratch (each piece 256-byte aligned).
struct SqBatchLayout {
  size_t items, chunk_item, claim, work, contrib, keys, iters, seed_q, seed_L, ck, bytes;
  std::vector<size_t> rp, hist, total, perm, partials, out;
  std::vector<long long> s0, c0, nchunks;
  std::vector<int> slots;
  long long n_flat = 0, chunks = 0;
  int nck = 0, max_slots = 0;
};

SqBatchLayout sq_batch_layout(const SqBatchReq* r, int K, int bwd_rows) {
  SqBatchLayout L;
  size_t at = 0;
  auto take = [&](size_t b) {
    const size_t o = at;
    at += (b + 255) / 256 * 256;
    return o;
  };
  for (int i = 0; i < K; i++) {
    const long long nc = std::max<long long>(1, (r[i].n + SQ_CH - 1) / SQ_CH);
    L.s0.push_back(L.n_flat);
    L.c0.push_back(L.chunks);
    L.nchunks.push_back(nc);
    L.n_flat += nc * SQ_CH;
    L.chunks += nc;
    L.nck = std::max(L.nck, r[i].max_it > 0 ? (r[i].max_it - 1) / SQ_CK + 1 : 0);
    L.slots.push_back(1 + 5 * (r[i].nt + r[i].nb) + 1 + 1);
    L.max_slots = std::max(L.max_slots, L.slots.back());
  }
  const size_t nf = (size_t)L.n_flat;
  L.items = take(sizeof(SqItem) * (size_t)K);
  L.chunk_item = take(sizeof(int) * (size_t)L.chunks);
  L.claim = take(sizeof(unsigned long long));
  L.work = take(2 * sizeof(unsigned long long));
  L.contrib = take(sizeof(double) * nf);
  L.keys = take(sizeof(int) * nf);
  L.iters = take(sizeof(int) * nf);
  L.seed_q = take(sizeof(V4<float>) * nf);
  L.seed_L = take(sizeof(float) * nf);
  L.ck = take(sizeof(V4<float>) * nf * (size_t)std::max(L.nck, 1));
  for (int i = 0; i < K; i++) {
    const size_t nr = (size_t)(r[i].nt + r[i].nb), n = (size_t)std::max<long long>(r[i].n, 0);
    L.rp.push_back(take(sizeof(float) * 5 * nr));
    L.hist.push_back(take(sizeof(int) * (size_t)(r[i].max_it + 1) * (size_t)L.nchunks[i]));
    L.total.push_back(take(sizeof(int)));
    L.perm.push_back(take(sizeof(unsigned) * std::max<size_t>(n, 1)));
    // after the chunk rows: a row per group of 32 samples (one-lane adjoint)
    // or per block of the grouped adjoint (at most bwd_rows blocks)
    const long long rows = std::max<long long>((long long)(n + 31) / 32, bwd_rows);
    L.partials.push_back(take(sizeof(double) * (size_t)(L.nchunks[i] + rows) * L.slots[i]));
    L.out.push_back(take(sizeof(double) * L.slots[i]));
  }
  L.bytes = at;
  return L;
}

}  // namespace

size_t sq_batch_scratch_bytes(const SqBatchReq* r, int K) {
  return sq_batch_layout(r, K, sm_count() * SQ_BWD_PER_SM).bytes;
}

cudaError_t launch_sq_energy_batch(const SqBatchReq* r, int K, void* scratch, double** outs,
                                   cudaStream_t s, int* launches) {
  if (K <= 0) return cudaSuccess;
  const int sms = sm_count();
  const SqBatchLayout L = sq_batch_layout(r, K, sms * SQ_BWD_PER_SM);
  unsigned char* scr = static_cast<unsigned char*>(scratch);
  std::vector<SqItem> items((size_t)K);
  std::vector<int> chunk_item((size_t)L.chunks);
  for (int i = 0; i < K; i++) {
    SqItem& it = items[(size_t)i];
    it.xyz = r[i].xyz;
    it.target = r[i].target;
    it.rp = reinterpret_cast<const float*>(scr + L.rp[(size_t)i]);
    it.params = r[i].params;
    it.nt = r[i].nt;
    it.nb = r[i].nb;
    it.max_it = r[i].max_it;
    it.slots = L.slots[(size_t)i];
    it.slice = r[i].slice;
    it.escape = r[i].escape;
    it.d_sat = r[i].d_sat;
    it.s0 = L.s0[(size_t)i];
    it.n = r[i].n;
    it.c0 = L.c0[(size_t)i];
    it.rows0 = 0;
    it.total = reinterpret_cast<int*>(scr + L.total[(size_t)i]);
    it.perm = reinterpret_cast<unsigned*>(scr + L.perm[(size_t)i]);
    it.partials = reinterpret_cast<double*>(scr + L.partials[(size_t)i]);
    for (long long c = 0; c < L.nchunks[(size_t)i]; c++) chunk_item[(size_t)(L.c0[(size_t)i] + c)] = i;
    outs[i] = reinterpret_cast<double*>(scr + L.out[(size_t)i]);
  }
  SqItem* d_items = reinterpret_cast<SqItem*>(scr + L.items);
  int* d_chunk_item = reinterpret_cast<int*>(scr + L.chunk_item);
  unsigned long long* claim = reinterpret_cast<unsigned long long*>(scr + L.claim);
  unsigned long long* work = reinterpret_cast<unsigned long long*>(scr + L.work);
  cudaError_t e;
  // pageable sources: each copy has left the host buffer when it returns
  if ((e = cudaMemcpyAsync(d_items, items.data(), sizeof(SqItem) * (size_t)K,
                           cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemcpyAsync(d_chunk_item, chunk_item.data(), sizeof(int) * chunk_item.size(),
                           cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemsetAsync(claim, 0, sizeof(unsigned long long), s)) ||
      (e = cudaMemsetAsync(work, 0, 2 * sizeof(unsigned long long), s)))
    return e;
  int n_launch = 0;
  sq_item_roots_kernel<<<K, 128, 0, s>>>(d_items, K);
  n_launch++;
  SqFwdOut<float> o{};
  o.contrib = reinterpret_cast<double*>(scr + L.contrib);
  o.keys = reinterpret_cast<int*>(scr + L.keys);
  o.iters = reinterpret_cast<int*>(scr + L.iters);
  o.seed_q = reinterpret_cast<V4<float>*>(scr + L.seed_q);
  o.seed_L = reinterpret_cast<float*>(scr + L.seed_L);
  o.ck = reinterpret_cast<V4<float>*>(scr + L.ck);
  // persistent forward grid: as the single request's first call, a lane per
  // two samples of the batch (at least 3 blocks per SM, at most the resident
  // count), fewer when the batch is small
  int per_sm = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sq_fwd_batch_kernel, SQF_T, 0)))
    return e;
  const long long need = (L.n_flat + SQF_T - 1) / SQF_T;
  long long total_n = 0;
  for (int i = 0; i < K; i++) total_n += r[i].n;
  const long long lanes_per_sm = (long long)sms * SQF_T;
  const long long want = std::min<long long>(
      std::max(per_sm, 1),
      std::max<long long>(3, ((total_n + 1) / 2 + lanes_per_sm - 1) / lanes_per_sm));
  const int fblocks = (int)std::max<long long>(1, std::min<long long>((long long)sms * want, need));
  sq_fwd_batch_kernel<<<fblocks, SQF_T, 0, s>>>(d_items, d_chunk_item, L.n_flat, claim, o);
  n_launch++;
  // per item: chunk sums and histogram, the sort's scan and scatter
  for (int i = 0; i < K; i++) {
    const long long s0 = L.s0[(size_t)i];
    int* hist = reinterpret_cast<int*>(scr + L.hist[(size_t)i]);
    sq_chunk_kernel<<<(unsigned)L.nchunks[(size_t)i], SQC_T, 0, s>>>(
        o.contrib + s0, o.keys + s0, o.iters + s0, r[i].n, r[i].max_it, (int)L.nchunks[(size_t)i],
        hist, items[(size_t)i].partials, L.slots[(size_t)i], 0, work);
    sq_scan_kernel<<<1, 1024, 0, s>>>(hist, (long long)(r[i].max_it + 1) * L.nchunks[(size_t)i],
                                      items[(size_t)i].total);
    sq_scatter_kernel<<<(unsigned)L.nchunks[(size_t)i], 32, 0, s>>>(
        o.keys + s0, r[i].n, r[i].max_it, (int)L.nchunks[(size_t)i], hist, items[(size_t)i].perm);
    n_launch += 3;
  }
  // the adjoint: the roots over 16-lane groups while every item has at most
  // 64 roots a side (as a single call), else one lane per sample
  int ct = 0, cb = 0;
  for (int i = 0; i < K; i++) {
    ct = std::max(ct, (r[i].nt + 15) / 16);
    cb = std::max(cb, (r[i].nb + 15) / 16);
  }
  int grp_blocks = 0;  // blocks of the grouped adjoint (0: one-lane form)
  if (g_sq_bwd_roots.load(std::memory_order_relaxed) && ct <= 4 && cb <= 4) {
    const size_t shg = SQB_ROOT_BYTES + sizeof(double) * (SQ_T / 16) * (size_t)L.max_slots;
    int per_sm = 0;
    if (cb <= 1)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, sq_bwd_batch_roots_kernel<16, 4, 1, 8>, SQ_T, shg);
    else
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, sq_bwd_batch_roots_kernel<16, 4, 4, 1>, SQ_T, shg);
    if (e) return e;
    grp_blocks = std::max(1, std::min(sms * SQ_BWD_PER_SM, std::max(per_sm, 1) * sms));
    if (cb <= 1)
      sq_bwd_batch_roots_kernel<16, 4, 1, 8><<<grp_blocks, SQ_T, shg, s>>>(
          d_items, K, L.n_flat, o.keys, o.seed_q, o.seed_L, o.ck);
    else
      sq_bwd_batch_roots_kernel<16, 4, 4, 1><<<grp_blocks, SQ_T, shg, s>>>(
          d_items, K, L.n_flat, o.keys, o.seed_q, o.seed_L, o.ck);
  } else {
    const size_t sh = sizeof(double) * (SQ_T / 32) * (size_t)L.max_slots;
    sq_bwd_batch_kernel<<<sms * SQ_BWD_PER_SM, SQ_T, sh, s>>>(d_items, K, L.n_flat, o.keys,
                                                                o.seed_q, o.seed_L, o.ck, L.max_slots);
  }
  n_launch++;
  for (int i = 0; i < K; i++) {
    if (grp_blocks > 0)
      sq_reduce_kernel<<<L.slots[(size_t)i], 32 * SQR_W, 0, s>>>(
          items[(size_t)i].partials, (int)L.nchunks[(size_t)i] + grp_blocks, L.slots[(size_t)i],
          outs[i]);
    else
      sq_reduce_item_kernel<<<L.slots[(size_t)i], 32 * SQR_W, 0, s>>>(
          items[(size_t)i].partials, (int)L.nchunks[(size_t)i], items[(size_t)i].total,
          L.slots[(size_t)i], outs[i]);
    n_launch++;
  }
  if (launches) *launches = n_launch;
  return cudaGetLastError();
}

int sq_max_iterations() { return SQ_MAXIT; }

void set_energy_pairs(int on) { g_sq_pairs.store(on ? 1 : 0); }

void set_energy_adjoint_roots(int on) { g_sq_bwd_roots.store(on ? 1 : 0); }

void set_energy_forward_blocks(int per_sm) { g_sq_fwd_blocks.store(per_sm > 0 ? per_sm : 0); }

cudaError_t set_energy_fast(int on) {
  const int v = on ? 1 : 0;
  return cudaMemcpyToSymbol(c_sq_fast, &v, sizeof v);
}

size_t sq_scratch_bytes(bool fp64, bool grad, long long n, int max_it, int nt, int nb) {
  return sq_layout(fp64, grad, n, max_it, nt, nb, sm_count()).bytes;
}

cudaError_t launch_sq_energy(bool fp64, bool grad, const double* params, int nt, int nb,
                             const double* xyz, const double* target, long long n, double slice,
                             int max_it, double escape, double d_sat, void* scratch,
                             double** out, int* iters, cudaStream_t s, int* launches,
                             unsigned long long** work, long long steps_hint) {
  const int sms = sm_count();
  const SqLayout L = sq_layout(fp64, grad, n, max_it, nt, nb, sms);
  unsigned char* scr = static_cast<unsigned char*>(scratch);
  *out = reinterpret_cast<double*>(scr + L.out);
  *work = reinterpret_cast<unsigned long long*>(scr + L.work);
  if (fp64)
    return sq_launch<double>(grad, params, nt, nb, xyz, target, n, slice, max_it, escape, d_sat,
                             scr, L, iters, sms, s, launches, steps_hint);
  return sq_launch<float>(grad, params, nt, nb, xyz, target, n, slice, max_it, escape, d_sat, scr,
                          L, iters, sms, s, launches, steps_hint);
}

}  // namespace qj
