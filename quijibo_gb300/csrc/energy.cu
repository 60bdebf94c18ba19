// Fitting energies and their gradients.
//
// tanh_grad_kernel: the reference's tanh-weighted score and its analytic
// one-application gradients in one pass per voxel, FP64 in reference
// operation order:
//   score  = sum -tanh(alpha F) w                 weightScore, OPTIMIZE_3D.cpp:4502-4517
//   F      = the adaptive-precision map           computeRationalMapAP, :1374-1488
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

// FIELD_3D::operator()(const VEC3F&), FIELD_3D.cpp:966-1029.
__device__ double trilinear(const WeightGrid& wg, const double* __restrict__ data,
                            const double p[3]) {
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

// Per-warp accumulation of one slot (lane values summed by a shuffle tree).
__device__ __forceinline__ void warp_accum(double* acc, int slot, double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) acc[slot] += v;
}

template <bool POW_REF>
__global__ void __launch_bounds__(EN_T) tanh_grad_kernel(const __grid_constant__ MapParams m,
                                                         const GridParams g, const WeightGrid wg,
                                                         const double* __restrict__ weights,
                                                         int max_it, double alpha, double thr,
                                                         double* __restrict__ field,
                                                         double* __restrict__ partials, int slots) {
  extern __shared__ double acc_sh[];  // [EN_T / 32][slots]
  const int warp = threadIdx.x >> 5;
  double* acc = acc_sh + warp * slots;
  for (int k = threadIdx.x; k < (EN_T / 32) * slots; k += EN_T) acc_sh[k] = 0.0;
  __syncthreads();
  Q Pf[QJ_MAX_ROOTS];  // last iteration's factors (local memory)
  Q Sf[QJ_MAX_ROOTS];  // their suffix products
  const int nt = m.nt, nb = m.nb;
  const long long N = (long long)g.X * g.Y * g.Z;
  const double logs = log(m.scale);
  const int s_score = 3 + nt + nb, s_over = s_score + 1, s_bad = s_score + 2;
  // every lane of a warp walks the same number of rounds so shuffles stay full
  const long long stride = (long long)gridDim.x * EN_T;
  const long long rounds = (N + stride - 1) / stride;
  for (long long rd = 0; rd < rounds; rd++) {
    const long long idx = rd * stride + (long long)blockIdx.x * EN_T + threadIdx.x;
    const bool live = idx < N;
    double c_exp = 0, c_score = 0, c_over = 0, c_bad = 0, c_bulk_t = 0, c_bulk_b = 0;
    bool grad_ok = false;
    double dSdF = 0, RR = 0;
    Q R = {0, 0, 0, 0}, T = {1, 0, 0, 0}, B = {1, 0, 0, 0}, q0 = {0, 0, 0, 0};
    if (live) {
      const int x = (int)(idx % g.X), y = (int)((idx / g.X) % g.Y);
      const int z = (int)(idx / ((long long)g.X * g.Y));
      double p[3];
      cell_center(g, x, y, z, p);
      q0 = Q{p[0], p[1], p[2], g.slice};
      Q q = q0;
      double mg = mag(q);
      bool over = false, iterated = false;
      double fval = 0.0;
      if (!(mg < 1e-8)) {  // "if we hit the origin, move on"
        int it = 0;
        while (mg < 20.0 && it < max_it) {  // computeRationalMapAP's escape radius 20
          iterated = true;
#pragma unroll 1
          for (int side = 0; side < 2; side++) {
            const int lo = side ? nt : 0, hi = side ? nt + nb : nt;
            Q acc_q = {1, 0, 0, 0};
#pragma unroll 1
            for (int i = lo; i < hi; i++) {
              Q d{sub(q.w, m.r64[i][0]), sub(q.x, m.r64[i][1]), sub(q.y, m.r64[i][2]),
                  sub(q.z, m.r64[i][3])};
              Pf[i] = POW_REF ? qpow(d, m.e64[i]) : qpow_int(d, m.ie[i]);
              acc_q = (i == lo) ? Pf[i] : qmul(acc_q, Pf[i]);
            }
            if (side == 0)
              T = acc_q;
            else if (nb > 0)
              B = acc_q;
          }
          q = nb > 0 ? qdiv(T, B) : T;
          over = over || !isfinite(T.w) || !isfinite(T.x) || !isfinite(T.y) || !isfinite(T.z) ||
                 (nb > 0 && (!isfinite(B.w) || !isfinite(B.x) || !isfinite(B.y) || !isfinite(B.z)));
          q = qscale(q, m.scale);
          mg = mag(q);
          if (isinf(mg) || isnan(mg)) over = true;
          it++;
        }
        fval = log(mg);
      }
      if (field) field[idx] = fval;
      const double w = trilinear(wg, weights, p);
      c_score = mul(-tanh(mul(alpha, fval)), w);
      {
        const double S = tanh(mul(alpha, sub(fval, thr)));
        c_exp = mul(mul(-alpha, w), sub(1.0, mul(S, S)));
      }
      c_over = over ? 1.0 : 0.0;
      if (iterated && !over) {
        R = qdiv(T, B);
        const double Rm = mag(R);
        if (!(Rm <= 0.0 || isinf(Rm))) {
          const double F = add(log(Rm), logs);
          const double th = tanh(mul(alpha, sub(F, thr)));
          dSdF = mul(mul(-alpha, w), sub(1.0, mul(th, th)));
          RR = __ddiv_rn(1.0, qdot(R, R));
          grad_ok = true;
          // suffix products (POLYNOMIAL_4D.cpp:1066-1072), per side
#pragma unroll 1
          for (int side = 0; side < 2; side++) {
            const int lo = side ? nt : 0, hi = side ? nt + nb : nt;
            if (hi == lo) continue;
            Sf[hi - 1] = Pf[hi - 1];
#pragma unroll 1
            for (int i = hi - 2; i >= lo; i--) Sf[i] = qmul(Pf[i], Sf[i + 1]);
          }
        }
      }
    }
    warp_accum(acc, 0, c_exp);
    warp_accum(acc, s_score, c_score);
    warp_accum(acc, s_over, c_over);
    // top roots: left = forward[i-1], right = backward[i+1]
    Q left = {1, 0, 0, 0};
#pragma unroll 1
    for (int i = 0; i < nt; i++) {
      double c_i = 0;
      if (grad_ok) {
        const Q right = (nt > 1 && i < nt - 1) ? Sf[i + 1] : Q{1, 0, 0, 0};
        const Q base{sub(q0.w, m.r64[i][0]), sub(q0.x, m.r64[i][1]), sub(q0.y, m.r64[i][2]),
                     sub(q0.z, m.r64[i][3])};
        const Q pw = qpow(base, m.e64[i]);
        const Q lg = qlog(base);
#pragma unroll 1
        for (int pass = 0; pass < 2; pass++) {
          const double k = pass == 0 ? m.sigma[0] : m.ep[i];
          const Q dT = qmul(qmul(left, qmul(qscale(pw, k), lg)), right);
          const double dSdt = mul(dSdF, mul(RR, qdot(R, qdiv(dT, B))));
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
      if (grad_ok) {
        const Q right = (nb > 1 && j < nb - 1) ? Sf[nt + j + 1] : Q{1, 0, 0, 0};
        const Q base{sub(q0.w, m.r64[nt + j][0]), sub(q0.x, m.r64[nt + j][1]),
                     sub(q0.y, m.r64[nt + j][2]), sub(q0.z, m.r64[nt + j][3])};
        const Q pw = qpow(base, m.e64[nt + j]);
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
  __syncthreads();
  for (int k = threadIdx.x; k < slots; k += EN_T) {
    double s = 0;
    for (int wv = 0; wv < EN_T / 32; wv++) s += acc_sh[wv * slots + k];
    partials[(long long)blockIdx.x * slots + k] = s;
  }
}

// Neumaier-compensated sum of partials[b][k] over blocks b, in block order.
__global__ void reduce_partials_kernel(const double* __restrict__ partials, int nblocks,
                                       int slots, double* __restrict__ out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < slots; k += gridDim.x * blockDim.x) {
    double s = 0, c = 0;
    for (int b = 0; b < nblocks; b++) {
      const double v = partials[(long long)b * slots + k];
      const double t = s + v;
      c += (fabs(s) >= fabs(v)) ? (s - t) + v : (v - t) + s;
      s = t;
    }
    out[k] = s + c;
  }
}

}  // namespace

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
  const int slots = 6 + m.nt + m.nb;
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
  return cudaGetLastError();
}

}  // namespace qj
