// Limited-memory BFGS over the squared-error energy, state resident on the
// device: parameters, gradient, the (s, y) history and the search direction
// never leave HBM; the host sees only the scalar energies that the
// backtracking line search compares.  The reference's toothOptimizer runs a
// bound-constrained L-BFGS (BLMVM, src/TOUPEE/BLMVM.cpp) on the host over
// its own callback; this is an unconstrained L-BFGS (Nocedal & Wright,
// Algorithm 7.4 two-loop recursion, Armijo backtracking).
#include <cuda_runtime.h>

#include "qj_lbfgs.h"

namespace qj {

namespace {

constexpr int LB_T = 512;

__device__ double block_dot(const double* a, const double* b, int n) {
  __shared__ double sh[LB_T / 32];
  double v = 0;
  for (int i = threadIdx.x; i < n; i += LB_T) v += a[i] * b[i];
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0;
  for (int w = 0; w < LB_T / 32; w++) t += sh[w];
  __syncthreads();
  return t;
}

// d = -H g by the two-loop recursion over the newest `k` of `m` pairs
// stored in ring slots (head = slot of the newest pair).
__global__ void __launch_bounds__(LB_T) direction_kernel(const double* __restrict__ g,
                                                         const double* __restrict__ S,
                                                         const double* __restrict__ Y,
                                                         const double* __restrict__ rho, int n,
                                                         int m, int k, int head,
                                                         double* __restrict__ alpha,
                                                         double* __restrict__ d,
                                                         double* __restrict__ gd) {
  for (int i = threadIdx.x; i < n; i += LB_T) d[i] = -g[i];
  __syncthreads();
  for (int j = 0; j < k; j++) {  // newest to oldest
    const int s = (head - j + m) % m;
    const double a = rho[s] * block_dot(S + (size_t)s * n, d, n);
    if (threadIdx.x == 0) alpha[s] = a;
    for (int i = threadIdx.x; i < n; i += LB_T) d[i] -= a * Y[(size_t)s * n + i];
    __syncthreads();
  }
  if (k > 0) {  // H0 = (s.y / y.y) I for the newest pair
    const double yy = block_dot(Y + (size_t)head * n, Y + (size_t)head * n, n);
    const double gamma = (yy > 0 && rho[head] > 0) ? 1.0 / (rho[head] * yy) : 1.0;
    for (int i = threadIdx.x; i < n; i += LB_T) d[i] *= gamma;
    __syncthreads();
  }
  for (int j = k - 1; j >= 0; j--) {  // oldest to newest
    const int s = (head - j + m) % m;
    const double b = rho[s] * block_dot(Y + (size_t)s * n, d, n);
    const double a = alpha[s];
    for (int i = threadIdx.x; i < n; i += LB_T) d[i] += (a - b) * S[(size_t)s * n + i];
    __syncthreads();
  }
  const double dg = block_dot(d, g, n);
  if (threadIdx.x == 0) *gd = dg;
}

__global__ void axpy_kernel(const double* __restrict__ x, const double* __restrict__ d, double a,
                            int n, double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = x[i] + a * d[i];
}

// store s = x1 - x0, y = g1 - g0 in slot `slot`; rho = 1 / y.s (0 when y.s <= 0)
__global__ void __launch_bounds__(LB_T) update_kernel(const double* __restrict__ x0,
                                                      const double* __restrict__ x1,
                                                      const double* __restrict__ g0,
                                                      const double* __restrict__ g1, int n,
                                                      int slot, double* __restrict__ S,
                                                      double* __restrict__ Y,
                                                      double* __restrict__ rho) {
  double* s = S + (size_t)slot * n;
  double* y = Y + (size_t)slot * n;
  for (int i = threadIdx.x; i < n; i += LB_T) {
    s[i] = x1[i] - x0[i];
    y[i] = g1[i] - g0[i];
  }
  __syncthreads();
  const double ys = block_dot(y, s, n);
  if (threadIdx.x == 0) rho[slot] = ys > 0 ? 1.0 / ys : 0.0;
}

}  // namespace

cudaError_t lbfgs_direction(const double* g, const double* S, const double* Y, const double* rho,
                            int n, int m, int k, int head, double* alpha, double* d, double* gd,
                            cudaStream_t s) {
  direction_kernel<<<1, LB_T, 0, s>>>(g, S, Y, rho, n, m, k, head, alpha, d, gd);
  return cudaGetLastError();
}

cudaError_t lbfgs_axpy(const double* x, const double* d, double a, int n, double* out,
                       cudaStream_t s) {
  axpy_kernel<<<(n + 255) / 256, 256, 0, s>>>(x, d, a, n, out);
  return cudaGetLastError();
}

cudaError_t lbfgs_update(const double* x0, const double* x1, const double* g0, const double* g1,
                         int n, int slot, double* S, double* Y, double* rho, cudaStream_t s) {
  update_kernel<<<1, LB_T, 0, s>>>(x0, x1, g0, g1, n, slot, S, Y, rho);
  return cudaGetLastError();
}

}  // namespace qj
