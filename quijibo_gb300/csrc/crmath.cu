// Element-wise evaluation of the correctly rounded transcendentals of
// qj_crmath.h (measurement and test hook, no reference counterpart): the
// device results can be compared bit for bit with the same functions
// compiled for the host.
#include <cuda_runtime.h>

#include "../../include/quijibo_gpu_bench.h"
#include "qj_crmath.h"

namespace {

__global__ void __launch_bounds__(256) crmath_kernel(int fn, const double* __restrict__ x,
                                                     double* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = x[i];
    double r;
    switch (fn) {
      case QJG_CRM_EXP: r = crm_exp(v); break;
      case QJG_CRM_LOG: r = crm_log(v); break;
      case QJG_CRM_SIN: r = crm_sin(v); break;
      case QJG_CRM_COS: r = crm_cos(v); break;
      default: r = crm_acos(v); break;
    }
    y[i] = r;
  }
}

}  // namespace

extern "C" int qjg_crmath_eval(int fn, const double* d_x, double* d_y, int64_t n, void* stream) {
  if (fn < QJG_CRM_EXP || fn > QJG_CRM_ACOS || n < 0 || (n > 0 && (!d_x || !d_y)))
    return QJG_ERR_ARG;
  if (n == 0) return QJG_OK;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long most = 8ll * sms;  // grid-stride beyond eight blocks per SM
  const long long blocks = (n + 255) / 256 < most ? (n + 255) / 256 : most;
  crmath_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(fn, d_x, d_y, (long long)n);
  return cudaGetLastError() == cudaSuccess ? QJG_OK : QJG_ERR_CUDA;
}
