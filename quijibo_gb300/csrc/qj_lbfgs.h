// Host-side launchers of the device L-BFGS kernels (lbfgs.cu).
#pragma once
#include <cuda_runtime.h>

namespace qj {

cudaError_t lbfgs_direction(const double* g, const double* S, const double* Y, const double* rho,
                            int n, int m, int k, int head, double* alpha, double* d, double* gd,
                            cudaStream_t s);
cudaError_t lbfgs_axpy(const double* x, const double* d, double a, int n, double* out,
                       cudaStream_t s);
cudaError_t lbfgs_update(const double* x0, const double* x1, const double* g0, const double* g1,
                         int n, int slot, double* S, double* Y, double* rho, cudaStream_t s);

}  // namespace qj
