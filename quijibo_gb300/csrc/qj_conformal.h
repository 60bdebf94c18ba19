// Launchers of conformal.cu (the optimizer's set-up passes).
#pragma once
#include <cuda_runtime.h>

#include "qj_params.h"

namespace qj {

int conformal_blocks(long long n);
cudaError_t launch_shells(const double* dist, int X, int Y, int Z, double* w, cudaStream_t s);
cudaError_t launch_layer(const double* cur, double* next, int X, int Y, int Z,
                         unsigned long long* zeros_left, cudaStream_t s);
cudaError_t launch_invert(const double* dist, double* w, long long n, cudaStream_t s);
// out3 = {sum |w|, sum w*scale where dist < 0, sum w*scale where dist >= 0};
// part holds 3 * conformal_blocks(n) doubles
cudaError_t launch_side_sums(const double* dist, const double* w, long long n, double scale,
                             double* part, double* out3, cudaStream_t s);
// out3 = {sum w where md < 0 and fd > 0, sum w where md < 0 and fd < 0,
// count of md > 0}; part holds 3 * conformal_blocks(n) doubles
cudaError_t launch_region_sums(const double* md, const double* fd, const double* w, long long n,
                               double* part, double* out3, cudaStream_t s);
// out = w * k_poor (md < 0, fd > 0), w * k_well (md < 0, fd < 0), w (md < 0,
// fd = 0), `outside` (md >= 0)
cudaError_t launch_reweight(const double* md, const double* fd, const double* w, long long n,
                            double k_poor, double k_well, double outside, double* out,
                            cudaStream_t s);
cudaError_t launch_borders(double* f, int X, int Y, int Z, double value, cudaStream_t s);
cudaError_t launch_scale_sides(const double* dist, double* w, long long n, double scale,
                               double k_in, double k_out, cudaStream_t s);
// part: 4 doubles per block {sum of non-infinite values, their count, min, max}
cudaError_t launch_field_stats(const double* f, long long n, double* part, int* nblk,
                               cudaStream_t s);
cudaError_t launch_clamp_infs(double* f, long long n, double mean, cudaStream_t s);
cudaError_t launch_lookup(const GridParams& g, const WeightGrid& wg, const double* w, double* out,
                          cudaStream_t s);
// scores[t] = sum_i -tanh(alpha (f_i - thr[t])) w_i; part holds
// conformal_blocks(n) * nthr doubles
cudaError_t launch_scan(const double* f, const double* w, long long n, const double* thr,
                        int nthr, double alpha, double* part, double* scores, cudaStream_t s);

}  // namespace qj
