// Precision-mode 2pBVP kernels: the closed-form optimal time of precise.cuh
// for all ordered pairs of a sample set or for explicit pairs.  Compiled with
// multiply-add contraction (the mode is not bound to the reference's
// roundings).
#include "common.cuh"
#include "ctx.h"
#include "precise.cuh"

namespace pump {
namespace {

__device__ void precise_pair(const float *x0, const float *x1, float tmax, float *topt,
                             float *cost) {
  double t, c;
  precise_tau(x0, x1, tmax, &t, &c);
  *topt = (float)t;
  *cost = (float)c;
}

__global__ void __launch_bounds__(128) bvp_pairs_precision_kernel(const float *__restrict__ samples,
                                                                  int N, float tmax,
                                                                  float *__restrict__ copts,
                                                                  float *__restrict__ topts) {
  const long long npairs = (long long)N * (N - 1);
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < npairs;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / (N - 1));
    const int r = (int)(idx - (long long)i * (N - 1));
    const int j = r + (r >= i);
    float x0[kDim], x1[kDim];
#pragma unroll
    for (int d = 0; d < kDim; ++d) {
      x0[d] = __ldg(&samples[i * kDim + d]);
      x1[d] = __ldg(&samples[j * kDim + d]);
    }
    float tp, cp;
    precise_pair(x0, x1, tmax, &tp, &cp);
    topts[idx] = tp;
    copts[idx] = cp;
  }
}

__global__ void bvp_batch_precision_kernel(const float *__restrict__ x0s,
                                           const float *__restrict__ x1s, int n, float tmax,
                                           float *__restrict__ topt, float *__restrict__ cost) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float x0[kDim], x1[kDim];
#pragma unroll
  for (int d = 0; d < kDim; ++d) {
    x0[d] = x0s[k * kDim + d];
    x1[d] = x1s[k * kDim + d];
  }
  float tp, cp;
  precise_pair(x0, x1, tmax, &tp, &cp);
  if (topt) topt[k] = tp;
  if (cost) cost[k] = cp;
}

}  // namespace

pump_status_t bvp_pairs_precision_launch(const float *d_samples, int N, float tmax, float *d_copts,
                                         float *d_topts, cudaStream_t stream) {
  const long long npairs = (long long)N * (N - 1);
  long long blocks = (npairs + 127) / 128;
  if (blocks > 2147483647LL) blocks = 2147483647LL;
  bvp_pairs_precision_kernel<<<(unsigned)blocks, 128, 0, stream>>>(d_samples, N, tmax, d_copts,
                                                                    d_topts);
  return launch_status("bvp_pairs_precision");
}

pump_status_t bvp_batch_precision_launch(const float *d_x0, const float *d_x1, int n, float tmax,
                                         float *d_topt, float *d_cost, cudaStream_t stream) {
  bvp_batch_precision_kernel<<<grid_for(n, 128), 128, 0, stream>>>(d_x0, d_x1, n, tmax, d_topt,
                                                                  d_cost);
  return launch_status("bvp_batch_precision");
}

}  // namespace pump
