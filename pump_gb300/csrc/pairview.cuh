// A query's N(N-1) ordered pair costs/times seen through the batch's shared
// roadmap.  Sample 0 is the query's init state, samples 1 .. N-2 are Halton
// points 1 .. N-2 (the same points for every N, sampler.cu:20-41) and sample
// N-1 is its goal.  Pairs of two Halton points come from the batch's shared
// pair arrays (Halton points 1 .. M, M >= N-2, pump_bvp_pairs layout
// a*(M-1) + b - (a < b)); pairs touching init or goal from the query's own
// arrays.  Pair idx is numbered as pump_bvp_pairs numbers it:
// idx = i*(N-1) + j - (i < j).
#pragma once

#include "common.cuh"

namespace pump {

struct PairView {
  int N;
  long long M;
  const float *sc, *st;     // shared: copt / topt
  const float *irc, *irt;   // init row   (0 -> j),   j = 1 .. N-1  at [j-1]
  const float *icc, *ict;   // init col   (i -> 0),   i = 1 .. N-1  at [i-1]
  const float *grc, *grt;   // goal row   (N-1 -> j), j = 1 .. N-2  at [j-1]
  const float *gcc, *gct;   // goal col   (i -> N-1), i = 1 .. N-2  at [i-1]

  __device__ __forceinline__ void pair(long long idx, int *i, int *j) const {
    const int a = (int)(idx / (N - 1));
    const int r = (int)(idx - (long long)a * (N - 1));
    *i = a;
    *j = r + (r >= a);
  }
  __device__ __forceinline__ long long shared_index(int i, int j) const {
    const long long a = i - 1, b = j - 1;
    return a * (M - 1) + b - (a < b);
  }
  __device__ __forceinline__ float copt(int i, int j) const {
    if (i == 0) return __ldg(&irc[j - 1]);
    if (j == 0) return __ldg(&icc[i - 1]);
    if (i == N - 1) return __ldg(&grc[j - 1]);
    if (j == N - 1) return __ldg(&gcc[i - 1]);
    return __ldg(&sc[shared_index(i, j)]);
  }
  // The bits of copt(i, j), loaded as an integer (sort keys never pass
  // through a float value).
  __device__ __forceinline__ uint32_t copt_bits(int i, int j) const {
    const float *p = i == 0           ? &irc[j - 1]
                     : j == 0         ? &icc[i - 1]
                     : i == N - 1     ? &grc[j - 1]
                     : j == N - 1     ? &gcc[i - 1]
                                      : &sc[shared_index(i, j)];
    return __ldg(reinterpret_cast<const unsigned int *>(p));
  }
  __device__ __forceinline__ float topt(int i, int j) const {
    if (i == 0) return __ldg(&irt[j - 1]);
    if (j == 0) return __ldg(&ict[i - 1]);
    if (i == N - 1) return __ldg(&grt[j - 1]);
    if (j == N - 1) return __ldg(&gct[i - 1]);
    return __ldg(&st[shared_index(i, j)]);
  }
};

}  // namespace pump
