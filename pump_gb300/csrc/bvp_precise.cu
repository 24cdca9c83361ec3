// Precision-mode 2pBVP kernels: the closed-form optimal time of precise.cuh
// for all ordered pairs of a sample set or for explicit pairs.  Compiled with
// multiply-add contraction (the mode is not bound to the reference's
// roundings).
#include "common.cuh"
#include "ctx.h"
#include "tune.h"
#include "precise.cuh"

namespace pump {
namespace {

__device__ void precise_pair(const float *x0, const float *x1, float tmax, float *topt,
                             float *cost) {
  double t, c;
  precise_tau(x0, x1, tmax, &t, &c);
  *topt = d2f_rn(t);
  *cost = d2f_rn(c);
}

__global__ void prepare_samples_kernel(const float *__restrict__ samples, int N,
                                       SampleF *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  float x[kDim];
#pragma unroll
  for (int d = 0; d < kDim; ++d) x[d] = samples[i * kDim + d];
  out[i] = to_sample_f(x);
}

__device__ __forceinline__ SampleF load_sample(const SampleF *__restrict__ s, int i) {
  const float4 *q = reinterpret_cast<const float4 *>(s + i);
  const float4 a = __ldg(q), b = __ldg(q + 1);
  SampleF r;
  r.p[0] = a.x; r.p[1] = a.y; r.p[2] = a.z;
  r.v[0] = a.w; r.v[1] = b.x; r.v[2] = b.y;
  r.vv.h = b.z; r.vv.l = b.w;
  return r;
}

// Row i = blockIdx.y, column r = blockIdx.x * T + threadIdx.x (j = r, or
// r + 1 past the diagonal): no index division per pair.  The block size T is
// picked by the autotuner.
template <int T>
__global__ void __launch_bounds__(T) bvp_pairs_precision_kernel(const SampleF *__restrict__ sf,
                                                                int N, float tmax,
                                                                float *__restrict__ copts,
                                                                float *__restrict__ topts) {
  const int i = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N - 1) return;
  const int j = r + (r >= i);
  double t, c;
  precise_tau(load_sample(sf, i), load_sample(sf, j), tmax, &t, &c);
  const long long idx = (long long)i * (N - 1) + r;
  topts[idx] = d2f_rn(t);
  copts[idx] = d2f_rn(c);
}

// Costs of the bracket-sample pairs: pair number floor((2q + 1) n / (2 S))
// for q < S, n = N(N-1).
__global__ void bracket_costs_kernel(const SampleF *__restrict__ sf, int N, float tmax, int S,
                                     unsigned int *__restrict__ out_bits) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= S) return;
  const long long n = (long long)N * (N - 1);
  const long long pos = ((2LL * q + 1) * n) / (2LL * S);
  const int i = (int)(pos / (N - 1));
  const int r = (int)(pos - (long long)i * (N - 1));
  const int j = r + (r >= i);
  double t, c;
  precise_tau(load_sample(sf, i), load_sample(sf, j), tmax, &t, &c);
  out_bits[q] = __float_as_uint(d2f_rn(c));
}

// bvp_pairs_precision_kernel plus the count pass of the rn superset: each
// warp adds its pairs whose cost's order key is below *key_hi to the counts
// of their 4096-pair tiles (a warp's 32 consecutive pairs meet at most two
// tiles: one atomic for each).  A warp wholly past its row's end leaves at
// once; the others reach the ballots with every lane.
template <int T>
__global__ void __launch_bounds__(T) bvp_pairs_precision_counted_kernel(
    const SampleF *__restrict__ sf, int N, float tmax, float *__restrict__ copts,
    float *__restrict__ topts, const unsigned long long *__restrict__ key_hi,
    unsigned int *__restrict__ tile_counts) {
  const int i = blockIdx.y;
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r - lane >= N - 1) return;
  const long long idx = (long long)i * (N - 1) + r;
  bool sel = false;
  if (r < N - 1) {
    const int j = r + (r >= i);
    double t, c;
    precise_tau(load_sample(sf, i), load_sample(sf, j), tmax, &t, &c);
    const unsigned int cb = __float_as_uint(d2f_rn(c));
    topts[idx] = d2f_rn(t);
    reinterpret_cast<unsigned int *>(copts)[idx] = cb;
    sel = (unsigned long long)key_of_bits(cb) < __ldg(key_hi);
  }
  const unsigned int m = __ballot_sync(0xffffffffu, sel);
  if (m) {
    const long long t0 = (idx - lane) / kRnCountTile;
    const unsigned int in0 = __ballot_sync(0xffffffffu, sel && idx / kRnCountTile == t0);
    if (lane == 0) {
      if (in0) atomicAdd(&tile_counts[t0], (unsigned int)__popc(in0));
      if (m & ~in0) atomicAdd(&tile_counts[t0 + 1], (unsigned int)__popc(m & ~in0));
    }
  }
}

__global__ void bvp_batch_precision_kernel(const BvpJobs jb) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= jb.n * jb.jobs) return;
  const int j = k >= jb.n ? 1 : 0;
  k -= j * jb.n;
  float x0[kDim], x1[kDim];
#pragma unroll
  for (int d = 0; d < kDim; ++d) {
    x0[d] = jb.x0[k * kDim + d];
    x1[d] = jb.x1[(jb.x1_same ? 0 : k) * kDim + d];
  }
  float tp, cp;
  precise_pair(x0, x1, jb.tmax[j], &tp, &cp);
  if (jb.topt[j]) jb.topt[j][k] = tp;
  if (jb.cost[j]) jb.cost[j][k] = cp;
}

}  // namespace

pump_status_t bvp_pairs_precision_launch(const float *d_samples, int N, float tmax, float *d_copts,
                                         float *d_topts, cudaStream_t stream) {
  if (N > 65535) return set_error(PUMP_ERR_CAPACITY, "bvp_pairs: N = %d exceeds 65535 rows", N);
  SampleF *sd = nullptr;
  PUMP_CUDA_TRY(pool_malloc_async((void **)&sd, sizeof(SampleF) * (size_t)N, stream));
  prepare_samples_kernel<<<grid_for(N, 128), 128, 0, stream>>>(d_samples, N, sd);
  pump_status_t st = launch_status("prepare_samples");
  // block sizes 64, 128 (default), 256
  auto run = [&](int c) -> pump_status_t {
    const int T = c == 0 ? 64 : (c == 1 ? 128 : 256);
    const dim3 grid(grid_for(N - 1, T), (unsigned)N);
    if (c == 0) bvp_pairs_precision_kernel<64><<<grid, 64, 0, stream>>>(sd, N, tmax, d_copts, d_topts);
    else if (c == 1)
      bvp_pairs_precision_kernel<128><<<grid, 128, 0, stream>>>(sd, N, tmax, d_copts, d_topts);
    else bvp_pairs_precision_kernel<256><<<grid, 256, 0, stream>>>(sd, N, tmax, d_copts, d_topts);
    return launch_status("bvp_pairs_precision");
  };
  if (st == PUMP_OK) {
    int choice = 1;
    bool ran = false;
    st = tune_choice(kTuneBvpPairs, tune_bucket(N), 3, 1, stream, run, &choice, &ran);
    if (st == PUMP_OK && !ran) st = run(choice);
  }
  cudaFreeAsync(sd, stream);
  return st;
}

pump_status_t bvp_pairs_precision_counted(const float *d_samples, int N, float tmax,
                                          float *d_copts, float *d_topts, int S,
                                          float *d_sample_costs,
                                          const std::function<pump_status_t()> &bracket,
                                          const unsigned long long *d_key_hi,
                                          unsigned int *d_tile_counts, cudaStream_t stream) {
  if (N > 65535) return set_error(PUMP_ERR_CAPACITY, "bvp_pairs: N = %d exceeds 65535 rows", N);
  SampleF *sd = nullptr;
  PUMP_CUDA_TRY(pool_malloc_async((void **)&sd, sizeof(SampleF) * (size_t)N, stream));
  prepare_samples_kernel<<<grid_for(N, 128), 128, 0, stream>>>(d_samples, N, sd);
  pump_status_t st = launch_status("prepare_samples");
  if (st == PUMP_OK) {
    bracket_costs_kernel<<<grid_for(S, 64), 64, 0, stream>>>(
        sd, N, tmax, S, reinterpret_cast<unsigned int *>(d_sample_costs));
    st = launch_status("bracket_costs");
  }
  if (st == PUMP_OK) st = bracket();
  if (st == PUMP_OK) {
    // the block size of the plain pass's default (the tuner's three shapes
    // measure within 1 % of each other)
    constexpr int T = 128;
    const dim3 grid(grid_for(N - 1, T), (unsigned)N);
    bvp_pairs_precision_counted_kernel<T><<<grid, T, 0, stream>>>(sd, N, tmax, d_copts, d_topts,
                                                                 d_key_hi, d_tile_counts);
    st = launch_status("bvp_pairs_precision_counted");
  }
  cudaFreeAsync(sd, stream);
  return st;
}

pump_status_t bvp_jobs_precision_launch(const BvpJobs &jb, cudaStream_t stream) {
  const long long total = (long long)jb.n * jb.jobs;
  const int threads = total < 152LL * 128 ? 32 : 128;
  bvp_batch_precision_kernel<<<grid_for(total, threads), threads, 0, stream>>>(jb);
  return launch_status("bvp_batch_precision");
}

}  // namespace pump
