// Precision-mode 2pBVP kernels: the closed-form optimal time of precise.cuh
// for all ordered pairs of a sample set or for explicit pairs.  Compiled with
// multiply-add contraction (the mode is not bound to the reference's
// roundings).
#include "common.cuh"
#include "ctx.h"
#include "tune.h"
#include "precise.cuh"
#include "bracket.cuh"

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

// The samples' binary64 forms and the rn bracket, one launch: blocks below
// nprep prepare 1024 samples each; the kBracketBlocks blocks after them
// compute, in their first kBracketPerBlock threads, the costs of the
// bracket-sample pairs (pair number floor((2q + 1) n / (2 S)), from the raw
// samples; spread over many SMs, as the binary64 pipe of one SM would take
// several times longer) and store their order keys, and the one of those
// that finishes last (a counter of finished blocks, reset by that block)
// runs the bracket's radix steps over all of them with its 1024 threads.
constexpr int kBracketPerBlock = 128;
constexpr int kBracketBlocks = kBracketSamples / kBracketPerBlock;
__global__ void __launch_bounds__(1024) prepare_bracket_kernel(
    const float *__restrict__ samples, int N, float tmax, int nprep, SampleF *__restrict__ sf,
    unsigned int rank, uint32_t *keys_g, unsigned int *done, unsigned long long *key_hi) {
  if ((int)blockIdx.x < nprep) {
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < N) {
      float x[kDim];
#pragma unroll
      for (int d = 0; d < kDim; ++d) x[d] = samples[i * kDim + d];
      sf[i] = to_sample_f(x);
    }
    return;
  }
  __shared__ uint32_t keys[kBracketSamples];
  __shared__ bool s_last;
  if (threadIdx.x < kBracketPerBlock) {
    const int q = ((int)blockIdx.x - nprep) * kBracketPerBlock + threadIdx.x;
    const long long n = (long long)N * (N - 1);
    const long long pos = ((2LL * q + 1) * n) / (2LL * kBracketSamples);
    const int i = (int)(pos / (N - 1));
    const int r = (int)(pos - (long long)i * (N - 1));
    const int j = r + (r >= i);
    float a[kDim], b[kDim];
#pragma unroll
    for (int d = 0; d < kDim; ++d) {
      a[d] = samples[i * kDim + d];
      b[d] = samples[j * kDim + d];
    }
    double t, c;
    precise_tau(a, b, tmax, &t, &c);
    keys_g[q] = key_of_bits(__float_as_uint(d2f_rn(c)));
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == kBracketBlocks - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int p = threadIdx.x; p < kBracketSamples; p += 1024) keys[p] = __ldcg(&keys_g[p]);
  __syncthreads();
  bracket_radix(keys, rank, key_hi);
  if (threadIdx.x == 0) *done = 0u;
}

// All pairs, one block per 128 consecutive pairs of a row (row i =
// blockIdx.y): each pair's cost and time are stored, and each warp stores
// the ballot of its 32 pairs whose cost's order key is below *key_hi (bit
// l = pair l of the warp), warp tile (row, column block, warp) in pair
// order.  No thread waits for another.
constexpr int kPairTile = 128;
__global__ void __launch_bounds__(kPairTile) bvp_pairs_masked_kernel(
    const SampleF *__restrict__ sf, int N, float tmax, float *__restrict__ copts,
    float *__restrict__ topts, const unsigned long long *__restrict__ key_hi,
    uint32_t *__restrict__ masks) {
  const int i = blockIdx.y;
  const int r = blockIdx.x * kPairTile + threadIdx.x;
  bool sel = false;
  if (r < N - 1) {
    const int j = r + (r >= i);
    const long long idx = (long long)i * (N - 1) + r;
    double t, c;
    precise_tau(load_sample(sf, i), load_sample(sf, j), tmax, &t, &c);
    const unsigned int cb = __float_as_uint(d2f_rn(c));
    reinterpret_cast<unsigned int *>(copts)[idx] = cb;
    topts[idx] = d2f_rn(t);
    sel = (unsigned long long)key_of_bits(cb) < __ldg(key_hi);
  }
  const unsigned int bal = __ballot_sync(0xffffffffu, sel);
  if ((threadIdx.x & 31) == 0)
    masks[((long long)i * gridDim.x + blockIdx.x) * (kPairTile / 32) + (threadIdx.x >> 5)] = bal;
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

pump_status_t bvp_pairs_precision_superset(Ctx *ctx, const float *d_samples, int N, float tmax,
                                           float *d_copts, float *d_topts, const PairSuperset &ps,
                                           cudaStream_t stream, cudaEvent_t between) {
  const long long n = (long long)N * (N - 1);
  if (N < 2 || N > 65535 || n >= (1LL << 32))
    return set_error(PUMP_ERR_CAPACITY, "bvp_pairs_superset: N = %d", N);
  const unsigned int nbx = grid_for(N - 1, kPairTile);
  const int per_row = (int)nbx * (kPairTile / 32);
  uint32_t *masks = nullptr;
  PUMP_TRY(ctx->scratch(Ctx::kPairStage, sizeof(uint32_t) * (size_t)per_row * N, (void **)&masks));
  ps.out->masks = masks;
  ps.out->nmasks = (long long)per_row * N;
  ps.out->masks_per_row = per_row;
  SampleF *sd = nullptr;
  PUMP_CUDA_TRY(pool_malloc_async((void **)&sd, sizeof(SampleF) * (size_t)N, stream));
  const int nprep = (N + 1023) / 1024;
  static_assert(kBracketSamples % kBracketPerBlock == 0, "whole bracket blocks");
  prepare_bracket_kernel<<<nprep + kBracketBlocks, 1024, 0, stream>>>(
      d_samples, N, tmax, nprep, sd, ps.rank, ps.sample_keys, ps.done, ps.key_hi);
  pump_status_t st = launch_status("prepare_bracket");
  if (st == PUMP_OK && between && cudaEventRecord(between, stream) != cudaSuccess)
    st = set_error(PUMP_ERR_CUDA, "cudaEventRecord");
  if (st == PUMP_OK) {
    const dim3 grid(nbx, (unsigned)N);
    bvp_pairs_masked_kernel<<<grid, kPairTile, 0, stream>>>(sd, N, tmax, d_copts, d_topts,
                                                           ps.key_hi, masks);
    st = launch_status("bvp_pairs_masked");
  }
  if (st == PUMP_OK && ps.after_pairs && cudaEventRecord(ps.after_pairs, stream) != cudaSuccess)
    st = set_error(PUMP_ERR_CUDA, "cudaEventRecord");
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
