// AABB collision checks and half-space caching (reference: sampler.cu:61-88,
// collisionCheck.cu, hsmc.cu, bvls.cu:259-273).
//
// Each block stages the obstacle set (numObs x 12 floats, lo[6] then hi[6])
// in shared memory with 16-byte loads, so the inner loops read boxes at
// shared-memory bandwidth instead of re-reading global memory per segment as
// the reference does.  The tests themselves are the reference's, operation
// for operation (binary32, no contraction): broadphase on the segment's
// bounding box, then the face-projection narrow phase with lambda not
// clamped to [0, 1], as in collisionCheck.cu:104-143.
#include <type_traits>

#include "common.cuh"

#include "collide.cuh"
#include "tune.h"

namespace pump {
namespace {

__global__ void sample_free_kernel(const float *__restrict__ obs, int numObs,
                                   const float *__restrict__ samples, int N,
                                   uint8_t *__restrict__ is_free) {
  extern __shared__ float4 s_obs4[];
  float *s_obs = reinterpret_cast<float *>(s_obs4);
  stage_obstacles(obs, numObs, s_obs);
  const int node = blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= N) return;
  float p[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) p[d] = samples[node * kDim + d];
  uint8_t fr = 1;
  for (int o = 0; o < numObs && fr; ++o) {
    const float *ob = &s_obs[o * 12];
    bool inside = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) inside = inside && p[d] > ob[d] && p[d] < ob[6 + d];
    if (inside) fr = 0;
  }
  is_free[node] = fr;
}

// halton, sampler.cu:43-57, in the same binary32 operations and order (this
// translation unit does not contract multiply-adds).
__device__ float halton_dev(int n, int b) {
  float hn = 0;
  int n0 = n;
  float f = 1 / ((float)b);
  while (n0 > 0) {
    float n1 = (float)(n0 / b);
    int r = (int)(n0 - n1 * b);
    hn += f * r;
    f = f / b;
    n0 = (int)n1;
  }
  return hn;
}

struct SampleBox {
  float lo[6], hi[6], init[6], goal[6];
};

// sampler.cu:20-41: sample n, dimension d = halton(n, base d) scaled into
// [lo, hi]; sample 0 is init and sample N-1 the goal, copied exactly.  With
// rows = N + 1 the goal row is written once more after the N samples.
__global__ void halton_kernel(int N, int rows, SampleBox bx, float *__restrict__ out) {
  const int bases[6] = {2, 3, 5, 7, 11, 13};
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)rows * kDim) return;
  const int n = (int)(t / kDim), d = (int)(t - (long long)n * kDim);
  float v;
  if (n == 0) v = bx.init[d];
  else if (n >= N - 1) v = bx.goal[d];
  else v = halton_dev(n, bases[d]) * (bx.hi[d] - bx.lo[d]) + bx.lo[d];
  out[t] = v;
}

// One thread per edge: freeEdges, collisionCheck.cu:5-37.
__global__ void __launch_bounds__(256) free_edges_kernel(const float *__restrict__ obs, int numObs,
                                                         const float *__restrict__ disc, long long E,
                                                         int numDisc,
                                                         uint8_t *__restrict__ is_free) {
  extern __shared__ float4 s_obs4[];
  float *s_obs = reinterpret_cast<float *>(s_obs4);
  stage_obstacles(obs, numObs, s_obs);
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= E) return;
  const float *wp = disc + e * (numDisc + 1) * kDim;
  float v[3], w[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) v[d] = __ldg(&wp[d]);
  bool ok = true;
  for (int i = 0; i < numDisc && ok; ++i) {
#pragma unroll
    for (int d = 0; d < 3; ++d) w[d] = __ldg(&wp[(i + 1) * kDim + d]);
    ok = segment_valid(v, w, numObs, s_obs);
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = w[d];
  }
  is_free[e] = ok ? 1 : 0;
}

// freeEdges (collisionCheck.cu:5-37) over the waypoints in disc, block of T
// edges: the block's waypoint positions (contiguous in disc) are staged in
// shared memory, then each warp tests its 32 edges with the pair queue of
// warp_queue_hits.  The block size T (64, 128, 256) is picked by the
// autotuner.
template <int T>
__global__ void __launch_bounds__(T) free_edges_queue_kernel(
    const float *__restrict__ obs, int numObs, const float *__restrict__ disc, long long E,
    int numDisc, uint8_t *__restrict__ is_free) {
  extern __shared__ float4 s_dyn4[];
  __shared__ int s_queue[T / 32][kQueueSlots];
  __shared__ uint8_t s_hit[T];
  float *s_obs = reinterpret_cast<float *>(s_dyn4);
  float *s_wp = s_obs + ((numObs * 12 + 3) & ~3);
  const int W = numDisc + 1;
  const long long e0 = blockIdx.x * (long long)T;
  const int nv = (int)(E - e0 < T ? E - e0 : T);
  {  // the block's waypoints are contiguous in disc; keep their positions
    // (24-byte records: an 8-byte load of x, y and a 4-byte load of z)
    const float *src = disc + e0 * W * kDim;
    for (int r = threadIdx.x; r < nv * W; r += T) {
      const float2 xy = __ldg(reinterpret_cast<const float2 *>(src + (long long)r * kDim));
      const float z = __ldg(src + (long long)r * kDim + 2);
      s_wp[r * 3] = xy.x;
      s_wp[r * 3 + 1] = xy.y;
      s_wp[r * 3 + 2] = z;
    }
  }
  stage_obstacles(obs, numObs, s_obs);  // ends with __syncthreads
  const int t = threadIdx.x, warp = t >> 5;
  const bool hit = warp_queue_hits(s_wp + warp * 32 * W * 3, W, s_obs, numObs, t < nv,
                                   s_queue[warp], s_hit + warp * 32);
  if (t < nv) is_free[e0 + t] = hit ? 0 : 1;
}

// free_edges_queue_kernel over the ragged waypoint layout: edge e's
// waypoints are records off[e] .. off[e+1]-1 (2 .. max_disc + 1 of them; a
// block holding an edge outside that range writes nothing and sets *error,
// when given, to PUMP_ERR_BAD_INPUT).  Each warp's lanes take their ranges
// from per-warp tables of first record and count.
template <int T>
__global__ void __launch_bounds__(T) free_edges_off_kernel(
    const float *__restrict__ obs, int numObs, const float *__restrict__ disc,
    const long long *__restrict__ off, long long E, int max_disc, uint8_t *__restrict__ is_free,
    int *error) {
  extern __shared__ float4 s_dyn4[];
  __shared__ int s_queue[T / 32][kQueueSlots];
  __shared__ uint8_t s_hit[T];
  __shared__ int s_first[T], s_cnt[T];
  float *s_obs = reinterpret_cast<float *>(s_dyn4);
  float *s_wp = s_obs + ((numObs * 12 + 3) & ~3);
  const long long e0 = blockIdx.x * (long long)T;
  const int nv = (int)(E - e0 < T ? E - e0 : T);
  const int t = threadIdx.x, warp = t >> 5;
  const long long base = off[e0];
  const long long cnt = t < nv ? off[e0 + t + 1] - off[e0 + t] : 0;
  if (__syncthreads_or(t < nv && (cnt < 2 || cnt > max_disc + 1))) {
    if (t == 0 && error) atomicExch(error, (int)PUMP_ERR_BAD_INPUT);
    return;
  }
  // lane ranges relative to the warp's first record
  const long long wbase = off[e0 + (warp * 32 < nv ? warp * 32 : 0)];
  s_first[t] = t < nv ? (int)(off[e0 + t] - wbase) : 0;
  s_cnt[t] = (int)cnt;
  const int total = (int)(off[e0 + nv] - base);
  {
    const float *src = disc + base * kDim;
    for (int r = t; r < total; r += T) {
      const float2 xy = __ldg(reinterpret_cast<const float2 *>(src + (long long)r * kDim));
      const float z = __ldg(src + (long long)r * kDim + 2);
      s_wp[r * 3] = xy.x;
      s_wp[r * 3 + 1] = xy.y;
      s_wp[r * 3 + 2] = z;
    }
  }
  stage_obstacles(obs, numObs, s_obs);  // ends with __syncthreads
  const bool hit = warp_queue_hits(s_wp + (wbase - base) * 3,
                                   RaggedLanes{s_first + warp * 32, s_cnt + warp * 32}, s_obs, numObs,
                                   t < nv, s_queue[warp], s_hit + warp * 32);
  if (t < nv) is_free[e0 + t] = hit ? 0 : 1;
}

// One thread per waypoint: setupAsBs (hsmc.cu:201-211) fused with
// cacheHalfspaces (hsmc.cu:10-99); unused slots get the defaults a = -1,
// b = 1111.
__global__ void __launch_bounds__(256) halfspace_kernel(const float *__restrict__ obs, int numObs,
                                                        const float *__restrict__ disc,
                                                        const uint8_t *__restrict__ is_free_edge,
                                                        long long E, int W, int maxHS, float maxd2,
                                                        float *__restrict__ as,
                                                        float *__restrict__ bs,
                                                        int *__restrict__ count) {
  extern __shared__ float4 s_obs4[];
  float *s_obs = reinterpret_cast<float *>(s_obs4);
  stage_obstacles(obs, numObs, s_obs);
  const long long wp = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (wp >= E * W) return;
  long long hsIdx = wp * maxHS;
  int stored = 0;
  if (is_free_edge[wp / W]) {
    float pos[3], vel[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      pos[d] = __ldg(&disc[wp * kDim + d]);
      vel[d] = __ldg(&disc[wp * kDim + 3 + d]);
    }
    for (int o = 0; o < numObs && stored < maxHS; ++o) {
      float a[3], b;
      if (!halfspace_of_box(pos, vel, &s_obs[o * 12], maxd2, a, &b)) continue;
#pragma unroll
      for (int d = 0; d < 3; ++d) as[hsIdx * 3 + d] = a[d];
      bs[hsIdx] = b;
      ++stored;
      ++hsIdx;
    }
  }
  for (long long h = hsIdx; h < (wp + 1) * maxHS; ++h) {
    as[h * 3 + 0] = -1.0f;
    as[h * 3 + 1] = -1.0f;
    as[h * 3 + 2] = -1.0f;
    bs[h] = 1111.0f;
  }
  if (count) count[wp] = stored;
}

// The same computation for a block of 256 consecutive waypoints, staged in
// shared memory: the block's waypoints (contiguous in disc) are loaded and
// its half-spaces (contiguous in as / bs) stored as whole lines.  Before the
// waypoints run, the boxes that cannot pass the distance gate anywhere on an
// edge are dropped once per edge: if for some axis the gap g between the
// edge's bounding box and the box has fl(g * g) > maxd2, every waypoint's
// d2 (a rounded sum of non-negative squares, each at least as large by the
// monotonicity of rounding) exceeds maxd2 as well.  Edges with a NaN
// waypoint, or maps with more than kFilterObs boxes, are not filtered.  The
// remaining boxes are visited in index order, so the first maxHS half-spaces
// are the reference's.  Used when maxHS <= kStagedMaxHS and the stage fits in
// shared memory.
constexpr int kStagedMaxHS = 8;
constexpr int kHsThreads = 256;
constexpr int kHsMaxEdges = kHsThreads / 2 + 2;  // W >= 2

// Dense: every slot written (unused ones get the defaults), int counts.
// Sparse (!Dense): only the stored half-spaces are written, straight to
// global memory, with one-byte counts; slots at or past a waypoint's count
// are left as they are (their readers stop at the count).
template <bool Dense>
__global__ void __launch_bounds__(kHsThreads) halfspace_staged_kernel(
    const float *__restrict__ obs, int numObs, const float *__restrict__ disc,
    const uint8_t *__restrict__ is_free_edge, long long E, int W, int maxHS, float maxd2,
    float *__restrict__ as, float *__restrict__ bs, int *__restrict__ count,
    uint8_t *__restrict__ count8) {
  extern __shared__ float4 s_dyn4[];
  __shared__ float s_eb[kHsMaxEdges][6];  // edge bounding box: min[3], max[3]
  __shared__ uint32_t s_mask[kHsMaxEdges][kFilterObs / 32];
  __shared__ uint8_t s_filter[kHsMaxEdges];  // 1: free edge whose boxes are filtered
  float *s_obs = reinterpret_cast<float *>(s_dyn4);
  float *s_wp = s_obs + ((numObs * 12 + 3) & ~3);
  float *s_a = s_wp + kHsThreads * kDim;
  float *s_b = s_a + kHsThreads * maxHS * 3;
  stage_obstacles(obs, numObs, s_obs);
  const long long wp0 = blockIdx.x * (long long)kHsThreads;
  const long long total = E * W;
  const int nv = (int)(total - wp0 < kHsThreads ? total - wp0 : kHsThreads);
  const long long e0 = wp0 / W;
  const int ne = (int)((wp0 + nv - 1) / W - e0) + 1;
  const int t = threadIdx.x;
  block_load(s_wp, disc + wp0 * kDim, nv * kDim);
  const bool filter = numObs <= kFilterObs;
  if (t < ne) {
    const long long e = e0 + t;
    bool use = filter && is_free_edge[e];
    float mn[3], mx[3];
    const float *w = disc + e * W * kDim;
#pragma unroll
    for (int d = 0; d < 3; ++d) mn[d] = mx[d] = __ldg(&w[d]);
    for (int i = 0; i < W; ++i)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float x = __ldg(&w[i * kDim + d]);
        use = use && x == x;
        mn[d] = fminf(mn[d], x);
        mx[d] = fmaxf(mx[d], x);
      }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      s_eb[t][d] = mn[d];
      s_eb[t][3 + d] = mx[d];
    }
    s_filter[t] = use;
#pragma unroll
    for (int k = 0; k < kFilterObs / 32; ++k) s_mask[t][k] = 0u;
  }
  __syncthreads();
  if (filter) {
    // (edge, box) pairs of the block: keep the boxes the gate can pass
    for (int q = t; q < ne * numObs; q += kHsThreads) {
      const int el = q / numObs, o = q - el * numObs;
      if (!s_filter[el]) continue;
      const bool keep = gate_keeps_box(s_eb[el], s_eb[el] + 3, &s_obs[o * 12], maxd2);
      if (keep) atomicOr(&s_mask[el][o >> 5], 1u << (o & 31));
    }
  }
  __syncthreads();
  if (t < nv) {
    const long long wp = wp0 + t;
    const int el = (int)(wp / W - e0);
    float *a = Dense ? s_a + t * maxHS * 3 : as + wp * maxHS * 3;
    float *b = Dense ? s_b + t * maxHS : bs + wp * maxHS;
    int stored = 0;
    if (is_free_edge[wp / W]) {
      float pos[3], vel[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        pos[d] = s_wp[t * kDim + d];
        vel[d] = s_wp[t * kDim + 3 + d];
      }
      const bool filt = s_filter[el];
      const int words = filt ? (numObs + 31) / 32 : 0;
      int o = -1;
      uint32_t m = 0u;
      int k = 0;
      while (stored < maxHS) {
        // next box in index order: from the edge's mask, or every box
        if (filt) {
          while (m == 0u && k < words) m = s_mask[el][k++];
          if (m == 0u) break;
          o = (k - 1) * 32 + __ffs(m) - 1;
          m &= m - 1;
        } else {
          if (++o >= numObs) break;
        }
        float ah[3], bh;
        if (!halfspace_of_box(pos, vel, &s_obs[o * 12], maxd2, ah, &bh)) continue;
#pragma unroll
        for (int d = 0; d < 3; ++d) a[stored * 3 + d] = ah[d];
        b[stored] = bh;
        ++stored;
      }
    }
    if (Dense) {
      for (int h = stored; h < maxHS; ++h) {
        a[h * 3 + 0] = -1.0f;
        a[h * 3 + 1] = -1.0f;
        a[h * 3 + 2] = -1.0f;
        b[h] = 1111.0f;
      }
      if (count) count[wp] = stored;
    } else {
      count8[wp] = (uint8_t)stored;
    }
  }
  if (Dense) {
    __syncthreads();
    block_store(as + wp0 * maxHS * 3, s_a, nv * maxHS * 3);
    block_store(bs + wp0 * maxHS, s_b, nv * maxHS);
  }
}

size_t halfspace_staged_smem(int numObs, int maxHS, bool dense) {
  return sizeof(float) * ((size_t)((numObs * 12 + 3) & ~3) + (size_t)kHsThreads * kDim +
                          (dense ? (size_t)kHsThreads * maxHS * 4 : 0));
}

pump_status_t obstacle_smem(int numObs, size_t *bytes) {
  *bytes = (size_t)numObs * 12 * sizeof(float);
  if (*bytes > 200 * 1024)
    return set_error(PUMP_ERR_CAPACITY, "%d obstacles exceed the shared-memory stage", numObs);
  return PUMP_OK;
}

}  // namespace

pump_status_t halton_samples_async(int N, const float *lo, const float *hi, const float *init,
                                   const float *goal, float *d_out, cudaStream_t stream,
                                   bool goal_row) {
  const int rows = goal_row ? N + 1 : N;
  SampleBox bx;
  for (int d = 0; d < 6; ++d) {
    bx.lo[d] = lo[d];
    bx.hi[d] = hi[d];
    bx.init[d] = init[d];
    bx.goal[d] = goal[d];
  }
  halton_kernel<<<grid_for((long long)rows * kDim, 256), 256, 0, stream>>>(N, rows, bx, d_out);
  return launch_status("halton_kernel");
}

}  // namespace pump

using namespace pump;

extern "C" pump_status_t pump_halton_samples(int N, const float *lo, const float *hi,
                                             const float *init, const float *goal,
                                             float *d_samples, pump_stream_t stream) {
  if (N < 2 || !lo || !hi || !init || !goal || !d_samples)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_halton_samples: bad arguments");
  return halton_samples_async(N, lo, hi, init, goal, d_samples, (cudaStream_t)stream, false);
}

extern "C" pump_status_t pump_sample_free(const float *d_obstacles, int numObs,
                                          const float *d_samples, int N, uint8_t *d_is_free,
                                          pump_stream_t stream) {
  if (numObs < 0 || N < 0 || (numObs > 0 && !d_obstacles) || (N > 0 && (!d_samples || !d_is_free)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_sample_free: bad arguments");
  if (N == 0) return PUMP_OK;
  size_t smem;
  PUMP_TRY(obstacle_smem(numObs, &smem));
  PUMP_TRY(smem_attr((const void *)sample_free_kernel, smem));
  sample_free_kernel<<<grid_for(N, 256), 256, smem, (cudaStream_t)stream>>>(d_obstacles, numObs,
                                                                          d_samples, N, d_is_free);
  return launch_status("sample_free");
}

extern "C" pump_status_t pump_free_edges(const float *d_obstacles, int numObs, const float *d_disc,
                                         long long E, int numDisc, uint8_t *d_is_free,
                                         pump_stream_t stream) {
  if (numObs < 0 || E < 0 || numDisc < 1 || (numObs > 0 && !d_obstacles) ||
      (E > 0 && (!d_disc || !d_is_free)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_free_edges: bad arguments");
  if (E == 0) return PUMP_OK;
  size_t smem;
  PUMP_TRY(obstacle_smem(numObs, &smem));
  auto staged = [&](int T) {
    return sizeof(float) * ((size_t)((numObs * 12 + 3) & ~3) + (size_t)T * (numDisc + 1) * 3);
  };
  if (staged(256) <= 200 * 1024 && numObs <= 0xFFFF) {
    cudaStream_t s = (cudaStream_t)stream;
    auto go = [&](auto block) -> pump_status_t {
      constexpr int T = decltype(block)::value;
      PUMP_TRY(smem_attr((const void *)free_edges_queue_kernel<T>, staged(T)));
      free_edges_queue_kernel<T><<<grid_for(E, T), T, staged(T), s>>>(d_obstacles, numObs, d_disc,
                                                                     E, numDisc, d_is_free);
      return launch_status("free_edges");
    };
    // block sizes 64, 128 (default), 256
    auto run = [&](int c) -> pump_status_t {
      if (c == 0) return go(std::integral_constant<int, 64>{});
      if (c == 1) return go(std::integral_constant<int, 128>{});
      return go(std::integral_constant<int, 256>{});
    };
    int choice = 1;
    bool ran = false;
    const uint64_t key = ((uint64_t)numDisc << 32) | tune_bucket(numObs);
    PUMP_TRY(tune_choice(kTuneFreeEdges, key, 3, 1, s, run, &choice, &ran));
    return ran ? PUMP_OK : run(choice);
  }
  PUMP_TRY(smem_attr((const void *)free_edges_kernel, smem));
  free_edges_kernel<<<grid_for(E, 256), 256, smem, (cudaStream_t)stream>>>(d_obstacles, numObs,
                                                                         d_disc, E, numDisc,
                                                                         d_is_free);
  return launch_status("free_edges");
}

namespace pump {
pump_status_t free_edges_off_async(const float *d_obstacles, int numObs, const float *d_disc,
                                   const long long *d_off, long long E, int max_disc,
                                   uint8_t *d_is_free, cudaStream_t s, int *error) {
  if (E <= 0) return PUMP_OK;
  constexpr int T = 128;
  const size_t smem = sizeof(float) * ((size_t)((numObs * 12 + 3) & ~3) + (size_t)T * (max_disc + 1) * 3);
  if (smem > 200 * 1024 || numObs > 0xFFFF)
    return set_error(PUMP_ERR_CAPACITY, "%d boxes and %d waypoints per edge exceed the edge check's stage",
                     numObs, max_disc + 1);
  PUMP_TRY(smem_attr((const void *)free_edges_off_kernel<T>, smem));
  free_edges_off_kernel<T><<<grid_for(E, T), T, smem, s>>>(d_obstacles, numObs, d_disc, d_off, E,
                                                          max_disc, d_is_free, error);
  return launch_status("free_edges_off");
}
}  // namespace pump

extern "C" pump_status_t pump_free_edges_off(const float *d_obstacles, int numObs, const float *d_disc,
                                             const long long *d_off, long long E, int max_disc,
                                             uint8_t *d_is_free, pump_stream_t stream) {
  if (numObs < 0 || E < 0 || max_disc < 1 || (numObs > 0 && !d_obstacles) ||
      (E > 0 && (!d_disc || !d_off || !d_is_free)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_free_edges_off: bad arguments");
  if (E == 0) return PUMP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int *d_err = nullptr;
  PUMP_CUDA_TRY(pool_malloc_async((void **)&d_err, sizeof(int), s));
  pump_status_t st = cuda_status(cudaMemsetAsync(d_err, 0, sizeof(int), s), "cudaMemsetAsync");
  if (st == PUMP_OK) st = free_edges_off_async(d_obstacles, numObs, d_disc, d_off, E, max_disc, d_is_free, s, d_err);
  int err = 0;
  if (st == PUMP_OK)
    st = cuda_status(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
  cudaFreeAsync(d_err, s);
  if (st == PUMP_OK) st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  PUMP_TRY(st);
  if (err)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_free_edges_off: an edge's waypoint count is outside "
                                         "[2, max_disc + 1]");
  return PUMP_OK;
}

extern "C" pump_status_t pump_cache_halfspaces(const float *d_obstacles, int numObs,
                                               const float *d_disc, const uint8_t *d_is_free_edge,
                                               long long E, int W, int maxHS, float maxd2,
                                               float *d_as, float *d_bs, int *d_count,
                                               pump_stream_t stream) {
  if (numObs < 0 || E < 0 || W < 2 || maxHS < 0 || (numObs > 0 && !d_obstacles) ||
      (E > 0 && maxHS > 0 && (!d_disc || !d_is_free_edge || !d_as || !d_bs)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_cache_halfspaces: bad arguments");
  if (E == 0) return PUMP_OK;
  if (maxHS == 0) {
    if (d_count) PUMP_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(int) * E * W, (cudaStream_t)stream));
    return PUMP_OK;
  }
  size_t smem;
  PUMP_TRY(obstacle_smem(numObs, &smem));
  const size_t staged = halfspace_staged_smem(numObs, maxHS, true);
  if (maxHS <= kStagedMaxHS && staged <= 220 * 1024) {
    PUMP_TRY(smem_attr((const void *)halfspace_staged_kernel<true>, staged));
    halfspace_staged_kernel<true><<<grid_for(E * W, kHsThreads), kHsThreads, staged,
                                    (cudaStream_t)stream>>>(
        d_obstacles, numObs, d_disc, d_is_free_edge, E, W, maxHS, maxd2, d_as, d_bs, d_count,
        nullptr);
    return launch_status("cache_halfspaces");
  }
  PUMP_TRY(smem_attr((const void *)halfspace_kernel, smem));
  halfspace_kernel<<<grid_for(E * W, 256), 256, smem, (cudaStream_t)stream>>>(
      d_obstacles, numObs, d_disc, d_is_free_edge, E, W, maxHS, maxd2, d_as, d_bs, d_count);
  return launch_status("cache_halfspaces");
}

extern "C" pump_status_t pump_cache_halfspaces_sparse(const float *d_obstacles, int numObs,
                                                      const float *d_disc,
                                                      const uint8_t *d_is_free_edge, long long E,
                                                      int W, int maxHS, float maxd2, float *d_as,
                                                      float *d_bs, uint8_t *d_count,
                                                      pump_stream_t stream) {
  if (numObs < 0 || E < 0 || W < 2 || maxHS < 0 || maxHS > kStagedMaxHS ||
      (numObs > 0 && !d_obstacles) ||
      (E > 0 && (!d_disc || !d_is_free_edge || !d_count || (maxHS > 0 && (!d_as || !d_bs)))))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_cache_halfspaces_sparse: bad arguments");
  if (E == 0) return PUMP_OK;
  if (maxHS == 0) {
    PUMP_CUDA_TRY(cudaMemsetAsync(d_count, 0, (size_t)E * W, (cudaStream_t)stream));
    return PUMP_OK;
  }
  const size_t staged = halfspace_staged_smem(numObs, maxHS, false);
  if (staged > 220 * 1024)
    return set_error(PUMP_ERR_CAPACITY, "%d obstacles exceed the shared-memory stage", numObs);
  PUMP_TRY(smem_attr((const void *)halfspace_staged_kernel<false>, staged));
  halfspace_staged_kernel<false><<<grid_for(E * W, kHsThreads), kHsThreads, staged,
                                   (cudaStream_t)stream>>>(
      d_obstacles, numObs, d_disc, d_is_free_edge, E, W, maxHS, maxd2, d_as, d_bs, nullptr,
      d_count);
  return launch_status("cache_halfspaces_sparse");
}
