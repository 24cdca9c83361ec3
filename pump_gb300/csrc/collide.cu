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
#include "common.cuh"

#include "collide.cuh"

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
      const float *l = &s_obs[o * 12], *u = l + 6;
      float x[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {  // bvlsShortcut, bvls.cu:259-273
        if (pos[d] <= l[d]) x[d] = l[d];
        else if (pos[d] >= u[d]) x[d] = u[d];
        else x[d] = pos[d];
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) x[d] = x[d] - pos[d];
      float d2 = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) d2 += x[d] * x[d];
      if (d2 > maxd2) continue;
      float xdotv = 0, vdotv = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        xdotv += x[d] * vel[d];
        vdotv += vel[d] * vel[d];
      }
      if (vdotv == 0) vdotv = (float)1e-5;
      const float dotratio = xdotv / vdotv;
#pragma unroll
      for (int d = 0; d < 3; ++d) x[d] = x[d] - dotratio * vel[d];
      float xdotx = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        as[hsIdx * 3 + d] = x[d];
        xdotx += x[d] * x[d];
      }
      bs[hsIdx] = xdotx;
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

pump_status_t obstacle_smem(int numObs, size_t *bytes) {
  *bytes = (size_t)numObs * 12 * sizeof(float);
  if (*bytes > 200 * 1024)
    return set_error(PUMP_ERR_CAPACITY, "%d obstacles exceed the shared-memory stage", numObs);
  return PUMP_OK;
}

pump_status_t set_smem_attr(const void *fn, size_t bytes) {
  if (bytes > 48 * 1024)
    PUMP_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return PUMP_OK;
}

}  // namespace
}  // namespace pump

using namespace pump;

extern "C" pump_status_t pump_sample_free(const float *d_obstacles, int numObs,
                                          const float *d_samples, int N, uint8_t *d_is_free,
                                          pump_stream_t stream) {
  if (numObs < 0 || N < 0 || (numObs > 0 && !d_obstacles) || (N > 0 && (!d_samples || !d_is_free)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_sample_free: bad arguments");
  if (N == 0) return PUMP_OK;
  size_t smem;
  PUMP_TRY(obstacle_smem(numObs, &smem));
  PUMP_TRY(set_smem_attr((const void *)sample_free_kernel, smem));
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
  PUMP_TRY(set_smem_attr((const void *)free_edges_kernel, smem));
  free_edges_kernel<<<grid_for(E, 256), 256, smem, (cudaStream_t)stream>>>(d_obstacles, numObs,
                                                                         d_disc, E, numDisc,
                                                                         d_is_free);
  return launch_status("free_edges");
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
  PUMP_TRY(set_smem_attr((const void *)halfspace_kernel, smem));
  halfspace_kernel<<<grid_for(E * W, 256), 256, smem, (cudaStream_t)stream>>>(
      d_obstacles, numObs, d_disc, d_is_free_edge, E, W, maxHS, maxd2, d_as, d_bs, d_count);
  return launch_status("cache_halfspaces");
}
