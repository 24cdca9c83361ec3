// AABB collision primitives shared by the edge check (collide.cu) and the
// Monte Carlo CP kernel (hsmc.cu).  Obstacles are numObs x 12 floats, lo[6]
// then hi[6]; only the three position dimensions are tested, as in the
// reference (collisionCheck.cu:104-143).
#pragma once

#include "common.cuh"

namespace pump {

// Cooperative copy of the obstacle array into shared memory (48 B per box,
// so 16-byte vector loads always apply when the base is 16-byte aligned).
__device__ __forceinline__ void stage_obstacles(const float *__restrict__ obs, int numObs,
                                                float *s_obs) {
  const int n = numObs * 12;
  if ((reinterpret_cast<uintptr_t>(obs) & 15) == 0) {
    const float4 *src = reinterpret_cast<const float4 *>(obs);
    float4 *dst = reinterpret_cast<float4 *>(s_obs);
    for (int i = threadIdx.x; i < n / 4; i += blockDim.x) dst[i] = __ldg(&src[i]);
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s_obs[i] = __ldg(&obs[i]);
  }
  __syncthreads();
}

// broadphaseValidQ, collisionCheck.cu:104-112
__device__ __forceinline__ bool broadphase_valid(const float *bbMin, const float *bbMax,
                                                 const float *o) {
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (bbMax[d] <= o[d] || o[6 + d] <= bbMin[d]) return true;
  return false;
}

// faceContainsProjection, collisionCheck.cu:133-143
__device__ __forceinline__ bool face_contains_projection(const float *v, const float *w, float lambda,
                                                         int j, const float *o) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float projection = v[d] + (w[d] - v[d]) * lambda;
    if (d != j && !(o[d] <= projection && projection <= o[6 + d])) return false;
  }
  return true;
}

// motionValidQ, collisionCheck.cu:114-131
__device__ __forceinline__ bool motion_valid(const float *v, const float *w, const float *o) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float v_to_w = w[d] - v[d];
    const float lambda = (v[d] < o[d]) ? (o[d] - v[d]) / v_to_w : (o[6 + d] - v[d]) / v_to_w;
    if (face_contains_projection(v, w, lambda, d, o)) return false;
  }
  return true;
}

// isMotionValid, collisionCheck.cu:65-102 (positions only).
__device__ __forceinline__ bool segment_valid(const float *v, const float *w, int numObs, const float *s_obs) {
  float bbMin[3], bbMax[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (v[d] > w[d]) { bbMin[d] = w[d]; bbMax[d] = v[d]; }
    else { bbMin[d] = v[d]; bbMax[d] = w[d]; }
  }
  for (int o = 0; o < numObs; ++o) {
    const float *ob = &s_obs[o * 12];
    if (!broadphase_valid(bbMin, bbMax, ob) && !motion_valid(v, w, ob)) return false;
  }
  return true;
}

// isMotionValid over the boxes whose bits are set in mask (box o is bit
// o % 32 of mask[o / 32]), in index order.  A box that is broadphase-disjoint
// from the whole edge's bounding box is disjoint from every segment's, so
// dropping it from the mask beforehand leaves the result unchanged.
__device__ __forceinline__ bool segment_valid_masked(const float *v, const float *w,
                                                     const uint32_t *mask, int words,
                                                     const float *s_obs) {
  float bbMin[3], bbMax[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (v[d] > w[d]) { bbMin[d] = w[d]; bbMax[d] = v[d]; }
    else { bbMin[d] = v[d]; bbMax[d] = w[d]; }
  }
  for (int k = 0; k < words; ++k) {
    uint32_t m = mask[k];
    while (m) {
      const int o = k * 32 + __ffs(m) - 1;
      m &= m - 1;
      const float *ob = &s_obs[o * 12];
      if (!broadphase_valid(bbMin, bbMax, ob) && !motion_valid(v, w, ob)) return false;
    }
  }
  return true;
}

}  // namespace pump
