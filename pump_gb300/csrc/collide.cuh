// AABB collision primitives shared by the edge check (collide.cu) and the
// Monte Carlo CP kernel (hsmc.cu).  Obstacles are numObs x 12 floats, lo[6]
// then hi[6]; only the three position dimensions are tested, as in the
// reference (collisionCheck.cu:104-143).
#pragma once

#include "common.cuh"

namespace pump {

// Edge-level box filters keep one bit per box in registers for maps of up to
// this many boxes (more boxes: every box is tested).
constexpr int kFilterObs = 128;

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

// One (segment, box) test of isMotionValid's loop (collisionCheck.cu:65-102):
// true when the segment v-w hits box ob.  isMotionValid is the AND of
// !segment_box_hit over its boxes, so any split of the boxes among threads
// gives the same result.
__device__ __forceinline__ bool segment_box_hit(const float *v, const float *w, const float *ob) {
  float bbMin[3], bbMax[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (v[d] > w[d]) { bbMin[d] = w[d]; bbMax[d] = v[d]; }
    else { bbMin[d] = v[d]; bbMax[d] = w[d]; }
  }
  return !broadphase_valid(bbMin, bbMax, ob) && !motion_valid(v, w, ob);
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

// The half-space box o contributes at a waypoint (pos, vel): cacheHalfspaces,
// hsmc.cu:10-99, with bvlsShortcut (bvls.cu:259-273) for the closest point.
// False when the point is farther than the distance gate (d2 > maxd2);
// otherwise a[3] and b = a.a.  Every operation in the reference's order
// (binary32; the callers' translation units do not contract).
__device__ __forceinline__ bool halfspace_of_box(const float *pos, const float *vel,
                                                 const float *box, float maxd2, float *a,
                                                 float *b) {
  const float *l = box, *u = box + 6;
  float x[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (pos[d] <= l[d]) x[d] = l[d];
    else if (pos[d] >= u[d]) x[d] = u[d];
    else x[d] = pos[d];
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) x[d] = x[d] - pos[d];
  float d2 = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) d2 += x[d] * x[d];
  if (d2 > maxd2) return false;
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
    a[d] = x[d];
    xdotx += x[d] * x[d];
  }
  *b = xdotx;
  return true;
}

// Whether box can pass the distance gate at some waypoint of an edge whose
// waypoints lie in [emin, emax]: if for some axis the gap g between that
// bounding box and the box has fl(g * g) > maxd2, every waypoint's d2 (a
// rounded sum of non-negative squares, each at least as large by the
// monotonicity of rounding) exceeds maxd2 as well.
__device__ __forceinline__ bool gate_keeps_box(const float *emin, const float *emax,
                                               const float *box, float maxd2) {
  const float *l = box, *u = box + 6;
  bool keep = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float above = l[d] - emax[d];  // box beyond the edge's max
    const float below = u[d] - emin[d];  // box below the edge's min
    if (above > 0.0f && above * above > maxd2) keep = false;
    if (below < 0.0f && below * below > maxd2) keep = false;
  }
  return keep;
}

}  // namespace pump
