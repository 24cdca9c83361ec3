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

// Slots of the per-warp ring of (edge, box) pairs of warp_queue_hits.
constexpr int kQueueSlots = 64;

// freeEdges's test (collisionCheck.cu:5-143) for the 32 edges of one warp:
// lane l holds edge l (when active), its W waypoint positions at
// s_wp_warp + l * W * 3 in shared memory; the boxes are at s_obs.  Each
// lane takes the bounding box of its edge's waypoints.  Then the warp walks
// the boxes in order: the edges whose bounding box a box is not
// broadphase-disjoint from (every edge when a waypoint is NaN) append the
// pair (edge, box) to the warp's ring q, and whenever 32 pairs are queued
// the warp tests them, one pair per lane: the pair's segments against its
// box, the reference's (segment, box) test.  The reference's result is the
// AND over the (segment, box) pairs, and a box disjoint from the edge's
// bounding box passes for every segment, so the filter and the order change
// no result; the queue keeps the lanes busy where per-lane box lists would
// leave most of a warp waiting for its longest list.  q: the warp's
// kQueueSlots ints, hit: its 32 bytes, both in shared memory.  Returns
// whether this lane's edge hits a box.
//
// The lanes' waypoint ranges come from a layout: every edge W waypoints
// (UniformLanes: lane l's at record l * W), or per-edge counts (RaggedLanes:
// first record and count per lane, in per-warp shared arrays).
struct UniformLanes {
  int W;
  __device__ int first(int l) const { return l * W; }
  __device__ int count(int) const { return W; }
};
struct RaggedLanes {
  const int *f, *c;  // per lane: first staged record, waypoint count
  __device__ int first(int l) const { return f[l]; }
  __device__ int count(int l) const { return c[l]; }
};
// per-lane ranges from staged offsets: lane l's records o[l] - o[0] ..
// o[l+1] - o[0] - 1
struct OffsetLanes {
  const int *o;
  __device__ int first(int l) const { return o[l] - o[0]; }
  __device__ int count(int l) const { return o[l + 1] - o[l]; }
};

template <class Lanes>
__device__ __forceinline__ bool warp_queue_hits(const float *s_wp_warp, Lanes lay, const float *s_obs,
                                                int numObs, bool active, int *q, uint8_t *hit) {
  constexpr int kPos = 3;  // floats per staged waypoint
  const int lane = threadIdx.x & 31;
  const unsigned int lt = (1u << lane) - 1u;
  hit[lane] = 0;
  __syncwarp();
  float emin[3], emax[3];
  bool nan = false;
  if (active) {
    const float *wp = s_wp_warp + lay.first(lane) * kPos;
    const int W = lay.count(lane);
#pragma unroll
    for (int d = 0; d < 3; ++d) emin[d] = emax[d] = wp[d];
    for (int i = 0; i < W; ++i)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float x = wp[i * kPos + d];
        nan = nan || x != x;
        emin[d] = fminf(emin[d], x);
        emax[d] = fmaxf(emax[d], x);
      }
  }
  // one queued pair: the edge's lane (high half), the box
  auto test_pair = [&](int ent) {
    const int el = ent >> 16, o = ent & 0xFFFF;
    if (hit[el]) return;  // the edge already hit a box
    const float *wp = s_wp_warp + lay.first(el) * kPos;
    const int numDisc = lay.count(el) - 1;
    const float *ob = &s_obs[o * 12];
    float v[3], w[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = wp[d];
    for (int i = 0; i < numDisc; ++i) {
#pragma unroll
      for (int d = 0; d < 3; ++d) w[d] = wp[(i + 1) * kPos + d];
      if (segment_box_hit(v, w, ob)) {
        hit[el] = 1;
        return;
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) v[d] = w[d];
    }
  };
  int head = 0, tail = 0;  // warp-uniform
  const float4 *s_obs4 = reinterpret_cast<const float4 *>(s_obs);
  for (int o = 0; o < numObs; ++o) {
    // broadphaseValidQ of the edge's bounding box, without branches: box o
    // is lo = (x0, y0, z0) at floats 0-2 and hi = (x1, y1, z1) at floats 6-8
    const float4 a = s_obs4[o * 3], b = s_obs4[o * 3 + 1], c = s_obs4[o * 3 + 2];
    const bool disjoint = (emax[0] <= a.x) | (b.z <= emin[0]) | (emax[1] <= a.y) |
                          (b.w <= emin[1]) | (emax[2] <= a.z) | (c.x <= emin[2]);
    const bool need = active && (nan || !disjoint);
    const unsigned int bal = __ballot_sync(0xffffffffu, need);
    if (need) q[(tail + __popc(bal & lt)) & (kQueueSlots - 1)] = (lane << 16) | o;
    tail += __popc(bal);
    if (tail - head >= 32) {
      __syncwarp();
      test_pair(q[(head + lane) & (kQueueSlots - 1)]);
      head += 32;
      __syncwarp();  // the slots just taken are rewritten by later boxes
    }
  }
  __syncwarp();
  if (lane < tail - head) test_pair(q[(head + lane) & (kQueueSlots - 1)]);
  __syncwarp();
  return hit[lane] != 0;
}

__device__ __forceinline__ bool warp_queue_hits(const float *s_wp_warp, int W, const float *s_obs,
                                                int numObs, bool active, int *q, uint8_t *hit) {
  return warp_queue_hits(s_wp_warp, UniformLanes{W}, s_obs, numObs, active, q, hit);
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
