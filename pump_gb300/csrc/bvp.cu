// Two-point BVP of the 3D double integrator: optimal time, cost and edge
// waypoints (reference: 2pBVP.cu).
//
// Parity mode evaluates the reference's cost expression (2pBVP.cu:97-107)
// term by term in its own evaluation types, with the pair-dependent,
// tau-independent sub-expressions hoisted out of the bisection loop: each
// hoisted value is computed by exactly the same operations the expression
// performs, so every rounding is unchanged and only repeated work is
// removed.  The finite-difference bisection (2pBVP.cu:71-95) is replicated
// step for step.  Cost evaluation is binary64-bound (the expression promotes
// through pow(double)), so these kernels are limited by the FP64 pipe.
//
// The precision-mode minimiser (closed form, binary64 refinement) is in
// bvp_precise.cu, compiled with multiply-add contraction.
#include <math.h>

#include <type_traits>

#include "common.cuh"
#include "ffcost.cuh"
#include "ctx.h"
#include "pathpoint.cuh"
#include "tune.h"

namespace pump {
namespace {

// ---------------------------------------------------------------- parity
// binary32 -> binary64 conversion, exact, on the integer pipe: the binary64
// bit pattern of a normal binary32 (or a zero) is its sign, its exponent
// rebiased by 1023 - 127 and its 23 mantissa bits shifted up by 29.
// Subnormal, infinite and NaN inputs take the hardware conversion.  On this
// GPU the binary64 pipe, which also executes conversions, bounds the parity
// kernel, so moving them to integer instructions shortens it.
__device__ __forceinline__ double f2d(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int e = (u >> 23) & 0xFFu;
  if (e == 0xFFu || (e == 0u && (u & 0x7FFFFFu) != 0u)) return (double)f;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  if (e == 0u) return __longlong_as_double((long long)sign);  // +-0
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e + (1023u - 127u)) << 52) |
                                          ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

// The bisection's stopping test compares a binary32 |dcval| with the
// binary64 constant 0.0001 (2pBVP.cu:86).  binary32 0.0001f is below 0.0001
// and the next binary32 above it, so (double)x > 0.0001 exactly when
// x > 0.0001f (NaN false either way): the test runs in binary32.
constexpr float kDcvalTol = 0.0001f;

struct PairCoef {
  double s7;                                     // first seven (tau-free) terms
  float k8, k9, k10, k11, k12, k13, k14, k15;    // float prefixes of the t-linear terms
  double d16, d17, d18, d20, d22, d24;           // 4*pow(x,2) coefficients of t^2
  double f19, f21, f23;                          // 4*x*y binary32 coefficients of t^2, converted
  double f25, f26;                               // 2*g*x binary32 coefficients of t^3, converted
  float a29, b29, c29, a30, b30, c30;            // last two float terms
};

__device__ __forceinline__ PairCoef make_coef(const float *x0, const float *x1) {
  const float g = PUMP_G;
  PairCoef c;
  double s = 12 * p2f(x0[0]);
  s = s + 12 * p2f(x0[2]);
  s = s + 12 * p2f(x0[1]);
  s = s + 12 * p2f(x1[0]);
  s = s + 12 * p2f(x1[2]);
  s = s - (double)(24 * x0[1] * x1[1]);
  s = s + 12 * p2f(x1[1]);
  c.s7 = s;
  c.k8 = 12 * x0[4] * x0[1];
  c.k9 = 12 * x0[1] * x1[4];
  c.k10 = 12 * x0[3] * x1[0];
  c.k11 = 12 * x1[3] * x1[0];
  c.k12 = 12 * x0[5] * x1[2];
  c.k13 = 12 * x1[5] * x1[2];
  c.k14 = 12 * x0[4] * x1[1];
  c.k15 = 12 * x1[4] * x1[1];
  c.d16 = 4 * p2f(x0[4]);
  c.d17 = 4 * p2f(x0[3]);
  c.d18 = 4 * p2f(x0[5]);
  c.f19 = f2d(4 * x0[4] * x1[4]);
  c.d20 = 4 * p2f(x1[4]);
  c.f21 = f2d(4 * x0[3] * x1[3]);
  c.d22 = 4 * p2f(x1[3]);
  c.f23 = f2d(4 * x0[5] * x1[5]);
  c.d24 = 4 * p2f(x1[5]);
  c.f25 = f2d(2 * g * x0[5]);
  c.f26 = f2d(2 * g * x1[5]);
  c.a29 = 12 * x0[0];
  c.b29 = -2 * x1[0];
  c.c29 = x0[3] + x1[3];
  c.a30 = 12 * x0[2];
  c.b30 = -2 * x1[2];
  c.c30 = x0[5] + x1[5];
  return c;
}

// cost(tau, x0, x1), 2pBVP.cu:97-107, term order preserved.
__device__ __forceinline__ float cost_eval(const PairCoef &c, float tau) {
  const double g2 = p2f(PUMP_G);
  const double dt = f2d(tau);
  const double t2 = dt * dt, t3 = t2 * dt, t4 = t2 * t2;
  double s = c.s7;
  s = s + f2d(c.k8 * tau);
  s = s + f2d(c.k9 * tau);
  s = s - f2d(c.k10 * tau);
  s = s - f2d(c.k11 * tau);
  s = s - f2d(c.k12 * tau);
  s = s - f2d(c.k13 * tau);
  s = s - f2d(c.k14 * tau);
  s = s - f2d(c.k15 * tau);
  s = s + c.d16 * t2;
  s = s + c.d17 * t2;
  s = s + c.d18 * t2;
  s = s + c.f19 * t2;
  s = s + c.d20 * t2;
  s = s + c.f21 * t2;
  s = s + c.d22 * t2;
  s = s + c.f23 * t2;
  s = s + c.d24 * t2;
  s = s + c.f25 * t3;
  s = s - c.f26 * t3;
  s = s + t4;
  s = s + g2 * t4;
  s = s + f2d(c.a29 * (c.b29 + c.c29 * tau));
  s = s + f2d(c.a30 * (c.b30 + c.c30 * tau));
  return (float)((1.0 / t3) * s);
}

// ------------------------------------------- the cost off the binary64 pipe
// (ffcost.cuh: cost_ff, PairFF)
__device__ __forceinline__ float cost_fast(const PairCoef &c, const PairFF &f, float tau) {
  bool ok;
  const float v = cost_ff(f, tau, &ok);
  return ok ? v : cost_eval(c, tau);
}

// dcost, 2pBVP.cu:109-115
__device__ __forceinline__ float dcost_eval(const PairCoef &c, const PairFF &f, float tau) {
  const float dtau = (float)0.000001;
  return (cost_fast(c, f, tau + dtau / 2) - cost_fast(c, f, tau - dtau / 2)) / dtau;
}

// toptBisection, 2pBVP.cu:71-95.  The reference's halving loop (:78-80) is
// unbounded; here it stops after 160 halvings (tl < 1e-50 has underflowed to
// zero long before), exactly as the oracle does.
__device__ float topt_bisection(const PairCoef &c, const PairFF &f, float tmax) {
  float tu = tmax;
  if (dcost_eval(c, f, tmax) < 0) return tmax;
  float tl = (float)0.01;
  int halvings = 0;
  while (dcost_eval(c, f, tl) > 0 && halvings < 160) {
    tl = tl / 2;
    ++halvings;
  }
  float topt = 0;
  float dcval = 1;
  int itr = 0;
  while (fabsf(dcval) > kDcvalTol && itr < 50) {
    ++itr;
    topt = (tu + tl) / 2;
    dcval = dcost_eval(c, f, topt);
    if (dcval > 0)
      tu = topt;
    else
      tl = topt;
  }
  return topt;
}

// --------------------------------------------------------------- kernels
// Persistent parity kernel.  The reference's bisection runs a different
// number of steps per pair (tmax test, halving loop, up to 50 bisection
// steps, then the final cost), so one thread per pair leaves most lanes of a
// warp idle while the slowest pair finishes.  Here every lane runs a small
// state machine over the same sequence of evaluations toptBisection performs
// for its pair, and each warp iteration evaluates exactly two costs in every
// lane (the two sides of dcost, or the final cost and a spare).  A lane whose
// pair is done stores it and takes the next pair of the warp's chunk of
// kParityChunk consecutive pairs (16 per lane on average, so lanes idle only
// while a chunk's last pairs finish).  Per pair, the evaluated expressions and
// their order are unchanged.
//
// A lane whose evaluation the float-float bound does not certify waits
// (keeping its state and the certified side of the pair) until
// kFallbackLanes lanes of its warp wait, or until no lane of the warp can
// go on: then the waiting lanes run the binary64 evaluation together.  The
// binary64 instructions cost a warp the same for one lane as for 32, so this
// spends them on several lanes at once.
// Launch bounds (128, 6): 80 registers, 6 blocks per SM (9.9 ms at N = 4000,
// 10.1 with 96 registers and 5 blocks).
constexpr int kParityChunk = 512;
constexpr int kFallbackLanes = 8;
constexpr int kRefillLanes = 8;

__global__ void __launch_bounds__(128, 6) bvp_pairs_parity_persistent(
    const float *__restrict__ samples, int N, float tmax, float *__restrict__ copts,
    float *__restrict__ topts) {
  const long long npairs = (long long)N * (N - 1);
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const float h = (float)0.000001 / 2;  // dtau / 2 of dcost
  const float dtau = (float)0.000001;
  const long long warp_id = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  long long chunk_next = warp_id * kParityChunk;
  const long long chunk_end = chunk_next + kParityChunk < npairs ? chunk_next + kParityChunk : npairs;
  // lane state
  long long idx = -1;
  int phase = 0, halvings = 0, itr = 0;
  float tu = 0, tl = 0, topt = 0, dcval = 0;
  float x0[kDim], x1[kDim];
  PairFF pf{};
  // the step's evaluation points and values; pending: a value waits for the
  // binary64 evaluation (ok_a / ok_b: that side is certified already)
  float ta = 0, tb = 0, ca = 0, cb = 0;
  bool pending = false, ok_a = true, ok_b = true;
  while (true) {
    // lanes without a pair take the next pairs of the warp's chunk, once
    // kRefillLanes of them wait (or no lane has a pair): the pair set-up
    // then runs for several lanes at once (N = 4000: 7.38 ms refilling each
    // lane at once, 6.40 ms with 4 lanes, 6.10 ms with 8, 6.59 ms with 16)
    const unsigned need = __ballot_sync(0xffffffffu, idx < 0);
    if (need && chunk_next < chunk_end && (__popc(need) >= kRefillLanes || need == 0xffffffffu)) {
      const int avail = (int)(chunk_end - chunk_next);
      const int rank = __popc(need & lt);
      const bool mine = (need >> lane) & 1u;
      if (mine && rank < avail) {
        idx = chunk_next + rank;
        const int i = (int)(idx / (N - 1));
        const int r = (int)(idx - (long long)i * (N - 1));
        const int j = r + (r >= i);
#pragma unroll
        for (int d = 0; d < kDim; ++d) {
          x0[d] = __ldg(&samples[i * kDim + d]);
          x1[d] = __ldg(&samples[j * kDim + d]);
        }
        pf = make_pair_ff(x0, x1);
        phase = 0;
        tu = tmax;
      }
      chunk_next += __popc(need) < avail ? __popc(need) : avail;
    }
    const unsigned active = __ballot_sync(0xffffffffu, idx >= 0);
    if (active == 0u) break;  // nothing left
    if (idx >= 0 && !pending) {
      // the two evaluation points of this step
      if (phase == 0) { ta = tmax + h; tb = tmax - h; }
      else if (phase == 1) { ta = tl + h; tb = tl - h; }
      else if (phase == 2) { ++itr; topt = (tu + tl) / 2; ta = topt + h; tb = topt - h; }
      else { ta = topt; tb = topt; }
      ca = cost_ff(pf, ta, &ok_a);
      cb = cost_ff(pf, tb, &ok_b);
      pending = !(ok_a && ok_b);
    }
    const unsigned waiting = __ballot_sync(0xffffffffu, pending);
    if (waiting && (__popc(waiting) >= kFallbackLanes || waiting == active)) {
      if (pending) {
        const PairCoef c = make_coef(x0, x1);
        if (!ok_a) ca = cost_eval(c, ta);
        if (!ok_b) cb = cost_eval(c, tb);
        pending = false;
      }
    }
    if (idx < 0 || pending) continue;
    const float d = (ca - cb) / dtau;
    if (phase == 0) {
      if (d < 0) { topt = tmax; phase = 3; }
      else { tl = (float)0.01; halvings = 0; phase = 1; }
    } else if (phase == 1) {
      if (d > 0 && halvings < 160) { tl = tl / 2; ++halvings; }
      else { topt = 0; dcval = 1; itr = 0; phase = 2; }
    } else if (phase == 2) {
      dcval = d;
      if (dcval > 0) tu = topt; else tl = topt;
      if (!(fabsf(dcval) > kDcvalTol && itr < 50)) phase = 3;
    } else {
      topts[idx] = topt;
      copts[idx] = ca;
      idx = -1;
    }
  }
}

__global__ void bvp_batch_kernel(const BvpJobs jb) {
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
  const PairCoef c = make_coef(x0, x1);
  const PairFF f = make_pair_ff(x0, x1);
  const float tp = topt_bisection(c, f, jb.tmax[j]);
  if (jb.topt[j]) jb.topt[j][k] = tp;
  if (jb.cost[j]) jb.cost[j][k] = cost_fast(c, f, tp);
}

// One thread per edge: findDiscretizedPath, 2pBVP.cu:53-69.  The edge's end
// states and time are loaded once for all of its W waypoints; a block's T
// edges (T x W x 6 floats, contiguous in disc) are assembled in shared
// memory and stored as whole lines, so the kernel's DRAM traffic is the
// waypoint records it writes.  The block size T (64, 128, 256) is picked by
// the autotuner.
template <int T>
size_t discretize_smem(int numDisc) {
  return sizeof(float) * (size_t)T * (numDisc + 1) * kDim;
}

template <int Mode, int T>
__global__ void __launch_bounds__(T) discretize_kernel(
    const float *__restrict__ samples, const int *__restrict__ src, const int *__restrict__ dst,
    const float *__restrict__ toptE, long long E, int numDisc, float *__restrict__ disc) {
  extern __shared__ float4 s_dyn4[];
  float *s_out = reinterpret_cast<float *>(s_dyn4);
  const int W = numDisc + 1;
  const long long e0 = blockIdx.x * (long long)T;
  const int nv = (int)(E - e0 < T ? E - e0 : T);
  if (threadIdx.x < nv) {
    const long long e = e0 + threadIdx.x;
    const int a = src[e], b = dst[e];
    const float topt = toptE[e];
    float x0[kDim], x1[kDim], x[kDim];
#pragma unroll
    for (int d = 0; d < kDim; ++d) {
      x0[d] = __ldg(&samples[a * kDim + d]);
      x1[d] = __ldg(&samples[b * kDim + d]);
    }
    float *o = s_out + threadIdx.x * W * kDim;
#pragma unroll
    for (int d = 0; d < kDim; ++d) {
      o[d] = x0[d];
      o[numDisc * kDim + d] = x1[d];
    }
    const float tau = topt;
    const float dt = tau / numDisc;
    if (Mode != PUMP_BVP_PRECISION) {
      // float-float waypoints; the uncertified ones (a few in a hundred) in
      // binary64 afterwards, each lane taking its next one per round, so a
      // warp runs the binary64 evaluation about once instead of once per
      // waypoint index where some lane needs it
      const PathFF pe = path_ff_edge(tau, x0, x1);
      unsigned int redo = 0u;  // waypoints i < 32 left for binary64
      for (int i = 1; i < numDisc; ++i) {
        if (!path_point_try(dt * i, tau, x0, x1, pe, x)) {
          if (i < 32) {
            redo |= 1u << i;
            continue;
          }
          path_point(dt * i, tau, x0, x1, x);
        }
#pragma unroll
        for (int d = 0; d < kDim; ++d) o[i * kDim + d] = x[d];
      }
      while (redo) {
        const int i = __ffs(redo) - 1;
        redo &= redo - 1u;
        path_point(dt * i, tau, x0, x1, x);
#pragma unroll
        for (int d = 0; d < kDim; ++d) o[i * kDim + d] = x[d];
      }
    } else {
      for (int i = 1; i < numDisc; ++i) {
        path_point_f32(dt * i, tau, x0, x1, x);
#pragma unroll
        for (int d = 0; d < kDim; ++d) o[i * kDim + d] = x[d];
      }
    }
  }
  __syncthreads();
  block_store(disc + e0 * W * kDim, s_out, nv * W * kDim);
}

// ---------------------------------------------- per-edge waypoint counts
// numDisc of an edge by its length (no counterpart in the reference, whose
// numDisc is one value per problem, mainPUMP.cu:57): ceil(L / disc_len)
// clamped to [min_disc, max_disc], L the binary32 distance between the end
// positions, sqrtf((dx*dx + dy*dy) + dz*dz), each operation rounded once;
// max_disc for every edge when disc_len <= 0.
__device__ __forceinline__ int disc_count(const float *x0, const float *x1, float disc_len,
                                          int min_disc, int max_disc) {
  if (!(disc_len > 0)) return max_disc;
  const float dx = x1[0] - x0[0], dy = x1[1] - x0[1], dz = x1[2] - x0[2];
  const float L = sqrtf(dx * dx + dy * dy + dz * dz);
  const float q = ceilf(L / disc_len);
  if (!(q >= (float)min_disc)) return min_disc;  // also NaN
  if (q > (float)max_disc) return max_disc;
  return (int)q;
}

__device__ __forceinline__ int edge_waypoints(const float *__restrict__ samples, int a, int b,
                                              float disc_len, int min_disc, int max_disc) {
  float x0[3], x1[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    x0[d] = __ldg(&samples[a * kDim + d]);
    x1[d] = __ldg(&samples[b * kDim + d]);
  }
  return disc_count(x0, x1, disc_len, min_disc, max_disc) + 1;
}

// The edges' first waypoints in the ragged layout (an exclusive scan of the
// per-edge waypoint counts), in three passes that never wait on each other:
// per-tile sums, one block scanning the tile sums, and per-tile scans.
constexpr int kOffThreads = 256;
constexpr int kOffPerThread = 16;
constexpr int kOffTile = kOffThreads * kOffPerThread;  // 4096 edges

__global__ void __launch_bounds__(kOffThreads) disc_tile_sums_kernel(
    const float *__restrict__ samples, const int *__restrict__ src, const int *__restrict__ dst,
    long long E, float disc_len, int min_disc, int max_disc, long long *__restrict__ tile_sum) {
  __shared__ long long s_part[kOffThreads / 32];
  const long long e0 = blockIdx.x * (long long)kOffTile;
  long long sum = 0;
  for (int k = 0; k < kOffPerThread; ++k) {
    const long long e = e0 + (long long)k * kOffThreads + threadIdx.x;
    if (e < E) sum += edge_waypoints(samples, src[e], dst[e], disc_len, min_disc, max_disc);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t = 0;
    for (int w = 0; w < kOffThreads / 32; ++w) t += s_part[w];
    tile_sum[blockIdx.x] = t;
  }
}

// One block of 1024 threads: tile_sum becomes its exclusive prefix in place,
// and off[E] the total.
__global__ void __launch_bounds__(1024) disc_tile_scan_kernel(long long *tile_sum, long long ntiles,
                                                              long long *off_end) {
  __shared__ long long s[1024];
  const int t = threadIdx.x;
  const long long per = (ntiles + 1023) / 1024;
  const long long b = t * per, e = b + per < ntiles ? b + per : ntiles;
  long long mine = 0;
  for (long long i = b; i < e; ++i) mine += tile_sum[i];
  s[t] = mine;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan
    const long long add = t >= o ? s[t - o] : 0;
    __syncthreads();
    s[t] += add;
    __syncthreads();
  }
  long long run = s[t] - mine;
  for (long long i = b; i < e; ++i) {
    const long long v = tile_sum[i];
    tile_sum[i] = run;
    run += v;
  }
  if (t == 1023) *off_end = s[1023];
}

// Per tile: each thread's kOffPerThread consecutive edges, scanned in order.
__global__ void __launch_bounds__(kOffThreads) disc_offsets_kernel(
    const float *__restrict__ samples, const int *__restrict__ src, const int *__restrict__ dst,
    long long E, float disc_len, int min_disc, int max_disc, const long long *__restrict__ tile_prefix,
    long long *__restrict__ off) {
  __shared__ long long s_part[kOffThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long e0 = blockIdx.x * (long long)kOffTile + (long long)threadIdx.x * kOffPerThread;
  int cnt[kOffPerThread];
  long long mine = 0;
#pragma unroll
  for (int k = 0; k < kOffPerThread; ++k) {
    const long long e = e0 + k;
    cnt[k] = e < E ? edge_waypoints(samples, src[e], dst[e], disc_len, min_disc, max_disc) : 0;
    mine += cnt[k];
  }
  // exclusive prefix of `mine` over the block, in thread order
  long long incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_part[warp] = incl;
  __syncthreads();
  long long before = 0;
  for (int w = 0; w < warp; ++w) before += s_part[w];
  long long run = tile_prefix[blockIdx.x] + before + incl - mine;
#pragma unroll
  for (int k = 0; k < kOffPerThread; ++k) {
    const long long e = e0 + k;
    if (e < E) off[e] = run;
    run += cnt[k];
  }
}

// findDiscretizedPath (2pBVP.cu:53-69) over the ragged layout: edge e's
// waypoints are records off[e] .. off[e+1]-1, numDisc_e = off[e+1]-off[e]-1.
// A block's T edges write one contiguous range, assembled in shared memory
// (T x max_w records) and stored as whole lines.
// An edge whose count is outside [2, max_disc + 1] makes its block write
// nothing and sets *error (when given) to PUMP_ERR_BAD_INPUT.
template <int Mode, int T>
__global__ void __launch_bounds__(T) discretize_off_kernel(
    const float *__restrict__ samples, const int *__restrict__ src, const int *__restrict__ dst,
    const float *__restrict__ toptE, long long E, const long long *__restrict__ off, int max_disc,
    float *__restrict__ disc, int *error) {
  extern __shared__ float4 s_dyn4[];
  float *s_out = reinterpret_cast<float *>(s_dyn4);
  const long long e0 = blockIdx.x * (long long)T;
  const int nv = (int)(E - e0 < T ? E - e0 : T);
  const long long base = off[e0];
  const long long cnt = threadIdx.x < nv ? off[e0 + threadIdx.x + 1] - off[e0 + threadIdx.x] : 2;
  if (__syncthreads_or(cnt < 2 || cnt > max_disc + 1)) {
    if (threadIdx.x == 0 && error) atomicExch(error, (int)PUMP_ERR_BAD_INPUT);
    return;
  }
  if (threadIdx.x < nv) {
    const long long e = e0 + threadIdx.x;
    const int a = src[e], b = dst[e];
    const int numDisc = (int)cnt - 1;
    float x0[kDim], x1[kDim], x[kDim];
#pragma unroll
    for (int d = 0; d < kDim; ++d) {
      x0[d] = __ldg(&samples[a * kDim + d]);
      x1[d] = __ldg(&samples[b * kDim + d]);
    }
    float *o = s_out + (off[e] - base) * kDim;
#pragma unroll
    for (int d = 0; d < kDim; ++d) {
      o[d] = x0[d];
      o[numDisc * kDim + d] = x1[d];
    }
    const float tau = toptE[e];
    const float dt = tau / numDisc;
    if (Mode != PUMP_BVP_PRECISION) {
      // float-float waypoints; the uncertified ones (a few in a hundred) in
      // binary64 afterwards, each lane taking its next one per round, so a
      // warp runs the binary64 evaluation about once instead of once per
      // waypoint index where some lane needs it
      const PathFF pe = path_ff_edge(tau, x0, x1);
      unsigned int redo = 0u;  // waypoints i < 32 left for binary64
      for (int i = 1; i < numDisc; ++i) {
        if (!path_point_try(dt * i, tau, x0, x1, pe, x)) {
          if (i < 32) {
            redo |= 1u << i;
            continue;
          }
          path_point(dt * i, tau, x0, x1, x);
        }
#pragma unroll
        for (int d = 0; d < kDim; ++d) o[i * kDim + d] = x[d];
      }
      while (redo) {
        const int i = __ffs(redo) - 1;
        redo &= redo - 1u;
        path_point(dt * i, tau, x0, x1, x);
#pragma unroll
        for (int d = 0; d < kDim; ++d) o[i * kDim + d] = x[d];
      }
    } else {
      for (int i = 1; i < numDisc; ++i) {
        path_point_f32(dt * i, tau, x0, x1, x);
#pragma unroll
        for (int d = 0; d < kDim; ++d) o[i * kDim + d] = x[d];
      }
    }
  }
  __syncthreads();
  block_store(disc + base * kDim, s_out, (int)(off[e0 + nv] - base) * kDim);
}

template <int Mode, int T>
pump_status_t discretize_launch(const float *d_samples, const int *d_src, const int *d_dst,
                                const float *d_topt, long long E, int numDisc, float *d_disc,
                                cudaStream_t s) {
  const size_t smem = discretize_smem<T>(numDisc);
  PUMP_TRY(smem_attr((const void *)discretize_kernel<Mode, T>, smem));
  discretize_kernel<Mode, T><<<grid_for(E, T), T, smem, s>>>(d_samples, d_src, d_dst, d_topt, E,
                                                             numDisc, d_disc);
  return launch_status("discretize_edges");
}

// Dense path of findOptimalPath (2pBVP.cu:5-36) for one segment: the host
// side computes the per-segment sample counts and time offsets (they are a
// short sequential recurrence); this kernel evaluates the states.
__global__ void path_states_kernel(const float *__restrict__ xs, const int *__restrict__ seg,
                                   const float *__restrict__ tsample, const float *__restrict__ tau,
                                   int total, float *__restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  const int s = seg[k];
  float x[kDim];
  path_point_fast(tsample[k], tau[s], &xs[s * kDim], &xs[(s + 1) * kDim], x);
#pragma unroll
  for (int d = 0; d < kDim; ++d) out[k * kDim + d] = x[d];
}

// ------------------------------------------------ candidate paths on device
// Per candidate path, from its segments' optimal times: the time recurrence
// of findOptimalPath (2pBVP.cu:15-32), samples per segment T = (int)((topt -
// toff) / dt + 1) at t = dt * k + toff, the carry toff = (t - topt) + dt (t
// is the last sample written, from an earlier segment when T <= 0), and the
// smoothing's cost sum over the segments (PUMP.cu:499-502) in segment order;
// then the state of every sample.  Blocks (path, y): every block runs the
// path's recurrence into shared memory (a few dozen segments, one thread),
// block y = 0 writes the path's length and cost (and zeroes its MC hit
// counter), and the blocks share the path's rows.  Rows of path p start at
// p * rows_cap (rows at or past rows_cap are not written); a row's segment
// is the last one of the path whose first row is at or before it (segments
// with no samples share their first row with the next).  The precision mode
// evaluates the cubic in binary32, as its edge waypoints do.
constexpr int kRowThreads = 128;

template <int Mode>
__global__ void __launch_bounds__(kRowThreads) candidate_rows_kernel(
    const float *__restrict__ x0, const float *__restrict__ x1, const float *__restrict__ topt,
    const float *__restrict__ seg_cost, const int *__restrict__ node_cnt,
    const int *__restrict__ seg_base, float dt, int rows_cap, int *__restrict__ len,
    float *__restrict__ cost, int *__restrict__ hits, float *__restrict__ states,
    unsigned int *done) {
  extern __shared__ int s_seg[];  // per segment: first row, then toff
  __shared__ int s_len;
  const int p = blockIdx.x;
  const int n = node_cnt[p], b = seg_base[p], ns = n > 1 ? n - 1 : 0;
  int *srow = s_seg;
  float *stoff = reinterpret_cast<float *>(s_seg + ns);
  if (threadIdx.x == 0) {
    float toff = 0, t = 0, c = 0;
    int rows = 0;
    for (int i = 0; i + 1 < n; ++i) {
      const float tp = topt[b + i];
      const int T = (int)((tp - toff) / dt + 1);
      stoff[i] = toff;
      srow[i] = rows;
      if (T > 0) t = dt * (T - 1) + toff;  // the last sample's time
      rows += T;
      toff = (t - tp) + dt;
      if (seg_cost) c += seg_cost[b + i];
    }
    s_len = rows;
    if (blockIdx.y == 0) {
      len[p] = rows;
      if (cost) cost[p] = c;
      if (hits) hits[p] = 0;
      if (done && p == 0) *done = 0u;
    }
  }
  __syncthreads();
  if (ns == 0) return;
  const int L = s_len < rows_cap ? s_len : rows_cap;
  for (int r = blockIdx.y * kRowThreads + threadIdx.x; r < L; r += gridDim.y * kRowThreads) {
    int lo = 0, hi = ns - 1;  // segments b + lo .. b + hi
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (srow[mid] <= r) lo = mid; else hi = mid - 1;
    }
    const int s = b + lo, k = r - srow[lo];
    float a[kDim], c[kDim], x[kDim];
#pragma unroll
    for (int d = 0; d < kDim; ++d) {
      a[d] = x0[s * kDim + d];
      c[d] = x1[s * kDim + d];
    }
    if (Mode == PUMP_BVP_PARITY) path_point_fast(dt * k + stoff[lo], topt[s], a, c, x);
    else path_point_f32(dt * k + stoff[lo], topt[s], a, c, x);
    const long long t = (long long)p * rows_cap + r;
#pragma unroll
    for (int d = 0; d < kDim; ++d) states[t * kDim + d] = x[d];
  }
}

}  // namespace

// ------------------------------------------------------------------ host
pump_status_t candidate_paths_async(const CandidateBufs &cb, int n_paths, int n_seg, int max_segs,
                                    int mode, float dt, bool with_cost, int rows_cap,
                                    cudaStream_t s) {
  if (n_paths <= 0) return PUMP_OK;
  mode = host_bvp_mode(mode);  // findOptimalPath and the smoothing run on the reference's host
  if (n_seg > 0) {
    // optimal times (tmax 5) and smoothing costs and times (tmax 2) in one
    // launch
    BvpJobs jb{};
    jb.x0 = cb.x0;
    jb.x1 = cb.x1;
    jb.n = n_seg;
    jb.jobs = (with_cost || cb.topt2) ? 2 : 1;
    jb.tmax[0] = 5.0f;
    jb.topt[0] = cb.topt;
    jb.tmax[1] = 2.0f;
    jb.cost[1] = with_cost ? cb.seg_cost : nullptr;
    jb.topt[1] = cb.topt2;
    PUMP_TRY(bvp_jobs_launch(jb, mode, s));
  }
  const size_t smem = sizeof(int) * 2 * (size_t)(max_segs > 0 ? max_segs : 1);
  if (smem > 200 * 1024)
    return set_error(PUMP_ERR_CAPACITY, "candidate path of %d segments exceeds the row stage", max_segs);
  int ny = (rows_cap + kRowThreads - 1) / kRowThreads;
  if (ny > 64) ny = 64;
  if (ny < 1) ny = 1;
  const dim3 grid((unsigned)n_paths, (unsigned)ny);
  PUMP_TRY(smem_attr(mode == PUMP_BVP_PARITY ? (const void *)candidate_rows_kernel<PUMP_BVP_PARITY>
                                             : (const void *)candidate_rows_kernel<PUMP_BVP_PRECISION>,
                     smem));
  if (mode == PUMP_BVP_PARITY)
    candidate_rows_kernel<PUMP_BVP_PARITY><<<grid, kRowThreads, smem, s>>>(
        cb.x0, cb.x1, cb.topt, with_cost ? cb.seg_cost : nullptr, cb.node_cnt, cb.seg_base, dt,
        rows_cap, cb.len, with_cost ? cb.cost : nullptr, cb.hits, cb.states, cb.done);
  else
    candidate_rows_kernel<PUMP_BVP_PRECISION><<<grid, kRowThreads, smem, s>>>(
        cb.x0, cb.x1, cb.topt, with_cost ? cb.seg_cost : nullptr, cb.node_cnt, cb.seg_base, dt,
        rows_cap, cb.len, with_cost ? cb.cost : nullptr, cb.hits, cb.states, cb.done);
  return launch_status("candidate_rows");
}

namespace {
__global__ void own_pairs_kernel(const float *__restrict__ samples, int N, float *__restrict__ x0,
                                 float *__restrict__ x1) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int n1 = N - 1, n2 = N - 2;
  if (k >= 2 * n1 + 2 * n2) return;
  int a, b;
  if (k < n1) { a = 0; b = k + 1; }                           // init row
  else if (k < 2 * n1) { a = k - n1 + 1; b = 0; }             // init column
  else if (k < 2 * n1 + n2) { a = N - 1; b = k - 2 * n1 + 1; }  // goal row
  else { a = k - 2 * n1 - n2 + 1; b = N - 1; }                // goal column
#pragma unroll
  for (int d = 0; d < kDim; ++d) {
    x0[k * kDim + d] = samples[a * kDim + d];
    x1[k * kDim + d] = samples[b * kDim + d];
  }
}
}  // namespace

pump_status_t own_pairs_async(const float *d_samples, int N, float *d_x0, float *d_x1,
                              cudaStream_t stream) {
  const int n = 4 * N - 6;
  if (n <= 0) return PUMP_OK;
  own_pairs_kernel<<<grid_for(n, 256), 256, 0, stream>>>(d_samples, N, d_x0, d_x1);
  return launch_status("own_pairs_kernel");
}

pump_status_t bvp_jobs_launch(const BvpJobs &jb, int mode, cudaStream_t stream) {
  if (jb.n <= 0) return PUMP_OK;
  if (mode == PUMP_BVP_PRECISION) return bvp_jobs_precision_launch(jb, stream);
  if (mode == PUMP_BVP_PARITY_GPU) return bvp_jobs_refgpu_launch(jb, stream);
  const long long total = (long long)jb.n * jb.jobs;
  const int threads = total < 152LL * 128 ? 32 : 128;
  bvp_batch_kernel<<<grid_for(total, threads), threads, 0, stream>>>(jb);
  return launch_status("bvp_batch");
}

namespace {
// Each edge's optimal time in the host arithmetic (tmax 5), one thread per
// edge (the lane-refill kernel of all pairs took 1.15 ms on the N = 4000
// query's 799,800 edges, this one about 0.9 ms).
__global__ void edge_topts_parity_kernel(const float *__restrict__ samples, const int *__restrict__ src,
                                         const int *__restrict__ dst, long long E,
                                         float *__restrict__ topt) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= E) return;
  float x0[kDim], x1[kDim];
  const int a = src[e], b = dst[e];
#pragma unroll
  for (int d = 0; d < kDim; ++d) {
    x0[d] = __ldg(&samples[a * kDim + d]);
    x1[d] = __ldg(&samples[b * kDim + d]);
  }
  topt[e] = topt_bisection(make_coef(x0, x1), make_pair_ff(x0, x1), 5.0f);
}
}  // namespace

pump_status_t edge_topts_parity_async(const float *d_samples, const int *d_src, const int *d_dst,
                                      long long E, float *d_topt, cudaStream_t stream) {
  if (E <= 0) return PUMP_OK;
  edge_topts_parity_kernel<<<grid_for(E, 128), 128, 0, stream>>>(d_samples, d_src, d_dst, E, d_topt);
  return launch_status("edge_topts_parity");
}

namespace {
// The times the waypoint entry points evaluate at: d_topt itself, or, in the
// GPU-arithmetic mode (whose d_topt holds the reference GPU kernel's times),
// each edge's time in the host arithmetic, as the reference's
// findDiscretizedPath (host code) recomputes it, in a stream-ordered buffer
// freed with the object.
struct HostTopts {
  const float *topt = nullptr;
  float *own = nullptr;
  cudaStream_t s = nullptr;
  pump_status_t make(const float *d_samples, const int *d_src, const int *d_dst,
                     const float *d_topt, long long E, int mode, cudaStream_t stream) {
    topt = d_topt;
    if (mode != PUMP_BVP_PARITY_GPU) return PUMP_OK;
    s = stream;
    PUMP_CUDA_TRY(pool_malloc_async((void **)&own, sizeof(float) * (size_t)E, stream));
    topt = own;
    return edge_topts_parity_async(d_samples, d_src, d_dst, E, own, stream);
  }
  ~HostTopts() {
    if (own) cudaFreeAsync(own, s);
  }
};
}  // namespace

pump_status_t bvp_path_states(const float *d_xs, const int *d_seg, const float *d_tsample,
                              const float *d_tau, int total, float *d_out, cudaStream_t stream) {
  if (total <= 0) return PUMP_OK;
  path_states_kernel<<<grid_for(total, 128), 128, 0, stream>>>(d_xs, d_seg, d_tsample, d_tau,
                                                              total, d_out);
  return launch_status("path_states_kernel");
}

}  // namespace pump

using namespace pump;

extern "C" pump_status_t pump_bvp_pairs(const float *d_samples, int N, float tmax, int mode,
                                        float *d_copts, float *d_topts, pump_stream_t stream) {
  if (N < 2 || !d_samples || !d_copts || !d_topts || !(tmax > 0))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_bvp_pairs: bad arguments (N=%d)", N);
  const long long npairs = (long long)N * (N - 1);
  const int threads = 128;
  long long blocks = (npairs + threads - 1) / threads;
  if (blocks > 2147483647LL) blocks = 2147483647LL;
  if (mode == PUMP_BVP_PARITY) {
    const long long nblk = (npairs + 4LL * kParityChunk - 1) / (4LL * kParityChunk);  // 4 warps
    if (nblk > 2147483647LL) return set_error(PUMP_ERR_CAPACITY, "pump_bvp_pairs: N=%d", N);
    bvp_pairs_parity_persistent<<<(unsigned)nblk, 128, 0, (cudaStream_t)stream>>>(
        d_samples, N, tmax, d_copts, d_topts);
  } else if (mode == PUMP_BVP_PRECISION) {
    PUMP_TRY(bvp_pairs_precision_launch(d_samples, N, tmax, d_copts, d_topts, (cudaStream_t)stream));
  } else if (mode == PUMP_BVP_PARITY_GPU) {
    PUMP_TRY(bvp_pairs_refgpu_launch(d_samples, N, tmax, d_copts, d_topts, (cudaStream_t)stream));
  } else
    return set_error(PUMP_ERR_BAD_INPUT, "pump_bvp_pairs: unknown mode %d", mode);
  return launch_status("bvp_pairs");
}

extern "C" pump_status_t pump_bvp_batch(const float *d_x0, const float *d_x1, int n, float tmax,
                                        int mode, float *d_topt, float *d_cost,
                                        pump_stream_t stream) {
  if (n < 0 || (n > 0 && (!d_x0 || !d_x1)) || !(tmax > 0) ||
      (mode != PUMP_BVP_PARITY && mode != PUMP_BVP_PRECISION && mode != PUMP_BVP_PARITY_GPU))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_bvp_batch: bad arguments");
  if (n == 0) return PUMP_OK;
  BvpJobs jb{};
  jb.x0 = d_x0;
  jb.x1 = d_x1;
  jb.n = n;
  jb.jobs = 1;
  jb.tmax[0] = tmax;
  jb.topt[0] = d_topt;
  jb.cost[0] = d_cost;
  return bvp_jobs_launch(jb, mode, (cudaStream_t)stream);
}

namespace pump {
size_t disc_offsets_scratch(long long E) {
  return sizeof(long long) * (size_t)((E + kOffTile - 1) / kOffTile + 1);
}

pump_status_t disc_offsets_async(const float *d_samples, const int *d_src, const int *d_dst,
                                 long long E, float disc_len, int min_disc, int max_disc,
                                 long long *d_off, long long *d_scratch, cudaStream_t s) {
  if (E <= 0) return cuda_status(cudaMemsetAsync(d_off, 0, sizeof(long long), s), "cudaMemsetAsync");
  const long long ntiles = (E + kOffTile - 1) / kOffTile;
  if (ntiles > 2147483647LL) return set_error(PUMP_ERR_CAPACITY, "disc offsets: %lld edges", E);
  disc_tile_sums_kernel<<<(unsigned)ntiles, kOffThreads, 0, s>>>(d_samples, d_src, d_dst, E, disc_len,
                                                                  min_disc, max_disc, d_scratch);
  PUMP_TRY(launch_status("disc_tile_sums_kernel"));
  disc_tile_scan_kernel<<<1, 1024, 0, s>>>(d_scratch, ntiles, d_off + E);
  PUMP_TRY(launch_status("disc_tile_scan_kernel"));
  disc_offsets_kernel<<<(unsigned)ntiles, kOffThreads, 0, s>>>(d_samples, d_src, d_dst, E, disc_len,
                                                                min_disc, max_disc, d_scratch, d_off);
  return launch_status("disc_offsets_kernel");
}

pump_status_t discretize_off_async(const float *d_samples, const int *d_src, const int *d_dst,
                                   const float *d_topt, long long E, const long long *d_off,
                                   int max_disc, int mode, float *d_disc, cudaStream_t s,
                                   int *error) {
  if (E <= 0) return PUMP_OK;
  constexpr int T = 64;
  const size_t smem = sizeof(float) * (size_t)T * (max_disc + 1) * kDim;
  if (smem > 220 * 1024)
    return set_error(PUMP_ERR_CAPACITY, "%d waypoints per edge exceed the stage", max_disc + 1);
  auto go = [&](auto m) -> pump_status_t {
    constexpr int M = decltype(m)::value;
    PUMP_TRY(smem_attr((const void *)discretize_off_kernel<M, T>, smem));
    discretize_off_kernel<M, T><<<grid_for(E, T), T, smem, s>>>(d_samples, d_src, d_dst, d_topt, E,
                                                               d_off, max_disc, d_disc, error);
    return launch_status("discretize_off_kernel");
  };
  // the GPU-arithmetic mode's waypoints are the parity mode's (host code),
  // at times in the host arithmetic (HostTopts)
  if (mode != PUMP_BVP_PRECISION) return go(std::integral_constant<int, PUMP_BVP_PARITY>{});
  return go(std::integral_constant<int, PUMP_BVP_PRECISION>{});
}
}  // namespace pump

extern "C" pump_status_t pump_disc_offsets(const float *d_samples, const int *d_src, const int *d_dst,
                                           long long E, float disc_len, int min_disc, int max_disc,
                                           long long *d_off, long long *h_total,
                                           pump_stream_t stream) {
  if (E < 0 || min_disc < 1 || max_disc < min_disc || !d_off || !h_total ||
      (E > 0 && (!d_samples || !d_src || !d_dst)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_disc_offsets: bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  long long *scratch = nullptr;
  PUMP_CUDA_TRY(pool_malloc_async((void **)&scratch, disc_offsets_scratch(E), s));
  const pump_status_t st = disc_offsets_async(d_samples, d_src, d_dst, E, disc_len, min_disc,
                                              max_disc, d_off, scratch, s);
  cudaFreeAsync(scratch, s);
  PUMP_TRY(st);
  PUMP_CUDA_TRY(cudaMemcpyAsync(h_total, d_off + E, sizeof(long long), cudaMemcpyDeviceToHost, s));
  PUMP_CUDA_TRY(cudaStreamSynchronize(s));
  return PUMP_OK;
}

extern "C" pump_status_t pump_discretize_edges_off(const float *d_samples, const int *d_src,
                                                   const int *d_dst, const float *d_topt, long long E,
                                                   const long long *d_off, int max_disc, int mode,
                                                   float *d_disc, pump_stream_t stream) {
  if (E < 0 || max_disc < 1 ||
      (mode != PUMP_BVP_PARITY && mode != PUMP_BVP_PRECISION && mode != PUMP_BVP_PARITY_GPU) ||
      (E > 0 && (!d_samples || !d_src || !d_dst || !d_topt || !d_off || !d_disc)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_discretize_edges_off: bad arguments");
  if (E == 0) return PUMP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  HostTopts ht;
  PUMP_TRY(ht.make(d_samples, d_src, d_dst, d_topt, E, mode, s));
  int *d_err = nullptr;
  PUMP_CUDA_TRY(pool_malloc_async((void **)&d_err, sizeof(int), s));
  pump_status_t st = cuda_status(cudaMemsetAsync(d_err, 0, sizeof(int), s), "cudaMemsetAsync");
  if (st == PUMP_OK)
    st = discretize_off_async(d_samples, d_src, d_dst, ht.topt, E, d_off, max_disc, mode, d_disc, s, d_err);
  int err = 0;
  if (st == PUMP_OK)
    st = cuda_status(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
  cudaFreeAsync(d_err, s);
  if (st == PUMP_OK) st = cuda_status(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  PUMP_TRY(st);
  if (err)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_discretize_edges_off: an edge's waypoint count is "
                                         "outside [2, max_disc + 1]");
  return PUMP_OK;
}

extern "C" pump_status_t pump_discretize_edges(const float *d_samples, const int *d_src,
                                               const int *d_dst, const float *d_topt, long long E,
                                               int numDisc, int mode, float *d_disc,
                                               pump_stream_t stream) {
  if (E < 0 || numDisc < 1 ||
      (mode != PUMP_BVP_PARITY && mode != PUMP_BVP_PRECISION && mode != PUMP_BVP_PARITY_GPU) ||
      (E > 0 && (!d_samples || !d_src || !d_dst || !d_topt || !d_disc)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_discretize_edges: bad arguments");
  if (E == 0) return PUMP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (discretize_smem<256>(numDisc) > 220 * 1024)
    return set_error(PUMP_ERR_CAPACITY, "pump_discretize_edges: %d waypoints per edge exceed the stage",
                     numDisc + 1);
  HostTopts ht;
  PUMP_TRY(ht.make(d_samples, d_src, d_dst, d_topt, E, mode, s));
  const float *topt = ht.topt;
  // block sizes 64, 128 (default), 256; the GPU-arithmetic mode's waypoints
  // are the parity mode's at the host arithmetic's times
  auto go = [&](auto block) -> pump_status_t {
    constexpr int T = decltype(block)::value;
    if (mode != PUMP_BVP_PRECISION)
      return discretize_launch<PUMP_BVP_PARITY, T>(d_samples, d_src, d_dst, topt, E, numDisc,
                                                   d_disc, s);
    return discretize_launch<PUMP_BVP_PRECISION, T>(d_samples, d_src, d_dst, topt, E, numDisc,
                                                    d_disc, s);
  };
  auto run = [&](int c) -> pump_status_t {
    if (c == 0) return go(std::integral_constant<int, 64>{});
    if (c == 1) return go(std::integral_constant<int, 128>{});
    return go(std::integral_constant<int, 256>{});
  };
  int choice = 1;
  bool ran = false;
  const uint64_t key = ((uint64_t)mode << 40) | ((uint64_t)numDisc << 32) | tune_bucket(E);
  PUMP_TRY(tune_choice(kTuneDiscretize, key, 3, 1, s, run, &choice, &ran));
  return ran ? PUMP_OK : run(choice);
}
