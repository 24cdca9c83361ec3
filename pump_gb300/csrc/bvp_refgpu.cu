// Pair BVPs in the arithmetic of the reference's own GPU kernel
// (fillCoptsTopts, 2pBVP.cu:133-150, with toptBisection :71-95, dcost
// :109-115 and cost :97-107, compiled by nvcc as the reference's Makefile
// compiles it).
//
// Two things make that arithmetic differ from the rounded-once parity
// arithmetic of bvp.cu: nvcc contracts multiply-adds by default, at sites of
// its own choosing, and in device code pow(float, int) promotes to CUDA's
// binary64 pow(double, double), which is not correctly rounded (on the
// GB300 pow(double(x), 2) differs from the exact square for about 6 % of
// binary32 x, pow(x, 3) and pow(x, 4) from the correctly rounded power for
// about 25 %).  Neither can be restated operation by operation, so this
// translation unit is compiled with contraction on, as the reference is,
// calls pow where the reference calls it, and writes the cost as the
// reference's expression with the same operands, types and order, so that
// the compiler sees the same expression tree.  The twelve pow(coordinate, 2)
// terms do not depend on tau and are evaluated once per pair; the tree the
// compiler contracts is unchanged (those leaves are pow results either way).
// A GPU test compares all N(N-1) pairs at N = 1000 and 4000 with the
// reference's fillCoptsTopts run on the GB300 (SHA-256 of both arrays).
//
// The kernel walks the pairs as bvp.cu's parity kernel does (a per-lane
// state machine over the bisection's evaluations, lanes refilled from the
// warp's chunk of pairs), which changes the order of work, not any pair's
// arithmetic.  Cost: 0.59 s for the 16 M pairs of N = 4000 (the reference's
// kernel 0.62 s); CUDA's pow for tau (three calls per evaluation) dominates.
#include <math.h>

#include "common.cuh"
#include "ctx.h"
#include "ffcost.cuh"

namespace pump {
namespace {

// the reference's `const float g = -9.81;` (2pBVP.cu:3)
const float kGRef = -9.81;

// pow(coordinate, 2) of both states: the tau-independent pow calls of cost
struct CoordPow {
  double a0, a1, a2, a3, a4, a5, b0, b1, b2, b3, b4, b5;
};
__device__ __forceinline__ CoordPow coord_pow(const float *a, const float *b) {
  CoordPow p;
  p.a0 = pow(a[0], 2); p.a1 = pow(a[1], 2); p.a2 = pow(a[2], 2);
  p.a3 = pow(a[3], 2); p.a4 = pow(a[4], 2); p.a5 = pow(a[5], 2);
  p.b0 = pow(b[0], 2); p.b1 = pow(b[1], 2); p.b2 = pow(b[2], 2);
  p.b3 = pow(b[3], 2); p.b4 = pow(b[4], 2); p.b5 = pow(b[5], 2);
  return p;
}

// cost, 2pBVP.cu:97-107: the same expression (a = x0, b = x1, p.aK and p.bK
// for pow(x0[K], 2) and pow(x1[K], 2))
__device__ __forceinline__ float cost_dev(float tau, const float *a, const float *b, const CoordPow &p) {
  const float g = kGRef;
  float c = (1/pow(tau,3))*(12*p.a0 + 12*p.a2 + 12*p.a1 + 12*p.b0 + 12*p.b2 - 24*a[1]*b[1] +
      12*p.b1 + 12*a[4]*a[1]*tau + 12*a[1]*b[4]*tau - 12*a[3]*b[0]*tau - 12*b[3]*b[0]*tau -
      12*a[5]*b[2]*tau - 12*b[5]*b[2]*tau - 12*a[4]*b[1]*tau - 12*b[4]*b[1]*tau + 4*p.a4*pow(tau,2) +
      4*p.a3*pow(tau,2) + 4*p.a5*pow(tau,2) + 4*a[4]*b[4]*pow(tau,2) + 4*p.b4*pow(tau,2) + 4*a[3]*b[3]*pow(tau,2) +
      4*p.b3*pow(tau,2) + 4*a[5]*b[5]*pow(tau,2) + 4*p.b5*pow(tau,2) + 2*g*a[5]*pow(tau,3) - 2*g*b[5]*pow(tau,3) + pow(tau,4) +
      pow(g,2)*pow(tau,4) + 12*a[0]*(-2*b[0] + (a[3] + b[3])*tau) + 12*a[2]*(-2*b[2] + (a[5] + b[5])*tau));
  return c;
}

// dcost, 2pBVP.cu:109-115
__device__ __forceinline__ float dcost_dev(float tau, const float *a, const float *b, const CoordPow &p) {
  float dtau = 0.000001;
  float d = (cost_dev(tau + dtau / 2, a, b, p) - cost_dev(tau - dtau / 2, a, b, p)) / dtau;
  return d;
}

// toptBisection, 2pBVP.cu:71-95; the halving loop, unbounded in the
// reference, stops after 160 halvings (as in bvp.cu and the oracle)
__device__ float topt_dev(const float *a, const float *b, const CoordPow &p, float tmax) {
  float tu = tmax;
  if (dcost_dev(tmax, a, b, p) < 0) return tmax;
  float tl = 0.01;
  int halvings = 0;
  while (dcost_dev(tl, a, b, p) > 0 && halvings < 160) {
    tl = tl / 2;
    ++halvings;
  }
  float topt = 0;
  float dcval = 1;
  int maxItrs = 50;
  int itr = 0;
  while (fabsf(dcval) > 0.0001 && itr < maxItrs && ++itr) {
    topt = (tu + tl) / 2;
    dcval = dcost_dev(topt, a, b, p);
    if (dcval > 0)
      tu = topt;
    else
      tl = topt;
  }
  return topt;
}

// The reference expression's costs at ta and tb (each when wanted); out of
// line, so that the registers of the binary64 powers do not count against
// the pair kernel's occupancy (80-96 registers instead of 106: 10.57 ms ->
// 10.04 ms at N = 4000 with 5 blocks of 128 per SM, 10.27 ms with 6).
struct PairStates {
  float a[kDim], b[kDim];
};
struct CostPair {
  float ca, cb;
};
__device__ __noinline__ CostPair refgpu_costs(const PairStates st, float ta, float tb, bool want_a,
                                              bool want_b) {
  const CoordPow p = coord_pow(st.a, st.b);
  CostPair r{0.0f, 0.0f};
  if (want_a) r.ca = cost_dev(ta, st.a, st.b, p);
  if (want_b) r.cb = cost_dev(tb, st.a, st.b, p);
  return r;
}

// All ordered pairs: per lane, the evaluations of toptBisection as a state
// machine (phase 0: the tmax test, 1: halving, 2: bisection, 3: the final
// cost), two cost evaluations per step; a lane whose pair is done takes the
// next pair of its warp's chunk of kChunk pairs.  Each evaluation is first
// certified in float-float (cost_ff, ffcost.cuh); a lane whose value is not
// certified waits until kFallback lanes of its warp wait (or no lane can go
// on), and they evaluate the reference's expression (CUDA's pow included)
// together.
constexpr int kChunk = 512;
constexpr int kFallback = 8;
constexpr int kRefill = 8;

__global__ void __launch_bounds__(128, 5) bvp_pairs_refgpu_kernel(const float *__restrict__ samples,
                                                               int N, float tmax,
                                                               float *__restrict__ copts,
                                                               float *__restrict__ topts) {
  const long long npairs = (long long)N * (N - 1);
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  float dtau = 0.000001;
  const float h = dtau / 2;
  const long long warp_id = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  long long chunk_next = warp_id * kChunk;
  const long long chunk_end = chunk_next + kChunk < npairs ? chunk_next + kChunk : npairs;
  long long idx = -1;
  int phase = 0, halvings = 0, itr = 0;
  float tu = 0, tl = 0, topt = 0, dcval = 0;
  float a[kDim], b[kDim];
  PairFF pf{};
  float ta = 0, tb = 0, ca = 0, cb = 0;
  bool pending = false, ok_a = true, ok_b = true;
  while (true) {
    // (refilled once kRefill lanes wait, or none has a pair, as in the parity
    // kernel)
    const unsigned need = __ballot_sync(0xffffffffu, idx < 0);
    if (need && chunk_next < chunk_end && (__popc(need) >= kRefill || need == 0xffffffffu)) {
      const int avail = (int)(chunk_end - chunk_next);
      const int rank = __popc(need & lt);
      if (((need >> lane) & 1u) && rank < avail) {
        idx = chunk_next + rank;
        const int i = (int)(idx / (N - 1));
        const int r = (int)(idx - (long long)i * (N - 1));
        const int j = r + (r >= i);
#pragma unroll
        for (int d = 0; d < kDim; ++d) {
          a[d] = __ldg(&samples[i * kDim + d]);
          b[d] = __ldg(&samples[j * kDim + d]);
        }
        pf = make_pair_ff(a, b);
        phase = 0;
        tu = tmax;
      }
      chunk_next += __popc(need) < avail ? __popc(need) : avail;
    }
    const unsigned active = __ballot_sync(0xffffffffu, idx >= 0);
    if (active == 0u) break;
    if (idx >= 0 && !pending) {
      if (phase == 0) { ta = tmax + h; tb = tmax - h; }
      else if (phase == 1) { ta = tl + h; tb = tl - h; }
      else if (phase == 2) { ++itr; topt = (tu + tl) / 2; ta = topt + h; tb = topt - h; }
      else { ta = topt; tb = topt; }
      ca = cost_ff(pf, ta, &ok_a);
      cb = cost_ff(pf, tb, &ok_b);
      pending = !(ok_a && ok_b);
    }
    const unsigned waiting = __ballot_sync(0xffffffffu, pending);
    if (waiting && (__popc(waiting) >= kFallback || waiting == active)) {
      if (pending) {
        PairStates st;
#pragma unroll
        for (int d = 0; d < kDim; ++d) {
          st.a[d] = a[d];
          st.b[d] = b[d];
        }
        const CostPair r = refgpu_costs(st, ta, tb, !ok_a, !ok_b);
        if (!ok_a) ca = r.ca;
        if (!ok_b) cb = r.cb;
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
      // (double)|dcval| > 0.0001 exactly when |dcval| > 0.0001f: binary32
      // 0.0001f is below 0.0001 and the next binary32 above it
      if (!(fabsf(dcval) > 0.0001f && itr < 50)) phase = 3;
    } else {
      topts[idx] = topt;
      copts[idx] = ca;
      idx = -1;
    }
  }
}

// Explicit pairs (the BvpJobs layout of ctx.h), one thread per (job, pair).
__global__ void bvp_batch_refgpu_kernel(const BvpJobs jb) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= jb.n * jb.jobs) return;
  const int j = k >= jb.n ? 1 : 0;
  k -= j * jb.n;
  float a[kDim], b[kDim];
#pragma unroll
  for (int d = 0; d < kDim; ++d) {
    a[d] = jb.x0[k * kDim + d];
    b[d] = jb.x1[(jb.x1_same ? 0 : k) * kDim + d];
  }
  const CoordPow p = coord_pow(a, b);
  const float tp = topt_dev(a, b, p, jb.tmax[j]);
  if (jb.topt[j]) jb.topt[j][k] = tp;
  if (jb.cost[j]) jb.cost[j][k] = cost_dev(tp, a, b, p);
}

}  // namespace

pump_status_t bvp_pairs_refgpu_launch(const float *d_samples, int N, float tmax, float *d_copts,
                                      float *d_topts, cudaStream_t stream) {
  const long long npairs = (long long)N * (N - 1);
  const long long nblk = (npairs + 4LL * kChunk - 1) / (4LL * kChunk);  // 4 warps per block
  if (nblk > 2147483647LL) return set_error(PUMP_ERR_CAPACITY, "pump_bvp_pairs: N=%d", N);
  bvp_pairs_refgpu_kernel<<<(unsigned)nblk, 128, 0, stream>>>(d_samples, N, tmax, d_copts, d_topts);
  return launch_status("bvp_pairs_refgpu");
}

pump_status_t bvp_jobs_refgpu_launch(const BvpJobs &jb, cudaStream_t stream) {
  if (jb.n <= 0) return PUMP_OK;
  const long long total = (long long)jb.n * jb.jobs;
  const int threads = total < 152LL * 128 ? 32 : 128;
  bvp_batch_refgpu_kernel<<<grid_for(total, threads), threads, 0, stream>>>(jb);
  return launch_status("bvp_batch_refgpu");
}

}  // namespace pump
