// Particle stream, half-space Monte Carlo (HSMC) propagation and full Monte
// Carlo collision probability (reference: PUMP.cu:613-758,
// collisionProbability.cu:4-92, hardCoded.cuh:12-19).
//
// Particle stream.  The reference reads precomputed closed-loop tracking
// errors (xcomb / xcombTime) from a data file that is not part of its source
// tree.  They are regenerated here from a documented model: per axis a
// double integrator at dt = 0.05 s under the PD tracking law a = w - (16 p +
// 5.6 v), w ~ N(0, 4^2), starting from zero error, simulated in binary64.
// Noise comes from Philox4x32-10 (Salmon et al., SC'11) at counter
// (particle, step, 0, 0), turned into Gaussians by Box-Muller whose log and
// sine/cosine are evaluated by fixed series with +,-,*,/ and sqrt only
// (atanh series for log, Taylor series on a quarter period for sin/cos), so
// the table is bit-identical on any IEEE machine that does not contract
// multiply-adds.
//
// HSMC.  One block per new path, threads over particles.  The half-spaces of
// a waypoint are the same for every particle of the path, so each test is a
// block-uniform branch on b >= 1000 followed by a 3-term dot product against
// the particle's offset row; offsets are read time-major so a warp reads 32
// consecutive particles (384 contiguous bytes).  Validity is kept as a bit
// per particle (__ballot_sync), and the hit count of calculateCP_HSMC is the
// block's popcount sum, so the CP needs no second pass over a byte array.
//
// Monte Carlo CP.  Thread per (particle, path) over many paths per launch;
// obstacles staged in shared memory; the same segment test as freeEdges.
#include "collide.cuh"
#include "search.h"

namespace pump {
namespace {

// ------------------------------------------------------- particle stream
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

__device__ double det_log(double x) {
  int e;
  double m = frexp(x, &e);
  if (m < 0.70710678118654752440) { m = m * 2.0; e = e - 1; }
  const double s = (m - 1.0) / (m + 1.0);
  const double z = s * s;
  double t = 1.0 / 25.0;
  t = t * z + 1.0 / 23.0;
  t = t * z + 1.0 / 21.0;
  t = t * z + 1.0 / 19.0;
  t = t * z + 1.0 / 17.0;
  t = t * z + 1.0 / 15.0;
  t = t * z + 1.0 / 13.0;
  t = t * z + 1.0 / 11.0;
  t = t * z + 1.0 / 9.0;
  t = t * z + 1.0 / 7.0;
  t = t * z + 1.0 / 5.0;
  t = t * z + 1.0 / 3.0;
  t = t * z + 1.0;
  return (double)e * 0.69314718055994530942 + 2.0 * s * t;
}

__device__ void det_sincos_2pi(double u, double *s, double *c) {
  const double q = u * 4.0;
  const int k = (int)q;
  const double f = q - (double)k;
  const double th = f * 1.57079632679489661923;
  const double z = th * th;
  double sn = -1.0 / 15511210043330985984000000.0;
  sn = sn * z + 1.0 / 25852016738884976640000.0;
  sn = sn * z - 1.0 / 51090942171709440000.0;
  sn = sn * z + 1.0 / 121645100408832000.0;
  sn = sn * z - 1.0 / 355687428096000.0;
  sn = sn * z + 1.0 / 1307674368000.0;
  sn = sn * z - 1.0 / 6227020800.0;
  sn = sn * z + 1.0 / 39916800.0;
  sn = sn * z - 1.0 / 362880.0;
  sn = sn * z + 1.0 / 5040.0;
  sn = sn * z - 1.0 / 120.0;
  sn = sn * z + 1.0 / 6.0;
  sn = sn * z - 1.0;
  sn = -(sn * th);
  double cs = 1.0 / 620448401733239439360000.0;
  cs = cs * z - 1.0 / 1124000727777607680000.0;
  cs = cs * z + 1.0 / 2432902008176640000.0;
  cs = cs * z - 1.0 / 6402373705728000.0;
  cs = cs * z + 1.0 / 20922789888000.0;
  cs = cs * z - 1.0 / 87178291200.0;
  cs = cs * z + 1.0 / 479001600.0;
  cs = cs * z - 1.0 / 3628800.0;
  cs = cs * z + 1.0 / 40320.0;
  cs = cs * z - 1.0 / 720.0;
  cs = cs * z + 1.0 / 24.0;
  cs = cs * z - 0.5;
  cs = cs * z + 1.0;
  switch (k & 3) {
    case 0: *s = sn; *c = cs; break;
    case 1: *s = cs; *c = -sn; break;
    case 2: *s = -sn; *c = -cs; break;
    default: *s = -cs; *c = sn; break;
  }
}

constexpr double kDT = 0.05, kH2 = 0.00125, kKP = 16.0, kKD = 5.6, kSigmaW = 4.0;

// The table in two launches.  Gaussians of every (particle, step) are
// independent: one thread each (Philox, Box-Muller) into a binary64 buffer
// z[t][p][3].  The closed-loop recurrence is sequential in time only: one
// thread per (particle, axis) runs it over the steps.  (A binary64 warp
// instruction occupies this GPU's FP64 pipe for the same time whether one
// lane or 32 are active, so the recurrence must not run in one lane of a warp
// while the others wait.)  Each value is produced by the same operations in
// the same order as a scalar loop, without contraction.
__global__ void __launch_bounds__(256) particle_gauss_kernel(uint32_t k0, uint32_t k1, int P, int T,
                                                             double *__restrict__ z) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)P * T) return;
  const int t = (int)(i / P), p = (int)(i - (long long)t * P);
  const double sc = 2.3283064365386962890625e-10;  // 2^-32
  uint32_t o[4];
  philox4x32_10((uint32_t)p, (uint32_t)t, 0u, 0u, k0, k1, o);
  const double u0 = ((double)o[0] + 0.5) * sc, u1 = ((double)o[1] + 0.5) * sc;
  const double u2 = ((double)o[2] + 0.5) * sc, u3 = ((double)o[3] + 0.5) * sc;
  const double r0 = sqrt(-2.0 * det_log(u0));
  const double r1 = sqrt(-2.0 * det_log(u2));
  double s0, c0, s1, c1;
  det_sincos_2pi(u1, &s0, &c0);
  det_sincos_2pi(u3, &s1, &c1);
  z[i * 3 + 0] = r0 * c0;
  z[i * 3 + 1] = r0 * s0;
  z[i * 3 + 2] = r1 * c1;
}

__global__ void __launch_bounds__(128) particle_table_kernel(const double *__restrict__ z, int P,
                                                             int T, float *__restrict__ tmajor,
                                                             float *__restrict__ pmajor) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P * 3) return;
  const int p = i / 3, d = i - 3 * (i / 3);
  double pos = 0, vel = 0;
  for (int t = 0; t < T; ++t) {
    const float v = (float)pos;
    if (tmajor) tmajor[((long long)t * P + p) * 3 + d] = v;
    if (pmajor) pmajor[((long long)p * T + t) * 3 + d] = v;
    const double a = kSigmaW * z[((long long)t * P + p) * 3 + d] - (kKP * pos + kKD * vel);
    const double pn = (pos + kDT * vel) + kH2 * a;
    const double vn = vel + kDT * a;
    pos = pn;
    vel = vn;
  }
}

// Per-axis position variance of the same closed loop: S' = A S A^T + g g^T
// with A = [[1 - H2 KP, DT - H2 KD], [-DT KP, 1 - DT KD]] and g = [H2, DT]
// sigma_w, from S = 0 (the particles start on the path).  A sequential
// recurrence of a few hundred steps: one thread, binary64.
__global__ void position_variance_kernel(int T, double *__restrict__ var) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const double a00 = 1.0 - kH2 * kKP, a01 = kDT - kH2 * kKD;
  const double a10 = -(kDT * kKP), a11 = 1.0 - kDT * kKD;
  const double g0 = kH2 * kSigmaW, g1 = kDT * kSigmaW;
  double spp = 0, spv = 0, svv = 0;
  for (int t = 0; t < T; ++t) {
    var[t] = spp;
    const double m00 = a00 * spp + a01 * spv, m01 = a00 * spv + a01 * svv;
    const double m10 = a10 * spp + a11 * spv, m11 = a10 * spv + a11 * svv;
    const double npp = m00 * a00 + m01 * a01 + g0 * g0;
    const double npv = m00 * a10 + m01 * a11 + g0 * g1;
    const double nvv = m10 * a10 + m11 * a11 + g1 * g1;
    spp = npp;
    spv = npv;
    svv = nvv;
  }
}

// ------------------------------------------------------------------ HSMC
// One warp per new path.  Lane l owns particles p = 32k + l (k < words), one
// bit per particle in bits[k/32] bit (k%32), so offset loads of a k-step are
// 32 consecutive particles (384 contiguous bytes) and word k of the packed
// mask is a single __ballot_sync.  The warp first finds the edge's W x H
// half-space slots that are active (the reference skips a half-space when
// b >= 1000, PUMP.cu:642); with none active the new mask is the parent's and
// only the hit count is computed.  Every active half-space is tested for
// every particle exactly as PUMP.cu:645-651 does (binary32, no
// contraction); AND-ing the tests in another order gives the same bits.
//
// Two sources of half-spaces.  Cached: the arrays of pump_cache_halfspaces
// (dense, or sparse with per-waypoint counts).  Boxes: the warp derives
// them itself from the edge's waypoints and the obstacle set staged in
// shared memory, with the same operations (halfspace_of_box), into its own
// shared-memory slots.  It first drops the boxes that no waypoint of the
// edge can bring within the distance gate (gate_keeps_box on the waypoints'
// bounding box; none dropped when a waypoint is NaN or there are more than
// kHsmcFilterObs boxes), then per waypoint takes the remaining boxes 32 at a
// time, one per lane: the lanes whose box passes the gate are ranked by a
// ballot and the first maxHS - stored of them, in index order, fill the next
// slots, which are the slots cacheHalfspaces fills.  Only the edges a
// wavefront propagates along get half-spaces, and no cache is written.
constexpr int kMaxHsmcWords = 128;   // P <= 4096 particles
constexpr int kMaxHsSlots = 256;     // W * maxHS <= 256
constexpr int kHsmcThreads = 128;
constexpr int kHsmcWarps = kHsmcThreads / 32;
// blocks of a launch that loops over a device-side path count
constexpr int kHsmcPersistBlocks = kNumSMs * 8;
// Paths per block chunk: a block's warps take the chunk's paths one at a
// time from a shared-memory counter, so a warp whose paths are cheap (no
// active half-space: the parent's masks copied) takes more of them while
// another tests particles, instead of leaving its slot idle until the
// block's slowest warp ends.
// Two paths per warp: a mid-size wavefront (a few thousand paths) still
// spreads over every warp of the launch.
constexpr int kHsmcChunk = 2 * kHsmcWarps;
constexpr int kHsmcFilterObs = 128;


// Shared memory of the boxes variant: the staged boxes, then per warp its
// half-space slots (a0, a1, a2, b), stored counts per waypoint and the list
// of boxes that survive the edge's gate bound.
__host__ __device__ inline size_t hsmc_boxes_obs_floats(int numObs) {
  return (size_t)((numObs * 12 + 3) & ~3);
}
// Per warp: W * maxHS half-space slots and W stored counts (rounded to 16
// bytes), sized for the launch's W and maxHS.
__host__ __device__ inline int hsmc_hs_stride(int W, int maxHS) { return W * maxHS; }
__host__ __device__ inline int hsmc_cnt_stride(int W) { return (W + 15) & ~15; }
__host__ __device__ inline size_t hsmc_boxes_smem(int numObs, int W, int maxHS) {
  return sizeof(float) * hsmc_boxes_obs_floats(numObs) +
         (size_t)kHsmcWarps * (sizeof(float4) * hsmc_hs_stride(W, maxHS) + hsmc_cnt_stride(W) +
                               sizeof(int) * kHsmcFilterObs);
}

// New path w (the whole warp).  valid_in[prev] is read, valid_out[w] /
// cp_out[w] written (the two may alias one path store with valid_out =
// store + base, as in the reference).  With hs_count (stored half-spaces per
// waypoint), slots at or past a waypoint's count are inactive without
// reading them (they hold the defaults b = 1111 in the dense layout); stored
// slots still need b < 1000.
template <bool Boxes, int Q>
__device__ __forceinline__ void hsmc_path(const HsmcParams &p, int w, const float *s_obs,
                                          float4 *hs, uint8_t *hcnt, int *klist) {
  const int lane = threadIdx.x & 31;
  const unsigned int lt = (1u << lane) - 1u;
  const int edge = p.wf_edge[w], prev = p.wf_prev[w];
  if (edge < 0 || edge >= p.num_edges || prev < 0 || prev >= p.num_prev) {
    if (lane == 0 && p.error) atomicExch(p.error, (int)PUMP_ERR_BAD_INPUT);
    return;
  }
  // the edge's waypoints: W records per edge, or its own range (at most p.W)
  int W = p.W;
  long long wp0 = (long long)edge * W;
  if (Boxes && p.disc_off) {
    wp0 = p.disc_off[edge];
    const long long n = p.disc_off[edge + 1] - wp0;
    if (n < 2 || n > p.W) {
      if (lane == 0 && p.error) atomicExch(p.error, (int)PUMP_ERR_BAD_INPUT);
      return;
    }
    W = (int)n;
  }
  const int maxHS = p.maxHS, P = p.P;
  const int words = (P + 31) >> 5;
  const int slots = W * maxHS;
  const long long hsHead = (long long)edge * slots;
  // parent's words: lane j holds words j, j+32, ... (issued first: their
  // latency overlaps the half-space work)
  uint32_t mine[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int j = q * 32 + lane;
    mine[q] = (j < words) ? p.valid_in[(long long)prev * words + j] : 0u;
  }
  if (Boxes) {
    // lane i holds waypoint i (W <= 32; otherwise waypoints are read per step)
    const float *ew = p.disc + wp0 * kDim;
    float my[kDim];
    const int mi = lane < W ? lane : 0;
#pragma unroll
    for (int d = 0; d < kDim; ++d) my[d] = __ldg(&ew[mi * kDim + d]);
    // the edge's waypoints bound the boxes worth testing
    float mn[3], mx[3];
    bool nan = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      mn[d] = mx[d] = my[d];
      nan = nan || my[d] != my[d];
    }
    for (int i = lane + 32; i < W; i += 32)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float x = __ldg(&ew[i * kDim + d]);
        nan = nan || x != x;
        mn[d] = fminf(mn[d], x);
        mx[d] = fmaxf(mx[d], x);
      }
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
        mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
      }
    nan = __any_sync(0xffffffffu, nan);
    const bool filt = !nan && p.numObs <= kHsmcFilterObs;
    int nk = p.numObs;
    if (filt) {
      nk = 0;
      for (int o0 = 0; o0 < p.numObs; o0 += 32) {
        const int o = o0 + lane;
        const bool keep = o < p.numObs && gate_keeps_box(mn, mx, &s_obs[o * 12], p.maxd2);
        const unsigned int bal = __ballot_sync(0xffffffffu, keep);
        if (keep) klist[nk + __popc(bal & lt)] = o;
        nk += __popc(bal);
      }
    }
    for (int i = lane; i < W; i += 32) hcnt[i] = 0;
    __syncwarp();
    for (int i = 0; i < W && nk > 0; ++i) {
      float pos[3], vel[3];
      if (i < 32) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          pos[d] = __shfl_sync(0xffffffffu, my[d], i);
          vel[d] = __shfl_sync(0xffffffffu, my[3 + d], i);
        }
      } else {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          pos[d] = __ldg(&ew[i * kDim + d]);
          vel[d] = __ldg(&ew[i * kDim + 3 + d]);
        }
      }
      int stored = 0;
      for (int c0 = 0; c0 < nk && stored < maxHS; c0 += 32) {
        const int c = c0 + lane;
        float ah[3] = {0.0f, 0.0f, 0.0f}, bh = 0.0f;
        bool pass = false;
        if (c < nk) {
          const int o = filt ? klist[c] : c;
          pass = halfspace_of_box(pos, vel, &s_obs[o * 12], p.maxd2, ah, &bh);
        }
        const unsigned int bal = __ballot_sync(0xffffffffu, pass);
        const int rank = __popc(bal & lt);
        if (pass && stored + rank < maxHS) hs[i * maxHS + stored + rank] = make_float4(ah[0], ah[1], ah[2], bh);
        const int got = __popc(bal);
        stored += got < maxHS - stored ? got : maxHS - stored;
      }
      if (lane == 0) hcnt[i] = (uint8_t)stored;
    }
    __syncwarp();
  }
  // which half-space slots are active (b < 1000 or NaN, as !(b >= 1000))
  uint32_t act[kMaxHsSlots / 32];
  int nact = 0;
#pragma unroll
  for (int c = 0; c < kMaxHsSlots / 32; ++c) {
    const int sidx = c * 32 + lane;
    bool a = false;
    if (c * 32 < slots && sidx < slots) {
      const int i = sidx / maxHS, s = sidx - i * maxHS;
      if (Boxes) {
        a = s < (int)hcnt[i] && !(hs[sidx].w >= 1000);
      } else {
        const bool stored = !p.hs_count || s < (int)__ldg(&p.hs_count[(long long)edge * W + i]);
        a = stored && !(__ldg(&p.bs[hsHead + sidx]) >= 1000);
      }
    }
    act[c] = (c * 32 < slots) ? __ballot_sync(0xffffffffu, a) : 0u;
    nact += __popc(act[c]);
  }
  int overflow = 0;
  if (nact > 0) {
    // unpack: bits[q] bit b = particle 32 * (32 q + b) + lane
    uint32_t bits[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      bits[q] = 0u;
      for (int b = 0; b < 32; ++b) {
        const int k = q * 32 + b;
        if (k >= words) break;
        const uint32_t wk = __shfl_sync(0xffffffffu, mine[q], b);
        bits[q] |= ((wk >> lane) & 1u) << b;
      }
    }
    const float dtLocal = p.topts[edge] / (W - 1);
    const float t0 = p.times[prev];
#pragma unroll
    for (int c = 0; c < kMaxHsSlots / 32; ++c) {
      uint32_t m = act[c];
      while (m) {
        const int sidx = c * 32 + __ffs(m) - 1;
        m &= m - 1;
        const int i = sidx / maxHS;
        const float time = t0 + i * dtLocal;
        int dtIdx = (int)(time / p.dt);
        if (dtIdx < 0 || dtIdx >= p.T_rows) {
          overflow = 1;
          dtIdx = dtIdx < 0 ? 0 : p.T_rows - 1;
        }
        float a0, a1, a2, b;
        if (Boxes) {
          const float4 h = hs[sidx];
          a0 = h.x;
          a1 = h.y;
          a2 = h.z;
          b = h.w;
        } else {
          b = __ldg(&p.bs[hsHead + sidx]);
          a0 = __ldg(&p.as[(hsHead + sidx) * 3 + 0]);
          a1 = __ldg(&p.as[(hsHead + sidx) * 3 + 1]);
          a2 = __ldg(&p.as[(hsHead + sidx) * 3 + 2]);
        }
        const float *row = p.offsets_t + (long long)dtIdx * p.Pmc * 3;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          if (q * 32 >= words) break;
          uint32_t bq = bits[q];
          if (bq == 0u) continue;  // this lane's particles of the group are all dead
          // the test of a particle already dead is computed and discarded,
          // so the loads do not wait on the bits and many are in flight
#pragma unroll 8
          for (int bb = 0; bb < 32; ++bb) {
            const int k = q * 32 + bb;
            const int pp = 32 * k + lane;
            if (k < words && pp < P) {
              const float *off = row + (long long)pp * 3;
              float LHS = 0;
              LHS += __ldg(&off[0]) * a0;
              LHS += __ldg(&off[1]) * a1;
              LHS += __ldg(&off[2]) * a2;
              if (!(LHS * p.offset_mult < b)) bq &= ~(1u << bb);
            }
          }
          bits[q] = bq;
        }
      }
    }
    // repack: word k = ballot of bit k over lanes; lane (k & 31) keeps it
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      uint32_t keep = 0u;
      for (int b = 0; b < 32; ++b) {
        const int k = q * 32 + b;
        if (k >= words) break;
        const bool live = 32 * k + lane < P;
        const uint32_t wk = __ballot_sync(0xffffffffu, live && ((bits[q] >> b) & 1u));
        if (b == lane) keep = wk;
      }
      mine[q] = keep;
    }
  }
  int valid_count = 0;
  const uint32_t tail = (P & 31) ? ((1u << (P & 31)) - 1u) : 0xffffffffu;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int j = q * 32 + lane;
    if (j < words) {
      if (j == words - 1) mine[q] &= tail;  // no bits past particle P-1
      p.valid_out[(long long)w * words + j] = mine[q];
      valid_count += __popc(mine[q]);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) valid_count += __shfl_down_sync(0xffffffffu, valid_count, off);
  if (lane == 0) {
    const float cp = ((float)(P - valid_count)) / P;
    p.cp_out[w] = cp;
    if (overflow && p.error) atomicExch(p.error, (int)PUMP_ERR_CAPACITY);
    if (p.epi_on) {
      // PUMP.cu:164-185: time, cost and the CP cut-off of new path w
      const HsmcEpilogue &e = p.epi;
      const int f = e.wf_open[w];
      e.new_time[w] = e.path_time[prev] + e.topt[f];
      e.new_cost[w] = e.path_cost[prev] + e.copt[f];
      const bool alive = !(cp > e.cp_cutoff);
      e.alive[w] = alive ? 1 : 0;
      if (alive) e.new_next[w] = atomicExch(&e.new_head[e.wf_node[w]], w);
    }
  }
}

template <bool Boxes, int Q>
__device__ __forceinline__ void hsmc_run(const HsmcParams &p) {
  extern __shared__ float4 s_dyn4[];
  const int warp = threadIdx.x >> 5;
  int n = p.num_new;
  if (p.num_new_dev) n = (p.skip_dev && *p.skip_dev) ? 0 : (int)*p.num_new_dev;
  // a block with no path leaves before staging anything (block-uniform)
  if ((long long)blockIdx.x * kHsmcChunk >= n) return;
  float *s_obs = reinterpret_cast<float *>(s_dyn4);
  float4 *hs = nullptr;
  uint8_t *hcnt = nullptr;
  int *klist = nullptr;
  if (Boxes) {
    stage_obstacles(p.obs, p.numObs, s_obs);  // block-wide, before any warp leaves
    const int hs_stride = hsmc_hs_stride(p.W, p.maxHS), cnt_stride = hsmc_cnt_stride(p.W);
    float4 *s_hs = reinterpret_cast<float4 *>(s_obs + hsmc_boxes_obs_floats(p.numObs));
    hs = s_hs + warp * hs_stride;
    uint8_t *s_cnt = reinterpret_cast<uint8_t *>(s_hs + kHsmcWarps * hs_stride);
    hcnt = s_cnt + warp * cnt_stride;
    int *s_klist = reinterpret_cast<int *>(s_cnt + kHsmcWarps * cnt_stride);
    klist = s_klist + warp * kHsmcFilterObs;
  }
  __shared__ int s_next;
  const int lane = threadIdx.x & 31;
  const long long nchunks = ((long long)n + kHsmcChunk - 1) / kHsmcChunk;
  for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {  // block-uniform
    __syncthreads();  // every warp is done with the previous chunk's counter
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    const long long base = ch * kHsmcChunk;
    const int cnt = (int)((long long)n - base < kHsmcChunk ? (long long)n - base : kHsmcChunk);
    while (true) {
      int t = 0;
      if (lane == 0) t = atomicAdd(&s_next, 1);
      t = __shfl_sync(0xffffffffu, t, 0);
      if (t >= cnt) break;  // warp-uniform
      hsmc_path<Boxes, Q>(p, (int)(base + t), s_obs, hs, hcnt, klist);
      __syncwarp();  // the warp's half-space slots are rewritten by its next path
    }
  }
}

// Q = 32-bit particle words per lane: P <= 1024 Q.
template <bool Boxes, int Q>
__global__ void __launch_bounds__(kHsmcThreads, 8) hsmc_kernel(const HsmcParams p) {
  hsmc_run<Boxes, Q>(p);
}

// The search loop on the device, for every query of a group: the chunks of
// the active queries' wavefronts in query order are the blocks' work items,
// taken in turn (grid-stride).  A block stages a query's parameters (the
// stored-path count, the bound on parents, from its loop state) and boxes
// when its next chunk belongs to another query.  The shared memory holds the
// layout of the group's largest box count, waypoint count and half-space
// count.
template <int Q>
__global__ void __launch_bounds__(kHsmcThreads, 8) hsmc_loop_kernel(const LoopGroup *g) {
  extern __shared__ float4 s_dyn4[];
  __shared__ int s_first[kLoopGroupMax + 1];  // first chunk of each query
  __shared__ HsmcParams s_p;
  __shared__ int s_next;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nq = g->nq;
  if (warp == 0) {
    int c = 0;
    if (lane < nq) {
      const LoopArgs *a = g->args[lane];
      if (*reinterpret_cast<const volatile int *>(&a->L.active)) {
        const HsmcParams &hp = a->hp;
        const int n = (hp.skip_dev && *hp.skip_dev) ? 0 : (int)*hp.num_new_dev;
        c = (n + kHsmcChunk - 1) / kHsmcChunk;
      }
    }
    // inclusive scan over the queries (nq <= 32 lanes)
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, c, o);
      if (lane >= o) c += u;
    }
    if (lane == 0) s_first[0] = 0;
    if (lane < kLoopGroupMax) s_first[lane + 1] = c;
  }
  __syncthreads();
  const int total = s_first[nq];
  // a block with no chunk leaves before staging anything (block-uniform)
  if ((int)blockIdx.x >= total) return;
  float *s_obs = reinterpret_cast<float *>(s_dyn4);
  int cur = -1;
  for (int ch = blockIdx.x; ch < total; ch += gridDim.x) {  // block-uniform
    int q = 0;
    while (q + 1 < nq && s_first[q + 1] <= ch) ++q;
    __syncthreads();  // every warp is done with the previous chunk (its counter, its query)
    if (q != cur) {
      if (warp == 0) {  // the query's parameters, word by word
        static_assert(sizeof(HsmcParams) % sizeof(int) == 0, "HsmcParams words");
        const int *src = reinterpret_cast<const int *>(&g->args[q]->hp);
        int *dst = reinterpret_cast<int *>(&s_p);
        for (int i = lane; i < (int)(sizeof(HsmcParams) / sizeof(int)); i += 32) dst[i] = src[i];
        __syncwarp();
        if (lane == 0) s_p.num_prev = g->args[q]->L.num_paths;
      }
      __syncthreads();
      stage_obstacles(s_p.obs, s_p.numObs, s_obs);  // ends with a barrier
      cur = q;
    }
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    const HsmcParams p = s_p;
    // this query's layout of the shared memory
    const int hs_stride = hsmc_hs_stride(p.W, p.maxHS), cnt_stride = hsmc_cnt_stride(p.W);
    float4 *s_hs = reinterpret_cast<float4 *>(s_obs + hsmc_boxes_obs_floats(p.numObs));
    uint8_t *s_cnt = reinterpret_cast<uint8_t *>(s_hs + kHsmcWarps * hs_stride);
    int *s_klist = reinterpret_cast<int *>(s_cnt + kHsmcWarps * cnt_stride);
    const int n = (p.skip_dev && *p.skip_dev) ? 0 : (int)*p.num_new_dev;
    const int base = (ch - s_first[q]) * kHsmcChunk;
    const int cnt = n - base < kHsmcChunk ? n - base : kHsmcChunk;
    while (true) {
      int t = 0;
      if (lane == 0) t = atomicAdd(&s_next, 1);
      t = __shfl_sync(0xffffffffu, t, 0);
      if (t >= cnt) break;  // warp-uniform
      hsmc_path<true, Q>(p, base + t, s_obs, s_hs + warp * hs_stride, s_cnt + warp * cnt_stride,
                         s_klist + warp * kHsmcFilterObs);
      __syncwarp();  // the warp's half-space slots are rewritten by its next path
    }
  }
}

// The kernel of P particles (Q = ceil(P / 1024), 1, 2 or 4).
inline int hsmc_q(int P) {
  const int q = (P + 1023) / 1024;
  return q <= 1 ? 1 : (q <= 2 ? 2 : 4);
}
template <bool Boxes>
const void *hsmc_kernel_for(int P) {
  switch (hsmc_q(P)) {
    case 1: return (const void *)hsmc_kernel<Boxes, 1>;
    case 2: return (const void *)hsmc_kernel<Boxes, 2>;
    default: return (const void *)hsmc_kernel<Boxes, 4>;
  }
}
inline const void *hsmc_loop_kernel_for(int P) {
  switch (hsmc_q(P)) {
    case 1: return (const void *)hsmc_loop_kernel<1>;
    case 2: return (const void *)hsmc_loop_kernel<2>;
    default: return (const void *)hsmc_loop_kernel<4>;
  }
}

// -------------------------------------------------------------- MC CP
// collisionProbability.cu:39-92.  A particle collides when any of the
// segments t = 0 .. T-3 of its perturbed path hits a box; the reference walks
// the segments in order and stops at the first hit, which gives the same
// answer as testing all of them.  Block = 32 particles (the lanes) x
// kMcWarps warps; warp w tests segments t = w, w + kMcWarps, ...; the
// per-particle OR over warps is taken in shared memory and the block adds
// its popcount to hits[k].  Grid (ceil(Pmc / 32), paths).
// MC CP of path k (blockIdx.y): 32 particles per block (one per lane), the
// kMcWarps warps splitting the path's segments (16: a smoothing batch of a
// few paths is a few hundred blocks, so the segments are split finely to
// shorten each warp's chain).  With rowmax (the largest |offset|
// per table row and axis), each block first marks, per segment, the boxes
// that some particle's segment could touch: the path segment's bounding box
// widened by fl(rowmax * |offset_mult|) on both ends.  A particle's position
// fl(path + fl(offset * offset_mult)) lies inside that box by the
// monotonicity of rounding, so a box disjoint from it is broadphase-disjoint
// from every particle's segment and the reference's test of it passes; only
// the marked boxes are tested, in index order.  Without rowmax (or with more
// than kMcFilterObs boxes, or a NaN state) every box is tested.
constexpr int kMcFilterObs = 128;
constexpr int kMcWarps = 16;

__global__ void __launch_bounds__(32 * kMcWarps) mc_cp_kernel(
    const float *__restrict__ paths, const int *__restrict__ offset, const int *__restrict__ len,
    const float *__restrict__ offsets_t, int Pmc, int T_rows, float offset_mult,
    const float *__restrict__ obs, int numObs, int k0, int *__restrict__ hits,
    const float *__restrict__ rowmax, const int *copy_src, int *copy_dst, int copy_words,
    unsigned int *done, unsigned int seq) {
  extern __shared__ float4 s_obs4[];
  float *s_obs = reinterpret_cast<float *>(s_obs4);
  uint32_t *s_mask = reinterpret_cast<uint32_t *>(s_obs + ((numObs * 12 + 3) & ~3));
  __shared__ unsigned int s_hit[kMcWarps];
  stage_obstacles(obs, numObs, s_obs);
  const int k = k0 + blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p = blockIdx.x * 32 + lane;
  const int T = len[k];
  const float *path = paths + (long long)offset[k] * kDim;
  const bool filter = rowmax != nullptr && numObs <= kMcFilterObs && T <= T_rows;
  if (filter) {
    const float om = fabsf(offset_mult);
    for (int t = threadIdx.x; t < T - 2; t += blockDim.x) {
      float lo[3], hi[3];
      bool nan = false;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float m0 = rowmax[t * 3 + d] * om, m1 = rowmax[(t + 1) * 3 + d] * om;
        const float a = path[t * kDim + d], b = path[(t + 1) * kDim + d];
        nan = nan || a != a || b != b;
        lo[d] = fminf(a - m0, b - m1);
        hi[d] = fmaxf(a + m0, b + m1);
      }
      uint32_t m[kMcFilterObs / 32] = {0u, 0u, 0u, 0u};
      for (int o = 0; o < numObs; ++o)
        if (nan || !broadphase_valid(lo, hi, &s_obs[o * 12])) m[o >> 5] |= 1u << (o & 31);
#pragma unroll
      for (int q = 0; q < kMcFilterObs / 32; ++q) s_mask[t * (kMcFilterObs / 32) + q] = m[q];
    }
    __syncthreads();
  }
  bool coll = false;
  if (p < Pmc && T <= T_rows) {
    const int words = (numObs + 31) / 32;
    for (int t = warp; t < T - 2 && !coll; t += kMcWarps) {
      float v[3], w[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        v[d] = path[t * kDim + d] + __ldg(&offsets_t[((long long)t * Pmc + p) * 3 + d]) * offset_mult;
        w[d] = path[(t + 1) * kDim + d] +
               __ldg(&offsets_t[((long long)(t + 1) * Pmc + p) * 3 + d]) * offset_mult;
      }
      coll = filter ? !segment_valid_masked(v, w, &s_mask[t * (kMcFilterObs / 32)], words, s_obs)
                    : !segment_valid(v, w, numObs, s_obs);
    }
  }
  const unsigned int bal = __ballot_sync(0xffffffffu, coll);
  if (lane == 0) s_hit[warp] = bal;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int any = 0;
    for (int q = 0; q < kMcWarps; ++q) any |= s_hit[q];
    const int total = __popc(any);
    if (total) atomicAdd(&hits[k], total);
  }
  if (copy_dst) {
    // the last block to finish copies the caller's results (hit counts
    // included) to host memory
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
      __threadfence();
      s_last = atomicAdd(done, 1u) == gridDim.x * gridDim.y - 1;
    }
    __syncthreads();
    if (s_last) {
      __threadfence();
      const volatile int *src = copy_src;
      for (int i = threadIdx.x; i < copy_words; i += blockDim.x) copy_dst[i] = src[i];
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence_system();
        // then the sequence word after the copy, for a host that waits on it
        *reinterpret_cast<volatile unsigned int *>(copy_dst + copy_words) = seq;
      }
    }
  }
}

// Largest |offset| per row and axis of the time-major table (T rows of P
// particles), for the MC CP box filter.
__global__ void particle_rowmax_kernel(const float *__restrict__ table, int P,
                                       float *__restrict__ rowmax) {
  const int t = blockIdx.x;
  float m[3] = {0.0f, 0.0f, 0.0f};
  for (int p = threadIdx.x; p < P; p += blockDim.x)
#pragma unroll
    for (int d = 0; d < 3; ++d) m[d] = fmaxf(m[d], fabsf(table[((long long)t * P + p) * 3 + d]));
  __shared__ float s_m[3][32];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float v = m[d];
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) s_m[d][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    float v = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmaxf(v, s_m[threadIdx.x][w]);
    rowmax[t * 3 + threadIdx.x] = v;
  }
}

__global__ void mc_cp_finish_kernel(const int *__restrict__ hits, const int *__restrict__ len,
                                    int n, int Pmc, int T_rows, float *__restrict__ cp,
                                    int *__restrict__ error) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  cp[k] = ((float)hits[k]) / ((float)Pmc);
  if (len[k] > T_rows && error) atomicExch(error, (int)PUMP_ERR_CAPACITY);
}

}  // namespace

pump_status_t particle_rowmax_async(const float *d_table, int P, int T, float *d_rowmax,
                                    cudaStream_t stream) {
  particle_rowmax_kernel<<<T, 256, 0, stream>>>(d_table, P, d_rowmax);
  return launch_status("particle_rowmax");
}

pump_status_t mc_cp_hits_async(const float *d_paths, const int *d_offset, const int *d_len,
                               int n_paths, const float *d_offsets_t, int Pmc, int T_rows,
                               float offset_mult, const float *d_obstacles, int numObs,
                               int *d_hits, cudaStream_t stream, const float *d_rowmax,
                               const int *copy_src, int *copy_dst, int copy_words,
                               unsigned int *done, unsigned int seq) {
  if (n_paths <= 0) return PUMP_OK;
  if (copy_dst && n_paths > 65535)
    return set_error(PUMP_ERR_BAD_INPUT, "mc_cp: copy-out with %d paths", n_paths);
  if (numObs > kMcFilterObs) d_rowmax = nullptr;
  size_t smem = sizeof(float) * (size_t)((numObs * 12 + 3) & ~3);
  if (d_rowmax) smem += sizeof(uint32_t) * (kMcFilterObs / 32) * (size_t)T_rows;
  if (smem > 200 * 1024) {
    if (!d_rowmax) return set_error(PUMP_ERR_CAPACITY, "mc_cp: %d obstacles", numObs);
    d_rowmax = nullptr;  // masks for this many rows do not fit: test every box
    smem = sizeof(float) * (size_t)((numObs * 12 + 3) & ~3);
    if (smem > 200 * 1024) return set_error(PUMP_ERR_CAPACITY, "mc_cp: %d obstacles", numObs);
  }
  PUMP_TRY(smem_attr((const void *)mc_cp_kernel, smem));
  for (int k0 = 0; k0 < n_paths; k0 += 65535) {
    const int nk = n_paths - k0 < 65535 ? n_paths - k0 : 65535;
    dim3 grid(grid_for(Pmc, 32), (unsigned)nk);
    mc_cp_kernel<<<grid, 32 * kMcWarps, smem, stream>>>(d_paths, d_offset, d_len, d_offsets_t, Pmc, T_rows,
                                              offset_mult, d_obstacles, numObs, k0, d_hits,
                                              d_rowmax, copy_src, copy_dst, copy_words, done,
                                              seq);
    PUMP_TRY(launch_status("mc_cp_kernel"));
  }
  return PUMP_OK;
}

pump_status_t mc_cp_async(const float *d_paths, const int *d_offset, const int *d_len, int n_paths,
                          const float *d_offsets_t, int Pmc, int T_rows, float offset_mult,
                          const float *d_obstacles, int numObs, int *d_hits, float *d_cp,
                          int *d_error, cudaStream_t stream, const float *d_rowmax) {
  if (n_paths <= 0) return PUMP_OK;
  PUMP_CUDA_TRY(cudaMemsetAsync(d_hits, 0, sizeof(int) * n_paths, stream));
  PUMP_TRY(mc_cp_hits_async(d_paths, d_offset, d_len, n_paths, d_offsets_t, Pmc, T_rows,
                            offset_mult, d_obstacles, numObs, d_hits, stream, d_rowmax, nullptr,
                            nullptr, 0, nullptr, 0u));
  mc_cp_finish_kernel<<<grid_for(n_paths, 128), 128, 0, stream>>>(d_hits, d_len, n_paths, Pmc,
                                                                  T_rows, d_cp, d_error);
  return launch_status("mc_cp_finish_kernel");
}

pump_status_t hsmc_staged_async(int num_new, int W, const int *d_edge, const int *d_prev,
                                long long num_edges, int num_prev, const float *d_as, const float *d_bs, int maxHS,
                                const float *d_times, const float *d_topt, float dt,
                                const float *d_offsets_t, int Pmc, int T_rows, float offset_mult,
                                const uint32_t *d_valid_in, uint32_t *d_valid_out, int P,
                                float *d_cp_out, int *d_error, const uint8_t *d_hs_count,
                                cudaStream_t stream, const unsigned long long *d_num_new,
                                const int *d_skip) {
  if (num_new <= 0) return PUMP_OK;
  if ((P + 31) / 32 > kMaxHsmcWords)
    return set_error(PUMP_ERR_CAPACITY, "hsmc: %d particles exceed %d", P, 32 * kMaxHsmcWords);
  if (W * maxHS > kMaxHsSlots)
    return set_error(PUMP_ERR_CAPACITY, "hsmc: %d half-space slots per edge exceed %d", W * maxHS,
                     kMaxHsSlots);
  HsmcParams hp{};
  hp.num_new = num_new;
  hp.W = W;
  hp.wf_edge = d_edge;
  hp.wf_prev = d_prev;
  hp.num_edges = num_edges;
  hp.num_prev = num_prev;
  hp.as = d_as;
  hp.bs = d_bs;
  hp.hs_count = d_hs_count;
  hp.maxHS = maxHS;
  hp.times = d_times;
  hp.topts = d_topt;
  hp.dt = dt;
  hp.offsets_t = d_offsets_t;
  hp.Pmc = Pmc;
  hp.T_rows = T_rows;
  hp.offset_mult = offset_mult;
  hp.valid_in = d_valid_in;
  hp.valid_out = d_valid_out;
  hp.P = P;
  hp.cp_out = d_cp_out;
  hp.error = d_error;
  hp.num_new_dev = d_num_new;
  hp.skip_dev = d_skip;
  // with a device-side count, num_new bounds it
  const long long want = ((long long)num_new + kHsmcChunk - 1) / kHsmcChunk;
  const unsigned blocks = d_num_new ? (unsigned)(want < kHsmcPersistBlocks ? want : kHsmcPersistBlocks)
                                    : grid_for(num_new, kHsmcChunk);
  void *args[] = {(void *)&hp};
  PUMP_CUDA_TRY(cudaLaunchKernel(hsmc_kernel_for<false>(P), dim3(blocks), dim3(kHsmcThreads), args,
                                 0, stream));
  return launch_status("hsmc_kernel");
}

bool hsmc_boxes_fits(int numObs, int W, int maxHS) {
  return numObs >= 0 && W <= kMaxHsSlots && W * maxHS <= kMaxHsSlots &&
         hsmc_boxes_smem(numObs, W, maxHS) <= 220 * 1024;
}

pump_status_t hsmc_boxes_fill(int num_new, int W, const int *d_edge, const int *d_prev,
                              long long num_edges, int num_prev, const float *d_obs, int numObs,
                              const float *d_disc, float maxd2, int maxHS, const float *d_times,
                              const float *d_topt, float dt, const float *d_offsets_t, int Pmc,
                              int T_rows, float offset_mult, const uint32_t *d_valid_in,
                              uint32_t *d_valid_out, int P, float *d_cp_out, int *d_error,
                              const unsigned long long *d_num_new, const int *d_skip,
                              const HsmcEpilogue *epi, HsmcParams *out,
                              const long long *d_disc_off) {
  if ((P + 31) / 32 > kMaxHsmcWords)
    return set_error(PUMP_ERR_CAPACITY, "hsmc: %d particles exceed %d", P, 32 * kMaxHsmcWords);
  if (!hsmc_boxes_fits(numObs, W, maxHS))
    return set_error(PUMP_ERR_CAPACITY, "hsmc: %d boxes or %d half-space slots per edge exceed the stage",
                     numObs, W * maxHS);
  HsmcParams hp{};
  hp.num_new = num_new;
  hp.W = W;
  hp.wf_edge = d_edge;
  hp.wf_prev = d_prev;
  hp.num_edges = num_edges;
  hp.num_prev = num_prev;
  hp.obs = d_obs;
  hp.numObs = numObs;
  hp.disc = d_disc;
  hp.disc_off = d_disc_off;
  hp.maxd2 = maxd2;
  hp.maxHS = maxHS;
  hp.times = d_times;
  hp.topts = d_topt;
  hp.dt = dt;
  hp.offsets_t = d_offsets_t;
  hp.Pmc = Pmc;
  hp.T_rows = T_rows;
  hp.offset_mult = offset_mult;
  hp.valid_in = d_valid_in;
  hp.valid_out = d_valid_out;
  hp.P = P;
  hp.cp_out = d_cp_out;
  hp.error = d_error;
  hp.num_new_dev = d_num_new;
  hp.skip_dev = d_skip;
  if (epi) {
    hp.epi = *epi;
    hp.epi_on = 1;
  }
  *out = hp;
  return PUMP_OK;
}

pump_status_t hsmc_boxes_async(int num_new, int W, const int *d_edge, const int *d_prev,
                               long long num_edges, int num_prev, const float *d_obs, int numObs,
                               const float *d_disc, float maxd2, int maxHS, const float *d_times,
                               const float *d_topt, float dt, const float *d_offsets_t, int Pmc,
                               int T_rows, float offset_mult, const uint32_t *d_valid_in,
                               uint32_t *d_valid_out, int P, float *d_cp_out, int *d_error,
                               cudaStream_t stream, const unsigned long long *d_num_new,
                               const int *d_skip, const HsmcEpilogue *epi,
                               const long long *d_disc_off) {
  if (num_new <= 0) return PUMP_OK;
  HsmcParams hp{};
  PUMP_TRY(hsmc_boxes_fill(num_new, W, d_edge, d_prev, num_edges, num_prev, d_obs, numObs, d_disc,
                           maxd2, maxHS, d_times, d_topt, dt, d_offsets_t, Pmc, T_rows, offset_mult,
                           d_valid_in, d_valid_out, P, d_cp_out, d_error, d_num_new, d_skip, epi,
                           &hp, d_disc_off));
  const size_t smem = hsmc_boxes_smem(numObs, W, maxHS);
  const void *kern = hsmc_kernel_for<true>(P);
  PUMP_TRY(smem_attr(kern, smem));
  // with a device-side count, num_new bounds it
  const long long want = ((long long)num_new + kHsmcChunk - 1) / kHsmcChunk;
  const unsigned blocks = d_num_new ? (unsigned)(want < kHsmcPersistBlocks ? want : kHsmcPersistBlocks)
                                    : grid_for(num_new, kHsmcChunk);
  void *args[] = {(void *)&hp};
  PUMP_CUDA_TRY(cudaLaunchKernel(kern, dim3(blocks), dim3(kHsmcThreads), args, smem, stream));
  return launch_status("hsmc_kernel (boxes)");
}

pump_status_t hsmc_loop_prepare(int numObs, int W, int maxHS, int P) {
  return smem_attr(hsmc_loop_kernel_for(P), hsmc_boxes_smem(numObs, W, maxHS));
}

pump_status_t hsmc_loop_launch(const LoopGroup *d_group, int numObs, int W, int maxHS, int P,
                               int blocks, cudaStream_t stream) {
  void *args[] = {(void *)&d_group};
  PUMP_CUDA_TRY(cudaLaunchKernel(hsmc_loop_kernel_for(P), dim3(blocks), dim3(kHsmcThreads), args,
                                 hsmc_boxes_smem(numObs, W, maxHS), stream));
  return launch_status("hsmc_loop_kernel");
}

// Generates the tables on `stream`; the binary64 noise buffer (24 B per
// particle and step) is allocated and freed in stream order.
pump_status_t particle_tables_async(uint64_t seed, int P, int T, float *d_tmajor, float *d_pmajor,
                                    cudaStream_t stream) {
  double *z = nullptr;
  PUMP_CUDA_TRY(pool_malloc_async((void **)&z, sizeof(double) * 3 * (size_t)P * T, stream));
  particle_gauss_kernel<<<grid_for((long long)P * T, 256), 256, 0, stream>>>(
      (uint32_t)seed, (uint32_t)(seed >> 32), P, T, z);
  pump_status_t st = launch_status("particle_gauss_kernel");
  if (st == PUMP_OK) {
    particle_table_kernel<<<grid_for((long long)P * 3, 128), 128, 0, stream>>>(z, P, T, d_tmajor,
                                                                              d_pmajor);
    st = launch_status("particle_table_kernel");
  }
  cudaFreeAsync(z, stream);
  return st;
}

}  // namespace pump

using namespace pump;

extern "C" pump_status_t pump_particle_tables(uint64_t seed, int P, int T, float *d_tmajor,
                                              float *d_pmajor, pump_stream_t stream) {
  if (P <= 0 || T <= 0 || (!d_tmajor && !d_pmajor))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_particle_tables: bad arguments");
  return particle_tables_async(seed, P, T, d_tmajor, d_pmajor, (cudaStream_t)stream);
}

extern "C" pump_status_t pump_position_variance(int T, double *d_var, pump_stream_t stream) {
  if (T <= 0 || !d_var) return set_error(PUMP_ERR_BAD_INPUT, "pump_position_variance: bad arguments");
  position_variance_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(T, d_var);
  return launch_status("position_variance");
}

extern "C" pump_status_t pump_hsmc_propagate(int num_new, int W, const int *d_edge, const int *d_prev,
                                             long long num_edges, int base, const float *d_as,
                                             const float *d_bs,
                                             int maxHS, const float *d_times, const float *d_topt,
                                             float dt, const float *d_offsets_t, int Pmc,
                                             int T_rows, float offset_mult, uint32_t *d_valid,
                                             int P, float *d_path_cp, int *d_error,
                                             const uint8_t *d_hs_count, pump_stream_t stream) {
  if (num_new < 0 || W < 2 || maxHS < 0 || P <= 0 || P > Pmc || T_rows <= 0 || base < 0 ||
      num_edges < 0 ||
      (num_new > 0 && (!d_edge || !d_prev || !d_times || !d_topt || !d_offsets_t || !d_valid ||
                       !d_path_cp || (maxHS > 0 && (!d_as || !d_bs)))))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_hsmc_propagate: bad arguments");
  const size_t words = (size_t)((P + 31) / 32);
  return hsmc_staged_async(num_new, W, d_edge, d_prev, num_edges, base, d_as, d_bs, maxHS, d_times,
                           d_topt, dt,
                           d_offsets_t, Pmc, T_rows, offset_mult, d_valid,
                           d_valid + (size_t)base * words, P, d_path_cp + base, d_error,
                           d_hs_count, (cudaStream_t)stream, nullptr, nullptr);
}

extern "C" pump_status_t pump_hsmc_propagate_boxes_off(
    int num_new, int max_w, const int *d_edge, const int *d_prev, long long num_edges, int base,
    const float *d_obstacles, int numObs, const float *d_disc, const long long *d_disc_off,
    float maxd2, int maxHS, const float *d_times, const float *d_topt, float dt,
    const float *d_offsets_t, int Pmc, int T_rows, float offset_mult, uint32_t *d_valid, int P,
    float *d_path_cp, int *d_error, pump_stream_t stream) {
  if (num_new < 0 || max_w < 2 || maxHS < 0 || P <= 0 || P > Pmc || T_rows <= 0 || base < 0 ||
      num_edges < 0 || numObs < 0 || (numObs > 0 && !d_obstacles) ||
      (num_new > 0 && (!d_edge || !d_prev || !d_times || !d_topt || !d_offsets_t || !d_valid ||
                       !d_path_cp || !d_disc || !d_disc_off)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_hsmc_propagate_boxes_off: bad arguments");
  const size_t words = (size_t)((P + 31) / 32);
  return hsmc_boxes_async(num_new, max_w, d_edge, d_prev, num_edges, base, d_obstacles, numObs,
                          d_disc, maxd2, maxHS, d_times, d_topt, dt, d_offsets_t, Pmc, T_rows,
                          offset_mult, d_valid, d_valid + (size_t)base * words, P, d_path_cp + base,
                          d_error, (cudaStream_t)stream, nullptr, nullptr, nullptr, d_disc_off);
}

extern "C" pump_status_t pump_hsmc_propagate_boxes(
    int num_new, int W, const int *d_edge, const int *d_prev, long long num_edges, int base,
    const float *d_obstacles, int numObs, const float *d_disc, float maxd2, int maxHS,
    const float *d_times, const float *d_topt, float dt, const float *d_offsets_t, int Pmc,
    int T_rows, float offset_mult, uint32_t *d_valid, int P, float *d_path_cp, int *d_error,
    pump_stream_t stream) {
  if (num_new < 0 || W < 2 || maxHS < 0 || P <= 0 || P > Pmc || T_rows <= 0 || base < 0 ||
      num_edges < 0 || numObs < 0 || (numObs > 0 && !d_obstacles) ||
      (num_new > 0 && (!d_edge || !d_prev || !d_times || !d_topt || !d_offsets_t || !d_valid ||
                       !d_path_cp || !d_disc)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_hsmc_propagate_boxes: bad arguments");
  const size_t words = (size_t)((P + 31) / 32);
  return hsmc_boxes_async(num_new, W, d_edge, d_prev, num_edges, base, d_obstacles, numObs, d_disc,
                          maxd2, maxHS, d_times, d_topt, dt, d_offsets_t, Pmc, T_rows, offset_mult,
                          d_valid, d_valid + (size_t)base * words, P, d_path_cp + base, d_error,
                          (cudaStream_t)stream, nullptr, nullptr, nullptr, nullptr);
}

extern "C" pump_status_t pump_mc_cp(const float *d_paths, const int *d_offset, const int *d_len,
                                    int n_paths, const float *d_offsets_t, int Pmc, int T_rows,
                                    float offset_mult, const float *d_obstacles, int numObs,
                                    int *d_hits, float *d_cp, int *d_error, pump_stream_t stream) {
  if (n_paths < 0 || Pmc <= 0 || T_rows <= 0 || numObs < 0 || (numObs > 0 && !d_obstacles) ||
      (n_paths > 0 && (!d_paths || !d_offset || !d_len || !d_offsets_t || !d_hits || !d_cp)))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_mc_cp: bad arguments");
  return mc_cp_async(d_paths, d_offset, d_len, n_paths, d_offsets_t, Pmc, T_rows, offset_mult,
                     d_obstacles, numObs, d_hits, d_cp, d_error, (cudaStream_t)stream, nullptr);
}
