// The bracket of the one-read rn selection (select.cu, bvp_precise.cu).
#pragma once
#include "common.cuh"

namespace pump {
namespace {

// The reference sorts all N(N-1) pair costs to read rn and then scans them
// again for the edges below rn.  Here a strided sample of kBracketSamples
// costs gives a key bound key_hi (the upper edge of the 22-bit key bin of the
// sample at a rank a few standard deviations above k): one compaction pass
// keeps the pairs with key < key_hi (the superset, in index order, a few
// percent of the pairs), the exact radix select for rank k runs over the
// superset only, and the edges are compacted from it.  Every pair below rn
// is in the superset whenever the superset holds more than k pairs, so rn
// and the edges are exactly those of the full select; when it does not (the
// sample misled) or the superset overflows its buffer, the host falls back to
// the three-pass select and the full compaction.
constexpr int kBracketSamples = 8192;

// Rank r among the 2048 counts of hist (a block of 1024 threads, two bins
// each): the bin and the rank within it land in *bin and *rem.
__device__ void find_bin_2048(const unsigned int *hist, unsigned int r, unsigned int *s_warp,
                              unsigned int *bin, unsigned int *rem) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const unsigned int h0 = hist[2 * t], h1 = hist[2 * t + 1];
  const unsigned int v = h0 + h1;
  unsigned int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const unsigned int w = s_warp[lane];
    unsigned int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned int u = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += u;
    }
    s_warp[lane] = wi - w;
  }
  __syncthreads();
  const unsigned int ex = s_warp[warp] + incl - v;
  if (r >= ex && r < ex + v) {
    if (r < ex + h0) {
      *bin = 2 * t;
      *rem = r - ex;
    } else {
      *bin = 2 * t + 1;
      *rem = r - ex - h0;
    }
  }
  __syncthreads();
}

// A block of 1024 threads, keys[kBracketSamples] (shared, complete): two
// 11-bit radix steps to the 22-bit key prefix of the key of the given rank;
// thread 0 stores *key_hi = the prefix's upper edge.
__device__ void bracket_radix(const uint32_t *keys, unsigned int rank,
                              unsigned long long *key_hi) {
  __shared__ unsigned int hist[2048];
  __shared__ unsigned int s_warp[32];
  __shared__ unsigned int s_bin, s_rem;
  const int t = threadIdx.x;
  uint32_t prefix = 0u, mask = 0u;
  unsigned int r = rank;
  for (int pass = 0; pass < 2; ++pass) {
    const int shift = pass == 0 ? 21 : 10;
    hist[2 * t] = 0u;
    hist[2 * t + 1] = 0u;
    __syncthreads();
    for (int q = t; q < kBracketSamples; q += 1024) {
      const uint32_t k = keys[q];
      if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 2047u], 1u);
    }
    __syncthreads();
    find_bin_2048(hist, r, s_warp, &s_bin, &s_rem);
    prefix |= s_bin << shift;
    mask |= 2047u << shift;
    r = s_rem;
  }
  if (t == 0) *key_hi = ((unsigned long long)(prefix >> 10) + 1ull) << 10;
}

}  // namespace
}  // namespace pump
