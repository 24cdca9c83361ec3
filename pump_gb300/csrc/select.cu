// Order statistics and stable compaction (reference: mainPUMP.cu:289-346,
// GMT.cu:48-76 and 166-176).
//
// rn selection: the reference sorts all N(N-1) pair costs (thrust::sort) and
// reads element floor(0.05 N(N-1)).  Here an exact three-pass radix select
// over order-preserving 32-bit keys (11, 11 and 10 bits) finds the same
// element with three reads of the array and no sort.
//
// Edge list and frontier: stable compaction (compact.cuh) of the pairs below
// rn and of the frontier flags.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "bracket.cuh"
#include "compact.cuh"
#include "rnfinish.cuh"
#include "ctx.h"
#include "pairview.cuh"

namespace pump {
namespace {


__device__ __forceinline__ uint32_t ldg_bits(const float *p) {
  return __ldg(reinterpret_cast<const unsigned int *>(p));
}

// ---------------------------------------------------------- radix select
struct SelectState {
  uint32_t prefix;
  uint32_t mask;
  unsigned long long k;
  uint32_t result;  // the bits of the k-th value
};

// Sources of pair costs: src.bits(idx) for pair number idx, and
// src.bits_at(idx, i, j) / src.at(idx, i, j) when the caller already knows
// the pair (i, j) of idx.
struct FlatSrc {
  static constexpr bool kPairs = false;
  const float *v;
  __device__ uint32_t bits(long long i) const { return ldg_bits(&v[i]); }
  __device__ uint32_t bits_at(long long i, int, int) const { return ldg_bits(&v[i]); }
  __device__ float at(long long i, int, int) const { return __ldg(&v[i]); }
};
struct PairCoptSrc {
  static constexpr bool kPairs = true;
  PairView pv;
  __device__ uint32_t bits(long long idx) const {
    int i, j;
    pv.pair(idx, &i, &j);
    return pv.copt_bits(i, j);
  }
  __device__ uint32_t bits_at(long long, int i, int j) const { return pv.copt_bits(i, j); }
  __device__ float at(long long, int i, int j) const { return pv.copt(i, j); }
};
// Optimal times of the same pairs.
struct FlatTopt {
  const float *v;
  __device__ float at(long long i, int, int) const { return __ldg(&v[i]); }
};
struct PairTopt {
  PairView pv;
  __device__ float at(long long, int i, int j) const { return pv.topt(i, j); }
};

constexpr int kSelectBatch = 8;
constexpr int kSelectThreads = 256;

// One block of kSelectThreads threads after a pass's histogram is complete:
// find the bin holding rank k, narrow the prefix, clear the histogram for
// the next pass.
__device__ void select_pick(SelectState *st, int shift, int bits, unsigned int *hist) {
  __shared__ unsigned long long cum[kSelectThreads];
  const int nb = 1 << bits;
  const int per = nb / kSelectThreads;  // 4 or 8 bins per thread
  const int t = threadIdx.x;
  unsigned long long mine = 0;
  for (int q = 0; q < per; ++q) mine += __ldcg(&hist[t * per + q]);
  cum[t] = mine;
  __syncthreads();
  for (int off = 1; off < kSelectThreads; off <<= 1) {  // inclusive Hillis-Steele scan
    unsigned long long add = t >= off ? cum[t - off] : 0;
    __syncthreads();
    cum[t] += add;
    __syncthreads();
  }
  const unsigned long long k = st->k;
  const unsigned long long before = cum[t] - mine;
  if (k >= before && k < cum[t]) {
    unsigned long long c = before;
    for (int q = 0; q < per; ++q) {
      const unsigned int h = __ldcg(&hist[t * per + q]);
      if (k < c + h) {
        const uint32_t bin = (uint32_t)(t * per + q);
        st->prefix |= bin << shift;
        st->mask |= (uint32_t)(nb - 1) << shift;
        st->k = k - c;
        if (shift == 0) st->result = bits_of_key(st->prefix);
        break;
      }
      c += h;
    }
  }
  __syncthreads();
  for (int q = 0; q < per; ++q) hist[t * per + q] = 0;
}

// Src(i) -> the i-th value (a flat array, or a virtual pair array).  One
// pass of the radix select: every block adds its keys' bins (under the
// state's prefix) to hist; the block that finishes last (a counter of
// finished blocks, *done, reset by that block) picks the bin of rank k.
template <class Src>
__global__ void __launch_bounds__(kSelectThreads) select_hist_kernel(Src src, long long n, const unsigned long long *d_n,
                                   SelectState *__restrict__ st, int shift, int bits,
                                   unsigned int *__restrict__ hist, unsigned int *done) {
  __shared__ unsigned int sh[2048];
  __shared__ bool s_last;
  const int nb = 1 << bits;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sh[b] = 0;
  __syncthreads();
  const uint32_t prefix = st->prefix, mask = st->mask;
  if (d_n && (long long)*d_n < n) n = (long long)*d_n;
  // kSelectBatch loads in flight per thread before their shared-memory atomics
  const long long stride = (long long)gridDim.x * blockDim.x * kSelectBatch;
  // the loop bound is the warp's first item, so all 32 lanes reach the match
  const long long w_first = blockIdx.x * (long long)blockDim.x * kSelectBatch + (threadIdx.x & ~31);
  for (long long w0 = w_first; w0 < n; w0 += stride) {
    const long long i0 = w0 + (threadIdx.x & 31);
    uint32_t key[kSelectBatch];
#pragma unroll
    for (int u = 0; u < kSelectBatch; ++u) {
      const long long i = i0 + (long long)u * blockDim.x;
      key[u] = i < n ? key_of_bits(src.bits(i)) : 0u;
    }
    // equal bins within a warp are added once (many costs share a bin)
#pragma unroll
    for (int u = 0; u < kSelectBatch; ++u) {
      const long long i = i0 + (long long)u * blockDim.x;
      const bool in = i < n && (key[u] & mask) == prefix;
      const uint32_t bin = in ? (key[u] >> shift) & (nb - 1) : 0xFFFFFFFFu;
      const unsigned int peers = __match_any_sync(0xffffffffu, bin);
      if (in && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&sh[bin], __popc(peers));
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    if (sh[b]) atomicAdd(&hist[b], sh[b]);
  // the last block to finish sees every block's additions
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  select_pick(st, shift, bits, hist);
  if (threadIdx.x == 0) *done = 0u;
}

// Start state of a selection, a cleared histogram and block counter (a
// kernel instead of a host-to-device copy: a copy from pageable host memory
// would wait for the stream to drain first).
__global__ void __launch_bounds__(1024) select_init_kernel(SelectState *st, unsigned long long k,
                                                           unsigned int *hist, unsigned int *done) {
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) hist[i] = 0u;
  if (threadIdx.x == 0) {
    st->prefix = 0u;
    st->mask = 0u;
    st->k = k;
    st->result = 0u;
    *done = 0u;
  }
}

// ------------------------------------------------------ compaction users
struct FlagPred {
  const uint8_t *flags;
  __device__ bool operator()(long long i) const { return flags[i] != 0; }
};
struct IndexEmit {
  int *out;
  __device__ void operator()(long long idx, long long pos) const { out[pos] = (int)idx; }
};

__global__ void copy_count_kernel(const unsigned long long *total, int *out) { *out = (int)*total; }

// ------------------------------------------------- rn and edges in one read
// (the bracket: bracket.cuh)
// One block of 1024 threads: the keys of the samples at positions
// floor((2q + 1) n / (2 S)), then the bracket's radix steps.
template <class Src>
__global__ void __launch_bounds__(1024) bracket_kernel(Src src, long long n, unsigned int rank,
                                                       unsigned long long *key_hi) {
  __shared__ uint32_t keys[kBracketSamples];
  for (int q = threadIdx.x; q < kBracketSamples; q += 1024) {
    const long long pos = ((2LL * q + 1) * n) / (2LL * kBracketSamples);
    keys[q] = key_of_bits(src.bits(pos));
  }
  __syncthreads();
  bracket_radix(keys, rank, key_hi);
}

// Row a and column j of this thread's items of the tile at base (item r is
// pair base + r * 256 + tid): one division per tile, then steps of 256.
// Items at or past n get values that are never used.
__device__ __forceinline__ void tile_pairs(long long base, int N, int (&a)[kCompactRows],
                                           int (&j)[kCompactRows]) {
  const long long i0 = base + threadIdx.x;
  int aa = (int)(i0 / (N - 1));
  int bb = (int)(i0 - (long long)aa * (N - 1));
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    if (r) {
      bb += kCompactThreads;
      while (bb >= N - 1) {
        bb -= N - 1;
        ++aa;
      }
    }
    a[r] = aa;
    j[r] = bb + (bb >= aa);
  }
}

// The superset: pairs with key < key_hi, written as (pair number, cost) at
// positions below cap.
template <class Src>
struct SupersetLoader {
  using Item = uint32_t;  // the cost's bits
  using State = unsigned long long;
  Src src;
  int N;
  const unsigned long long *key_hi;
  long long cap;
  uint32_t *out_idx;
  uint32_t *out_bits;
  __device__ State begin() const { return *key_hi; }
  __device__ void load(long long base, long long n, uint32_t (&c)[kCompactRows]) const {
    if constexpr (Src::kPairs) {
      int a[kCompactRows], j[kCompactRows];
      tile_pairs(base, N, a, j);
#pragma unroll
      for (int r = 0; r < kCompactRows; ++r) {
        const long long i = base + r * kCompactThreads + threadIdx.x;
        c[r] = i < n ? src.bits_at(i, a[r], j[r]) : 0u;
      }
    } else {
#pragma unroll
      for (int r = 0; r < kCompactRows; ++r) {
        const long long i = base + r * kCompactThreads + threadIdx.x;
        c[r] = i < n ? src.bits_at(i, 0, 0) : 0u;
      }
    }
  }
  __device__ bool sel(State key_hi_v, uint32_t c) const {
    return (unsigned long long)key_of_bits(c) < key_hi_v;
  }
  __device__ void emit(long long i, uint32_t c, long long pos) const {
    if (pos < cap) {
      out_idx[pos] = (uint32_t)i;
      out_bits[pos] = c;
    }
  }
};

// Edges (mainPUMP.cu:327-346): pairs with cost < rn as (i, j, copt, topt);
// the optimal time is read for the selected pairs only.
struct PairItem {
  float c;
  int a, j;
};
template <class Src, class Topt>
struct EdgeLoader {
  using Item = PairItem;
  using State = int;
  Src src;
  Topt tsrc;
  int N;
  float rn;
  long long cap;
  int *e_src, *e_dst;
  float *e_copt, *e_topt;
  __device__ State begin() const { return 0; }
  __device__ void load(long long base, long long n, PairItem (&v)[kCompactRows]) const {
    int a[kCompactRows], j[kCompactRows];
    tile_pairs(base, N, a, j);
#pragma unroll
    for (int r = 0; r < kCompactRows; ++r) {
      const long long i = base + r * kCompactThreads + threadIdx.x;
      v[r].a = a[r];
      v[r].j = j[r];
      v[r].c = i < n ? src.at(i, a[r], j[r]) : 0.0f;
    }
  }
  __device__ bool sel(State, const PairItem &v) const { return v.c < rn; }
  __device__ void emit(long long i, const PairItem &v, long long pos) const {
    if (pos >= cap) return;
    e_src[pos] = v.a;
    e_dst[pos] = v.j;
    e_copt[pos] = v.c;
    e_topt[pos] = tsrc.at(i, v.a, v.j);
  }
};

// rn's bits, whether the superset held rank k within its buffer, the edge
// count and the compaction's wait-bound error word, for one read-back (the
// tail of the one-read pass that runs as separate launches).
__global__ void rn_pack_kernel(const float *rn, const unsigned long long *n_sup,
                               const unsigned long long *edges, long long k, long long cap,
                               const int *err, RnEdgesPack *out) {
  const unsigned long long ns = *n_sup;
  out->rn_bits = *reinterpret_cast<const unsigned int *>(rn);
  out->ok = (long long)ns > k && (long long)ns <= cap;
  out->edges = *edges;
  out->error = *err != 0;
  out->pad = 0;
}

// Edges from the superset (one-pass compaction): entries with cost < rn, in
// superset (= pair) order; rn is read on the device (the select's result).
struct SupBelowRn {
  const float *sc;
  const float *rn;
  __device__ bool operator()(long long q) const { return __ldg(&sc[q]) < *rn; }
};
template <class TSup>
struct SupEdgeEmit {
  const uint32_t *idx;
  const float *sc;
  TSup tsup;
  int N;
  long long cap;
  int *e_src, *e_dst;
  float *e_copt, *e_topt;
  __device__ void operator()(long long q, long long pos) const {
    if (pos >= cap) return;
    const uint32_t id = __ldg(&idx[q]);
    const uint32_t a = id / (uint32_t)(N - 1), b = id - a * (uint32_t)(N - 1);
    const int j = (int)b + (b >= a ? 1 : 0);
    e_src[pos] = (int)a;
    e_dst[pos] = j;
    e_copt[pos] = __ldg(&sc[q]);
    e_topt[pos] = tsup.at(q, id, (int)a, j);
  }
};

// The optimal time of superset entry q (pair number id, pair (a, j)) for
// the edge list, from the pair arrays.
template <class Topt>
struct SupToptPairs {
  Topt tsrc;
  __device__ float at(long long, uint32_t id, int a, int j) const {
    return tsrc.at((long long)id, a, j);
  }
};

// Device-side k-th smallest of src(0 .. n-1), or of src(0 .. *d_n - 1) when
// d_n (device) is given and below n: the result lands in the ctx select
// state; *d_result points at it (device).
template <class Src>
pump_status_t select_kth_src(Ctx *ctx, Src src, long long n, long long k, const float **d_result,
                             cudaStream_t stream, const unsigned long long *d_n = nullptr,
                             long long max_blocks = kNumSMs * 4) {
  if (n <= 0 || k < 0 || k >= n) return set_error(PUMP_ERR_BAD_INPUT, "select_kth: k=%lld n=%lld", k, n);
  char *scratch = nullptr;
  const size_t bytes = sizeof(SelectState) + 2049 * sizeof(unsigned int);
  PUMP_TRY(ctx->scratch(Ctx::kSelect, bytes, (void **)&scratch));
  SelectState *st = (SelectState *)scratch;
  unsigned int *hist = (unsigned int *)(scratch + sizeof(SelectState));
  unsigned int *done = hist + 2048;
  select_init_kernel<<<1, 1024, 0, stream>>>(st, (unsigned long long)k, hist, done);
  PUMP_TRY(launch_status("select_init_kernel"));
  long long blocks = (n + (long long)kSelectThreads * kSelectBatch - 1) /
                     ((long long)kSelectThreads * kSelectBatch);
  if (blocks > max_blocks) blocks = max_blocks;
  const int shifts[3] = {21, 10, 0}, bits[3] = {11, 11, 10};
  for (int pass = 0; pass < 3; ++pass) {
    select_hist_kernel<<<(unsigned)blocks, kSelectThreads, 0, stream>>>(src, n, d_n, st, shifts[pass],
                                                              bits[pass], hist, done);
    PUMP_TRY(launch_status("select_hist_kernel"));
  }
  *d_result = reinterpret_cast<const float *>(&st->result);
  return PUMP_OK;
}

}  // namespace

pump_status_t select_kth_device(Ctx *ctx, const float *d_v, long long n, long long k,
                                const float **d_result, cudaStream_t stream) {
  return select_kth_src(ctx, FlatSrc{d_v}, n, k, d_result, stream);
}

pump_status_t select_kth_pairs(Ctx *ctx, const PairView &pv, long long k, const float **d_result,
                               cudaStream_t stream) {
  return select_kth_src(ctx, PairCoptSrc{pv}, (long long)pv.N * (pv.N - 1), k, d_result, stream);
}

namespace {
// The edges below rn with their row starts, from any pair-cost source.
template <class Src, class Topt>
pump_status_t edges_src(Ctx *ctx, Src src, Topt tsrc, int N, float rn, long long max_edges,
                        int *d_src, int *d_dst, float *d_copt, float *d_topt, int *d_go_start,
                        long long *h_num_edges, cudaStream_t stream) {
  const long long npairs = (long long)N * (N - 1);
  TileScratch ts{};
  PUMP_TRY(run_chunked_tuned(ctx, kTuneCompactEdges, npairs,
                             EdgeLoader<Src, Topt>{src, tsrc, N, rn, max_edges, d_src, d_dst,
                                                   d_copt, d_topt},
                             stream, &ts));
  unsigned long long total = 0;
  PUMP_TRY(finish_compact(ts, &total, stream));
  *h_num_edges = (long long)total;
  if ((long long)total > max_edges)
    return set_error(PUMP_ERR_CAPACITY, "build_edges: %llu edges exceed capacity %lld", total, max_edges);
  if (d_go_start) PUMP_TRY(row_starts(d_src, (long long)total, N, d_go_start, stream));
  return PUMP_OK;
}
}  // namespace

pump_status_t build_edges_device(Ctx *ctx, const float *d_copts, const float *d_topts, int N, float rn,
                                 long long max_edges, int *d_src, int *d_dst, float *d_copt,
                                 float *d_topt, int *d_go_start, long long *h_num_edges,
                                 cudaStream_t stream) {
  return edges_src(ctx, FlatSrc{d_copts}, FlatTopt{d_topts}, N, rn, max_edges, d_src, d_dst,
                   d_copt, d_topt, d_go_start, h_num_edges, stream);
}

// Edges of one query of a batch from its pair view (same order and values as
// build_edges_device on the query's own pair arrays).
pump_status_t build_edges_pairs(Ctx *ctx, const PairView &pv, float rn, long long max_edges,
                                int *d_src, int *d_dst, float *d_copt, float *d_topt,
                                int *d_go_start, long long *h_num_edges, cudaStream_t stream) {
  return edges_src(ctx, PairCoptSrc{pv}, PairTopt{pv}, pv.N, rn, max_edges, d_src, d_dst, d_copt,
                   d_topt, d_go_start, h_num_edges, stream);
}

namespace {
// The one-read pass's shape for k of n pairs: the bracket sample's rank and
// the superset buffer's capacity; false when the pass does not apply (few
// pairs, 2^32 pairs or more, or a rank the sample cannot bracket).
struct RnPlan {
  long long rank, cap;
};
bool rn_plan(long long n, long long k, RnPlan *pl) {
  const int S = kBracketSamples;
  const double p = (double)(k + 1) / (double)n;
  pl->rank = (long long)std::ceil(p * S + 8.0 * std::sqrt(S * p * (1.0 - p))) + 16;
  if (n < 64LL * S || n >= (1LL << 32) || pl->rank >= S) return false;
  pl->cap = std::min(n, 2 * (pl->rank + 1) * (n / S + 1) + 65536);
  return k < pl->cap;
}

// Scratch of the one-read pass.  A zeroed head (per call): the bracket key,
// the read-back pack, the superset's size, the bracket's block counter, the
// finishing kernel's barrier words and error word, then its three select
// histograms; after it the finishing kernel's
// per-block partial sums, the bracket sample's keys and the superset (pair
// numbers, costs).
constexpr int kMaxFinishBlocks = 1024;
struct RnScratch {
  unsigned long long *key_hi;
  RnEdgesPack *pack;
  unsigned long long *n_sup;
  unsigned int *done, *bar;
  int *error;
  unsigned int *hist;
  unsigned long long *partial;
  uint32_t *sample_keys;
  uint32_t *sup_idx;
  float *sup_c;
};
pump_status_t rn_scratch(Ctx *ctx, long long cap, cudaStream_t stream, RnScratch *rs) {
  char *buf = nullptr;
  constexpr size_t kWords = 128;
  constexpr size_t kZeroed = kWords + 3 * 2048 * sizeof(unsigned int);
  const size_t head = kZeroed + 2 * kMaxFinishBlocks * sizeof(unsigned long long) +
                      sizeof(uint32_t) * kBracketSamples;
  PUMP_TRY(ctx->scratch(Ctx::kSuperset, head + (size_t)cap * 8, (void **)&buf));
  static_assert(sizeof(RnEdgesPack) <= 32, "pack fits its slot");
  rs->key_hi = (unsigned long long *)buf;
  rs->pack = (RnEdgesPack *)(buf + 16);
  rs->n_sup = (unsigned long long *)(buf + 48);
  rs->done = (unsigned int *)(buf + 56);
  rs->bar = (unsigned int *)(buf + 64);
  rs->error = (int *)(buf + 72);
  rs->hist = (unsigned int *)(buf + kWords);
  rs->partial = (unsigned long long *)(buf + kZeroed);
  rs->sample_keys = (uint32_t *)(rs->partial + 2 * kMaxFinishBlocks);
  rs->sup_idx = (uint32_t *)(buf + head);
  rs->sup_c = (float *)(rs->sup_idx + cap);
  PUMP_CUDA_TRY(cudaMemsetAsync(buf, 0, kZeroed, stream));
  return PUMP_OK;
}

// One block per SM for the finishing kernel (cooperative launch).
template <class TSup>
pump_status_t rn_finish_launch(const RnFinish<TSup> &a, cudaStream_t stream) {
  int dev = 0, sms = 0, coop = 0, occ = 0;
  PUMP_CUDA_TRY(cudaGetDevice(&dev));
  PUMP_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  PUMP_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  PUMP_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rn_finish_kernel<TSup>,
                                                              kFinishThreads, 0));
  if (!coop || occ < 1)
    return set_error(PUMP_ERR_CUDA, "rn_finish: cooperative launch unavailable");
  const int grid = std::min(sms, kMaxFinishBlocks);
  void *args[] = {(void *)&a};
  PUMP_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)rn_finish_kernel<TSup>, grid,
                                            kFinishThreads, args, 0, stream));
  return PUMP_OK;
}

// After the pair pass (the superset as per-warp masks over the pair costs
// d_copts, or contiguous in rs.sup_idx / rs.sup_c with its size in *n_in):
// the finishing kernel (select over the
// superset for rank k, the edges below rn, the row starts, the pack).
// Then either the deferred pack pointer, or one read-back: rn and the edge
// count, PUMP_ERR_TIMEOUT when a wait gave up, or the fallback when the
// superset missed rank k or overflowed.  err_pass: an earlier pass's
// wait-bound error word (or null).
template <class TSup, class Fallback>
pump_status_t rn_edges_tail(const RnScratch &rs, const PairStage *stage, const float *d_copts,
                            const unsigned long long *n_in, TSup tsup,
                            const int *err_pass, int N,
                            long long k, long long cap, long long max_edges, int *d_src,
                            int *d_dst, float *d_copt, float *d_topt, int *d_go_start,
                            float *h_rn, long long *h_num_edges, cudaStream_t stream,
                            Fallback fallback, const RnEdgesPack **deferred) {
  RnFinish<TSup> a{};
  if (stage) {
    a.masks = stage->masks;
    a.nmasks = stage->nmasks;
    a.masks_per_row = stage->masks_per_row;
    a.copts = d_copts;
  }
  a.n_in = n_in;
  a.sup_idx = rs.sup_idx;
  a.sup_c = rs.sup_c;
  a.tsup = tsup;
  a.cap = cap;
  a.k = k;
  a.max_edges = max_edges;
  a.N = N;
  a.e_src = d_src;
  a.e_dst = d_dst;
  a.e_copt = d_copt;
  a.e_topt = d_topt;
  a.go_start = d_go_start;
  a.hist = rs.hist;
  a.partial = rs.partial;
  a.bar = rs.bar;
  a.n_sup = rs.n_sup;
  a.err_in = err_pass;
  a.error = rs.error;
  a.pack = rs.pack;
  a.spin_limit = kBarrierSpin;
  PUMP_TRY(rn_finish_launch(a, stream));
  if (deferred) {
    *deferred = rs.pack;
    *h_num_edges = -1;
    return PUMP_OK;
  }
  RnEdgesPack pk{};
  PUMP_CUDA_TRY(cudaMemcpyAsync(&pk, rs.pack, sizeof pk, cudaMemcpyDeviceToHost, stream));
  PUMP_CUDA_TRY(cudaStreamSynchronize(stream));
  return rn_edges_unpack(pk, k, max_edges, h_rn, h_num_edges, fallback);
}

// The same after a contiguous superset, as separate launches that each
// take part of the GPU: the radix select, the one-pass edge compaction, the
// row starts and the pack.  Queries planned concurrently (batch workers) use
// this form: the finishing kernel's cooperative launch takes every SM's
// register file at once, so it would wait for the other workers' kernels to
// drain.
template <class TSup, class Fallback>
pump_status_t rn_edges_tail_streamed(Ctx *ctx, const RnScratch &rs, TSup tsup, int N, long long k,
                                     long long cap, long long max_edges, int *d_src, int *d_dst,
                                     float *d_copt, float *d_topt, int *d_go_start, float *h_rn,
                                     long long *h_num_edges, cudaStream_t stream,
                                     Fallback fallback, const RnEdgesPack **deferred) {
  const float *d_rn = nullptr;
  PUMP_TRY(select_kth_src(ctx, FlatSrc{rs.sup_c}, cap, k, &d_rn, stream, rs.n_sup));
  TileScratch ts2{};
  PUMP_TRY(run_compact(ctx, cap, SupBelowRn{rs.sup_c, d_rn},
                       SupEdgeEmit<TSup>{rs.sup_idx, rs.sup_c, tsup, N, max_edges, d_src, d_dst,
                                         d_copt, d_topt},
                       stream, &ts2, rs.n_sup));
  if (d_go_start) PUMP_TRY(row_starts(d_src, max_edges, N, d_go_start, stream, ts2.total));
  rn_pack_kernel<<<1, 1, 0, stream>>>(d_rn, rs.n_sup, ts2.total, k, cap, ts2.error, rs.pack);
  PUMP_TRY(launch_status("rn_pack_kernel"));
  if (deferred) {
    *deferred = rs.pack;
    *h_num_edges = -1;
    return PUMP_OK;
  }
  RnEdgesPack pk{};
  PUMP_CUDA_TRY(cudaMemcpyAsync(&pk, rs.pack, sizeof pk, cudaMemcpyDeviceToHost, stream));
  PUMP_CUDA_TRY(cudaStreamSynchronize(stream));
  return rn_edges_unpack(pk, k, max_edges, h_rn, h_num_edges, fallback);
}

// rn = the k-th smallest pair cost and the edges below it (same values and
// order as select_kth + build_edges) from one read of the pair costs: the
// bracket sample, the superset pass, then rn_edges_tail (cooperative) or
// rn_edges_tail_streamed.  `fallback` runs the three-pass select and the
// full compaction when the pass does not apply or (after the read-back) the
// superset missed rank k or overflowed.
template <class Src, class Topt, class Fallback>
pump_status_t rn_edges_src(Ctx *ctx, Src src, Topt tsrc, int N, long long k, long long max_edges,
                           int *d_src, int *d_dst, float *d_copt, float *d_topt, int *d_go_start,
                           float *h_rn, long long *h_num_edges, cudaStream_t stream,
                           Fallback fallback, const RnEdgesPack **deferred, bool cooperative) {
  if (deferred) *deferred = nullptr;
  const long long n = (long long)N * (N - 1);
  if (k < 0 || k >= n) return set_error(PUMP_ERR_BAD_INPUT, "rn_edges: k=%lld n=%lld", k, n);
  RnPlan pl;
  if (!rn_plan(n, k, &pl)) return fallback();
  RnScratch rs;
  PUMP_TRY(rn_scratch(ctx, pl.cap, stream, &rs));
  bracket_kernel<<<1, 1024, 0, stream>>>(src, n, (unsigned int)pl.rank, rs.key_hi);
  PUMP_TRY(launch_status("bracket_kernel"));
  TileScratch ts{};
  PUMP_TRY(run_chunked_tuned(ctx, kTuneCompactRn, n,
                             SupersetLoader<Src>{src, N, rs.key_hi, pl.cap, rs.sup_idx,
                                                 (uint32_t *)rs.sup_c},
                             stream, &ts, nullptr, rs.n_sup));
  if (!cooperative)
    return rn_edges_tail_streamed(ctx, rs, SupToptPairs<Topt>{tsrc}, N, k, pl.cap, max_edges, d_src,
                                  d_dst, d_copt, d_topt, d_go_start, h_rn, h_num_edges, stream,
                                  fallback, deferred);
  return rn_edges_tail(rs, nullptr, nullptr, rs.n_sup, SupToptPairs<Topt>{tsrc}, nullptr,
                       N, k, pl.cap,
                       max_edges, d_src, d_dst, d_copt, d_topt, d_go_start, h_rn, h_num_edges,
                       stream, fallback, deferred);
}

}  // namespace

pump_status_t rn_edges_unpack(const RnEdgesPack &pk, long long k, long long max_edges, float *h_rn,
                              long long *h_num_edges, const std::function<pump_status_t()> &fallback) {
  (void)k;
  if (pk.error)
    return set_error(PUMP_ERR_TIMEOUT, "rn and edges: a look-back wait exceeded its bound");
  if (!pk.ok) return fallback();
  std::memcpy(h_rn, &pk.rn_bits, sizeof(float));
  *h_num_edges = (long long)pk.edges;
  if ((long long)pk.edges > max_edges)
    return set_error(PUMP_ERR_CAPACITY, "build_edges: %llu edges exceed capacity %lld", pk.edges,
                     max_edges);
  return PUMP_OK;
}

pump_status_t rn_edges_fallback_device(Ctx *ctx, const float *d_copts, const float *d_topts, int N,
                                       long long k, long long max_edges, int *d_src, int *d_dst,
                                       float *d_copt, float *d_topt, int *d_go_start, float *h_rn,
                                       long long *h_num_edges, cudaStream_t stream) {
  const float *d_rn = nullptr;
  PUMP_TRY(select_kth_device(ctx, d_copts, (long long)N * (N - 1), k, &d_rn, stream));
  PUMP_CUDA_TRY(cudaMemcpyAsync(h_rn, d_rn, sizeof(float), cudaMemcpyDeviceToHost, stream));
  PUMP_CUDA_TRY(cudaStreamSynchronize(stream));
  return build_edges_device(ctx, d_copts, d_topts, N, *h_rn, max_edges, d_src, d_dst, d_copt,
                            d_topt, d_go_start, h_num_edges, stream);
}

pump_status_t rn_edges_fallback_pairs(Ctx *ctx, const PairView &pv, long long k,
                                      long long max_edges, int *d_src, int *d_dst, float *d_copt,
                                      float *d_topt, int *d_go_start, float *h_rn,
                                      long long *h_num_edges, cudaStream_t stream) {
  const float *d_rn = nullptr;
  PUMP_TRY(select_kth_pairs(ctx, pv, k, &d_rn, stream));
  PUMP_CUDA_TRY(cudaMemcpyAsync(h_rn, d_rn, sizeof(float), cudaMemcpyDeviceToHost, stream));
  PUMP_CUDA_TRY(cudaStreamSynchronize(stream));
  return build_edges_pairs(ctx, pv, *h_rn, max_edges, d_src, d_dst, d_copt, d_topt, d_go_start,
                           h_num_edges, stream);
}

pump_status_t rn_edges_device(Ctx *ctx, const float *d_copts, const float *d_topts, int N,
                              long long k, long long max_edges, int *d_src, int *d_dst,
                              float *d_copt, float *d_topt, int *d_go_start, float *h_rn,
                              long long *h_num_edges, cudaStream_t stream,
                              const RnEdgesPack **deferred, bool cooperative) {
  auto fallback = [&]() -> pump_status_t {
    if (deferred) *deferred = nullptr;
    return rn_edges_fallback_device(ctx, d_copts, d_topts, N, k, max_edges, d_src, d_dst, d_copt,
                                    d_topt, d_go_start, h_rn, h_num_edges, stream);
  };
  return rn_edges_src(ctx, FlatSrc{d_copts}, FlatTopt{d_topts}, N, k, max_edges, d_src, d_dst,
                      d_copt, d_topt, d_go_start, h_rn, h_num_edges, stream, fallback, deferred,
                      cooperative);
}

pump_status_t rn_edges_pairs(Ctx *ctx, const PairView &pv, long long k, long long max_edges,
                             int *d_src, int *d_dst, float *d_copt, float *d_topt,
                             int *d_go_start, float *h_rn, long long *h_num_edges,
                             cudaStream_t stream, const RnEdgesPack **deferred) {
  auto fallback = [&]() -> pump_status_t {
    if (deferred) *deferred = nullptr;
    return rn_edges_fallback_pairs(ctx, pv, k, max_edges, d_src, d_dst, d_copt, d_topt,
                                   d_go_start, h_rn, h_num_edges, stream);
  };
  return rn_edges_src(ctx, PairCoptSrc{pv}, PairTopt{pv}, pv.N, k, max_edges, d_src, d_dst, d_copt,
                      d_topt, d_go_start, h_rn, h_num_edges, stream, fallback, deferred, false);
}

pump_status_t roadmap_pairs_edges(Ctx *ctx, const float *d_samples, int N, float tmax,
                                  int bvp_mode, long long k, long long max_edges, float *d_copts,
                                  float *d_topts, int *d_src, int *d_dst, float *d_copt,
                                  float *d_topt, int *d_go_start, float *h_rn,
                                  long long *h_num_edges, cudaStream_t stream,
                                  const RnEdgesPack **deferred, float *stage_ms,
                                  bool cooperative) {
  if (deferred) *deferred = nullptr;
  if (N < 2) return set_error(PUMP_ERR_BAD_INPUT, "roadmap: N = %d", N);
  const long long n = (long long)N * (N - 1);
  if (k < 0 || k >= n) return set_error(PUMP_ERR_BAD_INPUT, "roadmap: k=%lld n=%lld", k, n);
  // stage events: start, pair kernel start, pair kernel end, end
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  struct EvGuard {
    cudaEvent_t *e;
    ~EvGuard() {
      for (int q = 0; q < 4; ++q)
        if (e[q]) cudaEventDestroy(e[q]);
    }
  } guard{ev};
  if (stage_ms && !deferred) {
    for (int q = 0; q < 4; ++q) PUMP_CUDA_TRY(cudaEventCreate(&ev[q]));
    PUMP_CUDA_TRY(cudaEventRecord(ev[0], stream));
  }
  auto finish = [&](pump_status_t st) -> pump_status_t {
    if (st != PUMP_OK || !ev[0]) return st;
    PUMP_CUDA_TRY(cudaEventRecord(ev[3], stream));
    PUMP_CUDA_TRY(cudaEventSynchronize(ev[3]));
    for (int q = 0; q < 3; ++q)
      PUMP_CUDA_TRY(cudaEventElapsedTime(&stage_ms[q], ev[q], ev[q + 1]));
    return st;
  };
  RnPlan pl;
  if (bvp_mode != PUMP_BVP_PRECISION || !rn_plan(n, k, &pl) || N > 65535 || !cooperative) {
    if (ev[1]) PUMP_CUDA_TRY(cudaEventRecord(ev[1], stream));
    PUMP_TRY(pump_bvp_pairs(d_samples, N, tmax, bvp_mode, d_copts, d_topts, (pump_stream_t)stream));
    if (ev[2]) PUMP_CUDA_TRY(cudaEventRecord(ev[2], stream));
    return finish(rn_edges_device(ctx, d_copts, d_topts, N, k, max_edges, d_src, d_dst, d_copt,
                                  d_topt, d_go_start, h_rn, h_num_edges, stream, deferred,
                                  cooperative));
  }
  RnScratch rs;
  PUMP_TRY(rn_scratch(ctx, pl.cap, stream, &rs));
  PairStage stage{};
  PairSuperset ps{};
  ps.rank = (unsigned int)pl.rank;
  ps.key_hi = rs.key_hi;
  ps.sample_keys = rs.sample_keys;
  ps.done = rs.done;
  ps.after_pairs = ev[2];
  ps.out = &stage;
  // the samples and bracket launch comes first; the pair kernel's own time
  // is ev[1]..ev[2]
  PUMP_TRY(bvp_pairs_precision_superset(ctx, d_samples, N, tmax, d_copts, d_topts, ps, stream,
                                        ev[1]));
  auto fallback = [&]() -> pump_status_t {
    if (deferred) *deferred = nullptr;
    return rn_edges_fallback_device(ctx, d_copts, d_topts, N, k, max_edges, d_src, d_dst, d_copt,
                                    d_topt, d_go_start, h_rn, h_num_edges, stream);
  };
  return finish(rn_edges_tail(rs, &stage, d_copts, nullptr, SupToptPairs<FlatTopt>{FlatTopt{d_topts}},
                              nullptr, N, k, pl.cap,
                              max_edges, d_src, d_dst, d_copt, d_topt, d_go_start, h_rn,
                              h_num_edges, stream, fallback, deferred));
}

pump_status_t frontier_compact_device(Ctx *ctx, const uint8_t *d_flags, int N, int *d_active,
                                      int *d_count, int **d_error_out, cudaStream_t stream) {
  TileScratch ts{};
  PUMP_TRY(run_compact(ctx, N, FlagPred{d_flags}, IndexEmit{d_active}, stream, &ts));
  copy_count_kernel<<<1, 1, 0, stream>>>(ts.total, d_count);
  if (d_error_out) *d_error_out = ts.error;
  return launch_status("copy_count_kernel");
}

}  // namespace pump

using namespace pump;

extern "C" pump_status_t pump_select_kth(pump_ctx *ctx, const float *d_v, long long n, long long k,
                                         float *h_kth, pump_stream_t stream) {
  if (!ctx || !d_v || !h_kth) return set_error(PUMP_ERR_BAD_INPUT, "pump_select_kth: null argument");
  Ctx *c = Ctx::from(ctx);
  PUMP_TRY(c->activate());
  const float *d_res = nullptr;
  PUMP_TRY(select_kth_device(c, d_v, n, k, &d_res, (cudaStream_t)stream));
  PUMP_CUDA_TRY(cudaMemcpyAsync(h_kth, d_res, sizeof(float), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  PUMP_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return PUMP_OK;
}

extern "C" pump_status_t pump_build_edges(pump_ctx *ctx, const float *d_copts, const float *d_topts,
                                          int N, float rn, long long max_edges, int *d_src,
                                          int *d_dst, float *d_copt, float *d_topt, int *d_go_start,
                                          long long *h_num_edges, pump_stream_t stream) {
  if (!ctx || N < 2 || !d_copts || !d_topts || !d_src || !d_dst || !d_copt || !d_topt ||
      !h_num_edges || max_edges < 0)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_build_edges: bad arguments");
  Ctx *c = Ctx::from(ctx);
  PUMP_TRY(c->activate());
  return build_edges_device(c, d_copts, d_topts, N, rn, max_edges, d_src, d_dst, d_copt, d_topt,
                            d_go_start, h_num_edges, (cudaStream_t)stream);
}

extern "C" pump_status_t pump_frontier_compact(pump_ctx *ctx, const uint8_t *d_flags, int N,
                                               int *d_active, int *d_count, pump_stream_t stream) {
  if (!ctx || N < 0 || (N > 0 && (!d_flags || !d_active)) || !d_count)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_frontier_compact: bad arguments");
  Ctx *c = Ctx::from(ctx);
  PUMP_TRY(c->activate());
  int *d_err = nullptr;
  PUMP_TRY(frontier_compact_device(c, d_flags, N, d_active, d_count, &d_err, (cudaStream_t)stream));
  int err = 0;
  PUMP_CUDA_TRY(cudaMemcpyAsync(&err, d_err, sizeof err, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  PUMP_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  if (err) return set_error(PUMP_ERR_TIMEOUT, "pump_frontier_compact: look-back wait exceeded its bound");
  return PUMP_OK;
}

// ---------------------------------------------------------------------------
// Bounded-wait self-test: tile 1 of a look-back whose tile 0 never publishes
// (its status word is zeroed and nothing writes it), so the wait can end only
// through its bound.  One warp; words[0..1] are the two status words,
// words[2] receives 1 when the wait gave up.
namespace pump {
namespace {
__global__ void selftest_wait_kernel(unsigned long long *words, long long spin_limit) {
  TileScratch ts{};
  ts.status = words;
  bool timed_out = false;
  lookback_warp(ts, 1, 1, &timed_out, spin_limit);
  if ((threadIdx.x & 31) == 0) words[2] = timed_out ? 1ull : 0ull;
}
}  // namespace
}  // namespace pump

extern "C" pump_status_t pump_selftest_wait(pump_ctx *ctx, long long spin_limit, pump_stream_t stream) {
  if (!ctx || spin_limit < 0 || spin_limit > kSpinLimit)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_selftest_wait: bad arguments");
  Ctx *c = Ctx::from(ctx);
  PUMP_TRY(c->activate());
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long *words = nullptr;
  PUMP_TRY(c->scratch(Ctx::kCompact, 3 * sizeof(unsigned long long), (void **)&words));
  PUMP_CUDA_TRY(cudaMemsetAsync(words, 0, 3 * sizeof(unsigned long long), s));
  selftest_wait_kernel<<<1, 32, 0, s>>>(words, spin_limit);
  PUMP_TRY(launch_status("selftest_wait_kernel"));
  unsigned long long gave_up = 0;
  PUMP_CUDA_TRY(cudaMemcpyAsync(&gave_up, words + 2, sizeof gave_up, cudaMemcpyDeviceToHost, s));
  PUMP_CUDA_TRY(cudaStreamSynchronize(s));
  if (gave_up) return set_error(PUMP_ERR_TIMEOUT, "pump_selftest_wait: the wait gave up after %lld polls", spin_limit);
  return PUMP_OK;
}

// ---------------------------------------------------------------------------
// Frontier compaction without any allocation.
//
// For callers that must not allocate device memory while they plan: a
// real-time control loop that reserves all of its memory at start-up so that
// no planning step can block in (or fail inside) the allocator, or a host
// framework that owns the device memory budget through its own pool and does
// not let plugins call cudaMalloc.  pump_frontier_compact takes its look-back
// scratch from the context's grow-only buffers, which may call cudaMalloc on
// first use or when N grows; this variant keeps that scratch in one
// fixed-size array in device memory instead.
//
// The array is a file-scope __device__ variable: every GPU that loads the
// library holds its 64 KiB until the process exits, and every call on that
// GPU uses the same array.  Host code cannot use the variable's name as a
// device address, so the address is looked up with cudaGetSymbolAddress
// (with the device current) on the first call made in each CUDA context on
// it -- once per device for the usual primary context, again after a device
// reset or in another context; make that first call before any stream
// capture.  Each call clears the
// words that must start at zero before its kernel runs; two calls that
// overlap on the GPU (for example on two streams) share the array and race,
// so serialise them.
namespace pump {
namespace {

constexpr long long kNoAllocMaxTiles = 8192;                   // 8192 tiles of 4096 flags
constexpr long long kNoAllocMaxFlags = kNoAllocMaxTiles * kTile;  // 33,554,432
// word 0: selected count; words 1 .. 8192: tile status; word 8193: unused;
// word 8194: tile counter (4 B) and error word (4 B)
constexpr int kNoAllocWords = 1 + (int)kNoAllocMaxTiles + 1 + 1;

static __device__ __align__(256) unsigned long long g_frontier_scratch[kNoAllocWords];

// The array's address belongs to the CUDA context that loaded the library's
// module, so it is cached per context: keyed by the context's unique id
// (cuCtxGetId), which a device reset or a different (non-primary) context on
// the same device changes, so a stale address is never reused.  The driver
// functions are reached through the runtime's entry-point query, so the
// library needs no link against libcuda.
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);

std::mutex g_scratch_mutex;
struct ScratchAddr {
  unsigned long long ctx_id;
  unsigned long long *addr;
};
std::vector<ScratchAddr> g_scratch_addr;

// *id = the current context's id, or 0 when no context is current yet.
pump_status_t current_context_id(unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    PUMP_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1));
    PUMP_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2));
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return set_error(PUMP_ERR_CUDA, "driver entry points cuCtxGetCurrent/cuCtxGetId unavailable");
    get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  void *ctx = nullptr;
  *id = 0;
  if (get_current(&ctx) != 0) return set_error(PUMP_ERR_CUDA, "cuCtxGetCurrent failed");
  if (ctx && get_id(ctx, id) != 0) return set_error(PUMP_ERR_CUDA, "cuCtxGetId failed");
  return PUMP_OK;
}

pump_status_t frontier_scratch_address(unsigned long long **out) {
  unsigned long long id = 0;
  PUMP_TRY(current_context_id(&id));
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  for (const ScratchAddr &a : g_scratch_addr)
    if (id != 0 && a.ctx_id == id) {
      *out = a.addr;
      return PUMP_OK;
    }
  // set-up for this context: the lookup also makes the device's primary
  // context current when no context was
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_frontier_scratch);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_frontier_scratch)");
  if (id == 0) PUMP_TRY(current_context_id(&id));
  if (id == 0) return set_error(PUMP_ERR_CUDA, "no current CUDA context after the symbol lookup");
  g_scratch_addr.push_back({id, static_cast<unsigned long long *>(p)});
  *out = static_cast<unsigned long long *>(p);
  return PUMP_OK;
}

}  // namespace
}  // namespace pump

extern "C" pump_status_t pump_frontier_compact_noalloc(const uint8_t *d_flags, int N, int *d_active,
                                                       int *d_count, pump_stream_t stream) {
  if (N < 0 || (N > 0 && (!d_flags || !d_active)) || !d_count)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_frontier_compact_noalloc: bad arguments");
  if ((long long)N > kNoAllocMaxFlags)
    return set_error(PUMP_ERR_CAPACITY,
                     "pump_frontier_compact_noalloc: N=%d exceeds the %lld flags its fixed "
                     "scratch array covers; use pump_frontier_compact",
                     N, kNoAllocMaxFlags);
  cudaStream_t s = (cudaStream_t)stream;
  unsigned long long *scratch = nullptr;
  PUMP_TRY(frontier_scratch_address(&scratch));
  const long long ntiles = N > 0 ? ((long long)N + kTile - 1) / kTile : 1;
  TileScratch ts{};
  ts.total = scratch;
  ts.status = scratch + 1;
  ts.tile_counter = reinterpret_cast<unsigned int *>(scratch + 2 + kNoAllocMaxTiles);
  ts.error = reinterpret_cast<int *>(ts.tile_counter + 1);
  // everything the look-back reads before writing starts at zero
  PUMP_CUDA_TRY(cudaMemsetAsync(ts.total, 0, sizeof(unsigned long long) * (ntiles + 2), s));
  PUMP_CUDA_TRY(cudaMemsetAsync(ts.tile_counter, 0, 2 * sizeof(unsigned int), s));
  if (N > 0) {
    compact_kernel<<<(unsigned)ntiles, kCompactThreads, 0, s>>>((long long)N, FlagPred{d_flags},
                                                                IndexEmit{d_active}, ts, nullptr);
    PUMP_TRY(launch_status("compact_kernel (no-alloc)"));
  }
  copy_count_kernel<<<1, 1, 0, s>>>(ts.total, d_count);
  PUMP_TRY(launch_status("copy_count_kernel (no-alloc)"));
  int err = 0;
  PUMP_CUDA_TRY(cudaMemcpyAsync(&err, ts.error, sizeof err, cudaMemcpyDeviceToHost, s));
  PUMP_CUDA_TRY(cudaStreamSynchronize(s));
  if (err)
    return set_error(PUMP_ERR_TIMEOUT, "pump_frontier_compact_noalloc: look-back wait exceeded its bound");
  return PUMP_OK;
}

extern "C" pump_status_t pump_roadmap(pump_ctx *ctx, const float *d_samples, int N, float tmax,
                                      int bvp_mode, long long k, long long max_edges,
                                      float *d_copts, float *d_topts, int *d_src, int *d_dst,
                                      float *d_copt, float *d_topt, int *d_go_start, float *h_rn,
                                      long long *h_num_edges, float *h_stage_ms,
                                      pump_stream_t stream) {
  if (!ctx || !d_samples || N < 2 || max_edges < 0 || !d_copts || !d_topts || !d_src || !d_dst ||
      !d_copt || !d_topt || !h_rn || !h_num_edges)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_roadmap: bad arguments");
  if (bvp_mode != PUMP_BVP_PARITY && bvp_mode != PUMP_BVP_PRECISION &&
      bvp_mode != PUMP_BVP_PARITY_GPU)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_roadmap: bvp_mode %d", bvp_mode);
  Ctx *c = Ctx::from(ctx);
  PUMP_TRY(c->activate());
  return roadmap_pairs_edges(c, d_samples, N, tmax, bvp_mode, k, max_edges, d_copts, d_topts, d_src,
                             d_dst, d_copt, d_topt, d_go_start, h_rn, h_num_edges,
                             (cudaStream_t)stream, nullptr, h_stage_ms);
}

extern "C" pump_status_t pump_roadmap_edges(pump_ctx *ctx, const float *d_copts, const float *d_topts,
                                            int N, long long k, long long max_edges, int *d_src,
                                            int *d_dst, float *d_copt, float *d_topt,
                                            int *d_go_start, float *h_rn, long long *h_num_edges,
                                            pump_stream_t stream) {
  if (!ctx || !d_copts || !d_topts || N < 2 || max_edges < 0 || !d_src || !d_dst || !d_copt ||
      !d_topt || !h_rn || !h_num_edges)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_roadmap_edges: bad arguments");
  Ctx *c = Ctx::from(ctx);
  PUMP_TRY(c->activate());
  return rn_edges_device(c, d_copts, d_topts, N, k, max_edges, d_src, d_dst, d_copt, d_topt,
                         d_go_start, h_rn, h_num_edges, (cudaStream_t)stream);
}
