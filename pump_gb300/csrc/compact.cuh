// Single-pass stable compaction and exclusive scan with decoupled look-back
// (Merrill & Garland, "Single-pass Parallel Prefix Scan with Decoupled
// Look-back", 2016).  A tile of 4096 items is processed row by row (rows of
// 256 consecutive items), so the rank of every selected item follows index
// order; a tile publishes its count, then its inclusive prefix, in a 64-bit
// status word that later tiles read.  Tiles take their index from an atomic
// counter, so every tile a block waits on has already started.  Every wait is
// bounded: a block that spins past kSpinLimit sets the error word and leaves,
// and the host reports PUMP_ERR_TIMEOUT.
#pragma once
#include <cuda/atomic>

#include "common.cuh"
#include "ctx.h"

namespace pump {
namespace {

constexpr int kCompactThreads = 256;
constexpr int kCompactRows = 16;
constexpr int kTile = kCompactThreads * kCompactRows;  // 4096 items
constexpr unsigned long long kFlagAggregate = 1ull << 62;
constexpr unsigned long long kFlagPrefix = 2ull << 62;
constexpr unsigned long long kValueMask = (1ull << 62) - 1;
constexpr long long kSpinLimit = 1ll << 22;

// ------------------------------------------------------ stable compaction
struct TileScratch {
  unsigned long long *status;  // one word per tile, zeroed before launch
  unsigned int *tile_counter;  // zeroed before launch
  unsigned long long *total;   // selected count (written by the last tile)
  int *error;                  // 1 = look-back wait gave up
};

// Exclusive prefix of this tile from its predecessors' status words, read by
// a whole warp: lane l reads the status of tile p - l, so one round trip to L2
// covers 32 predecessors.  The lanes up to the nearest inclusive prefix must
// all have published (at least an aggregate); otherwise the warp waits and
// reads the window again.  Called by every lane of one warp; every lane
// returns the same value.
__device__ unsigned long long lookback_warp(const TileScratch &ts, long long tile,
                                            unsigned long long agg, bool *timed_out) {
  using ref_t = cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>;
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) ref_t(ts.status[0]).store(kFlagPrefix | agg, cuda::memory_order_release);
    return 0;
  }
  if (lane == 0) ref_t(ts.status[tile]).store(kFlagAggregate | agg, cuda::memory_order_release);
  unsigned long long excl = 0;
  long long p = tile - 1;  // nearest tile of the window
  long long spins = 0;
  while (true) {
    const long long q = p - lane;
    // before tile 0 the prefix is 0 (a published prefix of value 0)
    const unsigned long long st =
        q >= 0 ? ref_t(ts.status[q]).load(cuda::memory_order_acquire) : kFlagPrefix;
    const unsigned long long flag = st & ~kValueMask;
    const unsigned int pref = __ballot_sync(0xffffffffu, flag == kFlagPrefix);
    const unsigned int none = __ballot_sync(0xffffffffu, flag == 0);
    const int stop = pref ? __ffs(pref) - 1 : 31;  // last lane needed in this window
    const unsigned int need = stop == 31 ? 0xffffffffu : ((2u << stop) - 1u);
    if (none & need) {
      if (++spins > kSpinLimit) {
        *timed_out = true;
        return 0;
      }
      __nanosleep(32);
      continue;
    }
    unsigned long long v = lane <= stop ? (st & kValueMask) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    excl += v;
    if (pref) break;
    p -= 32;
  }
  if (lane == 0) ref_t(ts.status[tile]).store(kFlagPrefix | (excl + agg), cuda::memory_order_release);
  return excl;
}

// Pred(i) -> bool, Emit(i, pos) writes item i at output position pos.
template <class Pred, class Emit>
__global__ void __launch_bounds__(kCompactThreads) compact_kernel(long long n, Pred pred, Emit emit,
                                                                  TileScratch ts) {
  __shared__ unsigned int s_tile;
  __shared__ unsigned int s_cnt[kCompactRows][kCompactThreads / 32];
  __shared__ unsigned long long s_excl;
  __shared__ bool s_timeout;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_tile = atomicAdd(ts.tile_counter, 1u);
    s_timeout = false;
  }
  __syncthreads();
  const long long tile = s_tile;
  const long long base = tile * kTile;
  // all predicates first (their loads in flight together), then the ballots
  bool f[kCompactRows];
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    const long long i = base + r * kCompactThreads + threadIdx.x;
    f[r] = i < n && pred(i);
  }
  unsigned int ballots[kCompactRows];
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    ballots[r] = __ballot_sync(0xffffffffu, f[r]);
    if (lane == 0) s_cnt[r][warp] = __popc(ballots[r]);
  }
  __syncthreads();
  // exclusive scan of the 16 x 8 counts in (row, warp) order by warp 0
  if (warp == 0) {
    unsigned int v[4];
    unsigned int run = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = lane * 4 + q;
      v[q] = s_cnt[e / 8][e % 8];
      run += v[q];
    }
    unsigned int incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned int o = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += o;
    }
    unsigned int ex = incl - run;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = lane * 4 + q;
      s_cnt[e / 8][e % 8] = ex;
      ex += v[q];
    }
    const unsigned int agg = __shfl_sync(0xffffffffu, incl, 31);
    bool to = false;
    const unsigned long long ex_tile = lookback_warp(ts, tile, agg, &to);
    if (lane == 0) {
      s_excl = ex_tile;
      if (to) {
        s_timeout = true;
        atomicExch(ts.error, 1);
      }
      const long long ntiles = (n + kTile - 1) / kTile;
      if (!to && tile == ntiles - 1) *ts.total = ex_tile + agg;
    }
  }
  __syncthreads();
  if (s_timeout) return;
  const unsigned long long excl = s_excl;
  const unsigned int lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    if (ballots[r] & (1u << lane)) {
      const long long i = base + r * kCompactThreads + threadIdx.x;
      emit(i, (long long)(excl + s_cnt[r][warp] + __popc(ballots[r] & lt)));
    }
  }
}

template <class Pred, class Emit>
pump_status_t run_compact(Ctx *ctx, long long n, Pred pred, Emit emit, cudaStream_t stream,
                          TileScratch *ts_out) {
  const long long ntiles = n > 0 ? (n + kTile - 1) / kTile : 1;
  const size_t bytes = sizeof(unsigned long long) * (ntiles + 2) + sizeof(unsigned int) * 4;
  char *scratch = nullptr;
  PUMP_TRY(ctx->scratch(Ctx::kCompact, bytes, (void **)&scratch));
  TileScratch ts{};
  ts.total = (unsigned long long *)scratch;
  ts.status = ts.total + 1;
  ts.tile_counter = (unsigned int *)(ts.status + ntiles + 1);
  ts.error = (int *)(ts.tile_counter + 1);
  PUMP_CUDA_TRY(cudaMemsetAsync(scratch, 0, bytes, stream));
  if (n > 0) {
    if (ntiles > 2147483647LL) return set_error(PUMP_ERR_CAPACITY, "compaction: too many tiles");
    compact_kernel<<<(unsigned)ntiles, kCompactThreads, 0, stream>>>(n, pred, emit, ts);
    PUMP_TRY(launch_status("compact_kernel"));
  }
  *ts_out = ts;
  return PUMP_OK;
}

// Reads the selected count and the wait-bound error word (synchronises).
pump_status_t finish_compact(const TileScratch &ts, unsigned long long *total, cudaStream_t stream) {
  int err = 0;
  PUMP_CUDA_TRY(cudaMemcpyAsync(total, ts.total, sizeof *total, cudaMemcpyDeviceToHost, stream));
  PUMP_CUDA_TRY(cudaMemcpyAsync(&err, ts.error, sizeof err, cudaMemcpyDeviceToHost, stream));
  PUMP_CUDA_TRY(cudaStreamSynchronize(stream));
  if (err) return set_error(PUMP_ERR_TIMEOUT, "compaction: look-back wait exceeded its bound");
  return PUMP_OK;
}

// The edge list (mainPUMP.cu:327-346): the pairs with copt < rn in index
// order, written as (i, j, copt, topt).  A specialisation of compact_kernel
// that reads both pair arrays coalesced in the first phase, so the emit
// phase does not wait on a dependent read per selected pair.
__global__ void __launch_bounds__(kCompactThreads) edge_compact_kernel(
    long long n, int N, const float *__restrict__ copts, const float *__restrict__ topts, float rn,
    long long cap, int *__restrict__ src, int *__restrict__ dst, float *__restrict__ copt,
    float *__restrict__ topt, TileScratch ts) {
  __shared__ unsigned int s_tile;
  __shared__ unsigned int s_cnt[kCompactRows][kCompactThreads / 32];
  __shared__ unsigned long long s_excl;
  __shared__ bool s_timeout;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_tile = atomicAdd(ts.tile_counter, 1u);
    s_timeout = false;
  }
  __syncthreads();
  const long long tile = s_tile;
  const long long base = tile * kTile;
  float c[kCompactRows], t[kCompactRows];
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    const long long i = base + r * kCompactThreads + threadIdx.x;
    c[r] = i < n ? __ldg(&copts[i]) : 0.0f;
    t[r] = i < n ? __ldg(&topts[i]) : 0.0f;
  }
  unsigned int ballots[kCompactRows];
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    const long long i = base + r * kCompactThreads + threadIdx.x;
    ballots[r] = __ballot_sync(0xffffffffu, i < n && c[r] < rn);
    if (lane == 0) s_cnt[r][warp] = __popc(ballots[r]);
  }
  __syncthreads();
  if (warp == 0) {
    unsigned int v[4];
    unsigned int run = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = lane * 4 + q;
      v[q] = s_cnt[e / 8][e % 8];
      run += v[q];
    }
    unsigned int incl = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned int o = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += o;
    }
    unsigned int ex = incl - run;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = lane * 4 + q;
      s_cnt[e / 8][e % 8] = ex;
      ex += v[q];
    }
    const unsigned int agg = __shfl_sync(0xffffffffu, incl, 31);
    bool to = false;
    const unsigned long long ex_tile = lookback_warp(ts, tile, agg, &to);
    if (lane == 0) {
      s_excl = ex_tile;
      if (to) {
        s_timeout = true;
        atomicExch(ts.error, 1);
      }
      const long long ntiles = (n + kTile - 1) / kTile;
      if (!to && tile == ntiles - 1) *ts.total = ex_tile + agg;
    }
  }
  __syncthreads();
  if (s_timeout) return;
  const unsigned long long excl = s_excl;
  const unsigned int lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    if (ballots[r] & (1u << lane)) {
      const long long i = base + r * kCompactThreads + threadIdx.x;
      const long long pos = (long long)(excl + s_cnt[r][warp] + __popc(ballots[r] & lt));
      if (pos < cap) {
        const int a = (int)(i / (N - 1));
        const int b = (int)(i - (long long)a * (N - 1));
        src[pos] = a;
        dst[pos] = b + (b >= a);
        copt[pos] = c[r];
        topt[pos] = t[r];
      }
    }
  }
}

// Exclusive scan of n counts: out[i] = count(0) + .. + count(i-1), the total
// written by the last tile to *ts.total.  Each thread takes kCompactRows
// consecutive items; tiles chain through the same look-back as compaction.
template <class Count>
__global__ void __launch_bounds__(kCompactThreads) scan_kernel(long long n, Count count,
                                                               unsigned int *out, TileScratch ts) {
  __shared__ unsigned int s_tile;
  __shared__ unsigned long long s_warp[kCompactThreads / 32];
  __shared__ unsigned long long s_excl;
  __shared__ bool s_timeout;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_tile = atomicAdd(ts.tile_counter, 1u);
    s_timeout = false;
  }
  __syncthreads();
  const long long tile = s_tile;
  const long long i0 = tile * kTile + (long long)threadIdx.x * kCompactRows;
  unsigned int v[kCompactRows];
  unsigned long long sum = 0;
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    v[r] = i0 + r < n ? count(i0 + r) : 0u;
    sum += v[r];
  }
  unsigned long long incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const unsigned long long w = lane < kCompactThreads / 32 ? s_warp[lane] : 0ull;
    unsigned long long wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long u = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += u;
    }
    if (lane < kCompactThreads / 32) s_warp[lane] = wi - w;
    const unsigned long long agg = __shfl_sync(0xffffffffu, wi, 31);
    bool to = false;
    const unsigned long long ex_tile = lookback_warp(ts, tile, agg, &to);
    if (lane == 0) {
      s_excl = ex_tile;
      if (to) {
        s_timeout = true;
        atomicExch(ts.error, 1);
      }
      const long long ntiles = (n + kTile - 1) / kTile;
      if (!to && tile == ntiles - 1) *ts.total = ex_tile + agg;
    }
  }
  __syncthreads();
  if (s_timeout) return;
  unsigned long long run = s_excl + s_warp[warp] + (incl - sum);
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    if (i0 + r < n) out[i0 + r] = (unsigned int)run;
    run += v[r];
  }
}

template <class Count>
pump_status_t run_scan(Ctx *ctx, long long n, Count count, unsigned int *out,
                       cudaStream_t stream, TileScratch *ts_out) {
  const long long ntiles = n > 0 ? (n + kTile - 1) / kTile : 1;
  const size_t bytes = sizeof(unsigned long long) * (ntiles + 2) + sizeof(unsigned int) * 4;
  char *scratch = nullptr;
  PUMP_TRY(ctx->scratch(Ctx::kCompact, bytes, (void **)&scratch));
  TileScratch ts{};
  ts.total = (unsigned long long *)scratch;
  ts.status = ts.total + 1;
  ts.tile_counter = (unsigned int *)(ts.status + ntiles + 1);
  ts.error = (int *)(ts.tile_counter + 1);
  PUMP_CUDA_TRY(cudaMemsetAsync(scratch, 0, bytes, stream));
  if (n > 0) {
    if (ntiles > 2147483647LL) return set_error(PUMP_ERR_CAPACITY, "scan: too many tiles");
    scan_kernel<<<(unsigned)ntiles, kCompactThreads, 0, stream>>>(n, count, out, ts);
    PUMP_TRY(launch_status("scan_kernel"));
  }
  *ts_out = ts;
  return PUMP_OK;
}

}  // namespace
}  // namespace pump
