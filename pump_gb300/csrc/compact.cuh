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
#include "tune.h"

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
  unsigned long long *offsets; // per-tile output offsets (three-kernel compaction)
  unsigned long long *copy_to; // optional second destination of the total
};

// Exclusive prefix of this tile from its predecessors' status words, read by
// a whole warp in windows of 32 x kLookbackPerLane tiles: lane l reads the
// status of tiles p - V l - v (v < V), so one round trip to L2 covers 128
// predecessors and the published-prefix front advances by up to 128 tiles per
// round trip.  The tiles up to the nearest inclusive prefix must all have
// published (at least an aggregate); otherwise the warp waits and reads the
// window again.  A status word carries its own value, so relaxed loads and
// stores suffice (an acquire load would also order the lane's V loads one
// after another).  Called by every lane of one warp; every lane returns the
// same value.
constexpr int kLookbackPerLane = 4;
__device__ unsigned long long lookback_warp(const TileScratch &ts, long long tile,
                                            unsigned long long agg, bool *timed_out,
                                            long long spin_limit = kSpinLimit) {
  using ref_t = cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>;
  constexpr int V = kLookbackPerLane;
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) ref_t(ts.status[0]).store(kFlagPrefix | agg, cuda::memory_order_relaxed);
    return 0;
  }
  if (lane == 0) ref_t(ts.status[tile]).store(kFlagAggregate | agg, cuda::memory_order_relaxed);
  unsigned long long excl = 0;
  long long p = tile - 1;  // nearest tile of the window
  long long spins = 0;
  while (true) {
    unsigned long long st[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const long long q = p - (long long)V * lane - v;
      // before tile 0 the prefix is 0 (a published prefix of value 0)
      st[v] = q >= 0 ? ref_t(ts.status[q]).load(cuda::memory_order_relaxed) : kFlagPrefix;
    }
    int first = V;  // this lane's nearest entry holding a prefix
#pragma unroll
    for (int v = V - 1; v >= 0; --v)
      if ((st[v] & ~kValueMask) == kFlagPrefix) first = v;
    const unsigned int pref = __ballot_sync(0xffffffffu, first < V);
    const int stop = pref ? __ffs(pref) - 1 : 32;  // lane holding the nearest prefix
    // entries this lane contributes: all V before the stop lane, up to its
    // prefix entry in the stop lane, none after it
    const int used = lane < stop ? V : (lane == stop ? first + 1 : 0);
    bool missing = false;
    unsigned long long sum = 0;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      if (v < used) {
        if ((st[v] & ~kValueMask) == 0) missing = true;
        sum += st[v] & kValueMask;
      }
    }
    if (__any_sync(0xffffffffu, missing)) {
      if (++spins > spin_limit) {
        *timed_out = true;
        return 0;
      }
      __nanosleep(32);
      continue;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    excl += sum;
    if (pref) break;
    p -= 32 * V;
  }
  if (lane == 0) ref_t(ts.status[tile]).store(kFlagPrefix | (excl + agg), cuda::memory_order_relaxed);
  return excl;
}

// Shared state of one compaction tile: per (row, warp) selected counts, turned
// into exclusive offsets within the tile, and the tile's exclusive prefix.
struct TileShared {
  unsigned int cnt[kCompactRows][kCompactThreads / 32];
  unsigned long long excl;
  bool timeout;
};

// Called by every thread after lane 0 of each warp stored its row counts in
// sh.cnt: warp 0 scans the 16 x 8 counts in (row, warp) order and finds the
// tile's prefix by look-back; the last tile writes the total.  False when the
// look-back wait gave up (the error word is set; the tile writes nothing).
// Warp 0: the tile's 16 x 8 (row, warp) counts, in (row, warp) order, turned
// into exclusive offsets in place; returns the tile's total (every lane).
__device__ __forceinline__ unsigned int scan_tile_counts(
    unsigned int (&cnt)[kCompactRows][kCompactThreads / 32]) {
  const int lane = threadIdx.x & 31;
  unsigned int v[4];
  unsigned int run = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int e = lane * 4 + q;
    v[q] = cnt[e / 8][e % 8];
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
    cnt[e / 8][e % 8] = ex;
    ex += v[q];
  }
  return __shfl_sync(0xffffffffu, incl, 31);
}

__device__ __forceinline__ bool tile_offsets(TileShared &sh, const TileScratch &ts, long long tile,
                                             long long n) {
  __syncthreads();
  const int lane = threadIdx.x & 31;
  if ((threadIdx.x >> 5) == 0) {
    const unsigned int agg = scan_tile_counts(sh.cnt);
    bool to = false;
    const unsigned long long ex_tile = lookback_warp(ts, tile, agg, &to);
    if (lane == 0) {
      sh.excl = ex_tile;
      sh.timeout = to;
      if (to) atomicExch(ts.error, 1);
      const long long ntiles = (n + kTile - 1) / kTile;
      if (!to && tile == ntiles - 1) {
        *ts.total = ex_tile + agg;
        if (ts.copy_to) *ts.copy_to = ex_tile + agg;
      }
    }
  }
  __syncthreads();
  return !sh.timeout;
}

// Tile index from the atomic counter (every tile a block waits on has started).
__device__ __forceinline__ long long next_tile(const TileScratch &ts) {
  __shared__ unsigned int s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(ts.tile_counter, 1u);
  __syncthreads();
  return s_tile;
}

// Pred(i) -> bool, Emit(i, pos) writes item i at output position pos.  With
// d_n the item count is *d_n when below n (n, the host's bound, sized the
// grid): tiles wholly past it leave at once (no tile waits on a later one).
template <class Pred, class Emit>
__global__ void __launch_bounds__(kCompactThreads) compact_kernel(long long n, Pred pred, Emit emit,
                                                                  TileScratch ts,
                                                                  const unsigned long long *d_n) {
  __shared__ TileShared sh;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long tile = next_tile(ts);
  const long long base = tile * kTile;
  if (d_n) {
    const unsigned long long d = *d_n;
    if ((long long)d < n) n = (long long)d;
    if (base >= n && tile > 0) return;
  }
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
    if (lane == 0) sh.cnt[r][warp] = __popc(ballots[r]);
  }
  if (!tile_offsets(sh, ts, tile, n)) return;
  const unsigned long long excl = sh.excl;
  const unsigned int lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    if (ballots[r] & (1u << lane)) {
      const long long i = base + r * kCompactThreads + threadIdx.x;
      emit(i, (long long)(excl + sh.cnt[r][warp] + __popc(ballots[r] & lt)));
    }
  }
}

// Zeroed tile status words, tile counter, total and error word for a pass
// over n items in tiles of tile_items (ctx compaction scratch);
// *ntiles_out = the tiles to launch.
pump_status_t prepare_tiles(Ctx *ctx, long long n, cudaStream_t stream, TileScratch *ts_out,
                            long long *ntiles_out, long long tile_items = kTile,
                            int slot = Ctx::kCompact) {
  const long long ntiles = n > 0 ? (n + tile_items - 1) / tile_items : 1;
  if (ntiles > 2147483647LL) return set_error(PUMP_ERR_CAPACITY, "compaction: too many tiles");
  const size_t zeroed = sizeof(unsigned long long) * (ntiles + 2) + sizeof(unsigned int) * 4;
  const size_t bytes = zeroed + sizeof(unsigned long long) * ntiles;
  char *scratch = nullptr;
  PUMP_TRY(ctx->scratch(slot, bytes, (void **)&scratch));
  TileScratch ts{};
  ts.total = (unsigned long long *)scratch;
  ts.status = ts.total + 1;
  ts.tile_counter = (unsigned int *)(ts.status + ntiles + 1);
  ts.error = (int *)(ts.tile_counter + 1);
  ts.offsets = (unsigned long long *)(scratch + zeroed);
  PUMP_CUDA_TRY(cudaMemsetAsync(scratch, 0, zeroed, stream));
  *ts_out = ts;
  *ntiles_out = ntiles;
  return PUMP_OK;
}

template <class Pred, class Emit>
pump_status_t run_compact(Ctx *ctx, long long n, Pred pred, Emit emit, cudaStream_t stream,
                          TileScratch *ts_out, const unsigned long long *d_n = nullptr) {
  TileScratch ts{};
  long long ntiles = 0;
  PUMP_TRY(prepare_tiles(ctx, n, stream, &ts, &ntiles));
  if (n > 0) {
    compact_kernel<<<(unsigned)ntiles, kCompactThreads, 0, stream>>>(n, pred, emit, ts, d_n);
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

// --------------------------------------- three-kernel tile compaction
// For large inputs: a count kernel (blocks stride over the tiles) adds each
// warp's selected count into its tile's count; one block scans the tile
// counts into output offsets; an emit kernel (the same striding) writes each
// tile's selected items from its offset, ranks in index order as in
// compact_kernel.  The input is read twice, but no block waits on another:
// on large inputs the look-back front of compact_kernel, not the reads, sets
// its pace.
//
// A loader L supplies the items: L::Item (per-item registers), L::State
// (per-block constants, from ld.begin()), ld.load(base, n, v) (this thread's
// kCompactRows items of the tile at base: item r is base + r * 256 + tid),
// ld.sel(st, item) and ld.emit(i, item, pos).
constexpr int kTileBlocks = kNumSMs * 4;

template <class L>
__device__ __forceinline__ void tile_ballots(const L &ld, const typename L::State &st,
                                             long long base, long long n,
                                             typename L::Item (&v)[kCompactRows],
                                             unsigned int (&b)[kCompactRows]) {
  ld.load(base, n, v);
#pragma unroll
  for (int r = 0; r < kCompactRows; ++r) {
    const long long i = base + r * kCompactThreads + threadIdx.x;
    b[r] = __ballot_sync(0xffffffffu, i < n && ld.sel(st, v[r]));
  }
}

// The item count: n, or *d_n when d_n is given and below n (a count left on
// the device by an earlier kernel; n is then the bound the grid was sized for).
__device__ __forceinline__ long long device_count(long long n, const unsigned long long *d_n) {
  if (d_n) {
    const unsigned long long d = *d_n;
    if ((long long)d < n) n = (long long)d;
  }
  return n;
}

// counts[tile] += each warp's selected count (counts zeroed before launch).
template <class L>
__global__ void __launch_bounds__(kCompactThreads) tile_count_kernel(long long n, L ld,
                                                                     unsigned int *counts,
                                                                     const unsigned long long *d_n) {
  const int lane = threadIdx.x & 31;
  n = device_count(n, d_n);
  const long long ntiles = (n + kTile - 1) / kTile;
  const typename L::State st = ld.begin();
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    typename L::Item v[kCompactRows];
    unsigned int b[kCompactRows];
    tile_ballots(ld, st, tile * kTile, n, v, b);
    unsigned int cnt = 0;
#pragma unroll
    for (int r = 0; r < kCompactRows; ++r) cnt += __popc(b[r]);
    if (lane == 0 && cnt) atomicAdd(&counts[tile], cnt);
  }
}

// One block of 1024 threads: offsets[t] = counts[0] + .. + counts[t-1] and
// *total (and *copy_to, when given) = the sum of all; each thread scans a
// contiguous run of tiles.
__global__ void __launch_bounds__(1024) tile_scan_kernel(const unsigned int *__restrict__ counts,
                                                         long long ntiles,
                                                         unsigned long long *__restrict__ offsets,
                                                         unsigned long long *total,
                                                         unsigned long long *copy_to) {
  __shared__ unsigned long long s_warp[32];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const long long per = (ntiles + 1023) / 1024;
  const long long t0 = t * per, t1 = t0 + per < ntiles ? t0 + per : ntiles;
  unsigned long long sum = 0;
  for (long long q = t0; q < t1; ++q) sum += counts[q];
  unsigned long long incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const unsigned long long w = s_warp[lane];
    unsigned long long wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long u = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += u;
    }
    s_warp[lane] = wi - w;
    if (lane == 31) {
      *total = wi;
      if (copy_to) *copy_to = wi;
    }
  }
  __syncthreads();
  unsigned long long run = s_warp[warp] + incl - sum;
  for (long long q = t0; q < t1; ++q) {
    offsets[q] = run;
    run += counts[q];
  }
}

template <class L>
__global__ void __launch_bounds__(kCompactThreads) tile_emit_kernel(
    long long n, L ld, const unsigned long long *__restrict__ offsets,
    const unsigned long long *d_n) {
  __shared__ unsigned int cnt[kCompactRows][kCompactThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  n = device_count(n, d_n);
  const long long ntiles = (n + kTile - 1) / kTile;
  const typename L::State st = ld.begin();
  const unsigned int lt = (1u << lane) - 1u;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long base = tile * kTile;
    const unsigned long long off = __ldg(&offsets[tile]);
    typename L::Item v[kCompactRows];
    unsigned int b[kCompactRows];
    tile_ballots(ld, st, base, n, v, b);
    if (lane == 0) {
#pragma unroll
      for (int r = 0; r < kCompactRows; ++r) cnt[r][warp] = __popc(b[r]);
    }
    __syncthreads();
    if (warp == 0) scan_tile_counts(cnt);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kCompactRows; ++r)
      if (b[r] & (1u << lane))
        ld.emit(base + r * kCompactThreads + threadIdx.x, v[r],
                (long long)(off + cnt[r][warp] + __popc(b[r] & lt)));
    __syncthreads();  // cnt is rewritten by the next tile
  }
}

// The scan and emit kernels of a three-kernel compaction whose tile counts
// are in place (ts from prepare_tiles; ntiles tiles).
template <class L>
pump_status_t run_chunked_emit(long long n, long long ntiles, const L &ld, cudaStream_t stream,
                               const TileScratch &ts, int blocks_per_sm,
                               const unsigned long long *d_n) {
  const long long grid = (long long)kNumSMs * blocks_per_sm;
  const unsigned blocks = (unsigned)(ntiles < grid ? ntiles : grid);
  tile_scan_kernel<<<1, 1024, 0, stream>>>(reinterpret_cast<unsigned int *>(ts.status), ntiles,
                                           ts.offsets, ts.total, ts.copy_to);
  PUMP_TRY(launch_status("tile_scan_kernel"));
  tile_emit_kernel<<<blocks, kCompactThreads, 0, stream>>>(n, ld, ts.offsets, d_n);
  return launch_status("tile_emit_kernel");
}

// Three-kernel compaction of n items (or of *d_n, when given and below n);
// the count lands in *ts_out->total and, when given, in *copy_to (the
// compaction scratch, and with it *total, is reused by the next compaction
// on the context).  The error word stays zero: nothing waits.
// blocks_per_sm sets the count and emit grids (the autotuner's choice where
// a caller tunes it).
template <class L>
pump_status_t run_chunked(Ctx *ctx, long long n, const L &ld, cudaStream_t stream,
                          TileScratch *ts_out, int blocks_per_sm = kTileBlocks / kNumSMs,
                          const unsigned long long *d_n = nullptr,
                          unsigned long long *copy_to = nullptr) {
  TileScratch ts{};
  long long ntiles = 0;
  PUMP_TRY(prepare_tiles(ctx, n, stream, &ts, &ntiles));  // zeroed status words hold the counts
  ts.copy_to = copy_to;
  if (n > 0) {
    const long long grid = (long long)kNumSMs * blocks_per_sm;
    const unsigned blocks = (unsigned)(ntiles < grid ? ntiles : grid);
    unsigned int *counts = reinterpret_cast<unsigned int *>(ts.status);
    tile_count_kernel<<<blocks, kCompactThreads, 0, stream>>>(n, ld, counts, d_n);
    PUMP_TRY(launch_status("tile_count_kernel"));
    PUMP_TRY(run_chunked_emit(n, ntiles, ld, stream, ts, blocks_per_sm, d_n));
  }
  *ts_out = ts;
  return PUMP_OK;
}

// run_chunked with the grid picked by the autotuner (2, 4 or 8 blocks per SM)
// for shape class (kernel, the input size's power-of-two bucket).
template <class L>
pump_status_t run_chunked_tuned(Ctx *ctx, int kernel, long long n, const L &ld,
                                cudaStream_t stream, TileScratch *ts_out,
                                const unsigned long long *d_n = nullptr,
                                unsigned long long *copy_to = nullptr) {
  static const int kPerSm[3] = {2, 4, 8};
  auto run = [&](int c) {
    return run_chunked(ctx, n, ld, stream, ts_out, kPerSm[c], d_n, copy_to);
  };
  int choice = 1;
  bool ran = false;
  PUMP_TRY(tune_choice(kernel, tune_bucket(n), 3, 1, stream, run, &choice, &ran));
  return ran ? PUMP_OK : run(choice);
}

// go_start[r] = the first edge whose source is >= r (edges sorted by source),
// r = 0 .. N: thread e (0 .. E) writes the rows (src[e-1], src[e]], with
// src[-1] = -1 and src[E] = N, so each row is written once.
__global__ void row_starts_kernel(const int *__restrict__ src, long long E, int N,
                                  int *__restrict__ go_start,
                                  const unsigned long long *__restrict__ E_dev) {
  if (E_dev) {  // the count from the device, never past the bound E
    const long long d = (long long)*E_dev;
    if (d < E) E = d;
  }
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e <= E;
       e += (long long)gridDim.x * blockDim.x) {
    const int prev = e > 0 ? src[e - 1] : -1;
    const int cur = e < E ? src[e] : N;
    for (int r = prev + 1; r <= cur; ++r) go_start[r] = (int)e;
  }
}

// Row starts of the edges' sources (sorted); with E_dev the edge count is
// read on the device and E only sizes the grid (an upper bound).
pump_status_t row_starts(const int *d_src, long long E, int N, int *d_go_start,
                         cudaStream_t stream, const unsigned long long *E_dev = nullptr) {
  long long blocks = (E + 1 + 255) / 256;
  if (blocks > kNumSMs * 8) blocks = kNumSMs * 8;
  row_starts_kernel<<<(unsigned)blocks, 256, 0, stream>>>(d_src, E, N, d_go_start, E_dev);
  return launch_status("row_starts_kernel");
}

}  // namespace
}  // namespace pump
