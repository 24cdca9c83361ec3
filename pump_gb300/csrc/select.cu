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
#include <mutex>

#include "common.cuh"
#include "compact.cuh"
#include "ctx.h"
#include "pairview.cuh"

namespace pump {
namespace {


__device__ __forceinline__ uint32_t float_key(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
  return __uint_as_float(u);
}

// ---------------------------------------------------------- radix select
struct SelectState {
  uint32_t prefix;
  uint32_t mask;
  unsigned long long k;
  float result;
};

struct FlatSrc {
  const float *v;
  __device__ float operator()(long long i) const { return __ldg(&v[i]); }
};
struct PairCoptSrc {
  PairView pv;
  __device__ float operator()(long long idx) const {
    int i, j;
    pv.pair(idx, &i, &j);
    return pv.copt(i, j);
  }
};

// Src(i) -> the i-th value (a flat array, or a virtual pair array).
template <class Src>
__global__ void select_hist_kernel(Src src, long long n, const SelectState *__restrict__ st,
                                   int shift, int bits, unsigned int *__restrict__ hist) {
  __shared__ unsigned int sh[2048];
  const int nb = 1 << bits;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) sh[b] = 0;
  __syncthreads();
  const uint32_t prefix = st->prefix, mask = st->mask;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint32_t key = float_key(src(i));
    if ((key & mask) == prefix) atomicAdd(&sh[(key >> shift) & (nb - 1)], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

// Start state of a selection and a cleared histogram (a kernel instead of a
// host-to-device copy: a copy from pageable host memory would wait for the
// stream to drain first).
__global__ void select_init_kernel(SelectState *st, unsigned long long k, unsigned int *hist) {
  for (int i = threadIdx.x; i < 2048; i += blockDim.x) hist[i] = 0u;
  if (threadIdx.x == 0) {
    st->prefix = 0u;
    st->mask = 0u;
    st->k = k;
    st->result = 0.0f;
  }
}

// One block of 1024 threads: find the bin holding rank k, narrow the prefix,
// clear the histogram for the next pass.
__global__ void select_pick_kernel(SelectState *st, int shift, int bits, unsigned int *hist) {
  __shared__ unsigned long long cum[1024];
  const int nb = 1 << bits;
  const int per = nb / 1024;  // 1 or 2 bins per thread
  const int t = threadIdx.x;
  unsigned long long mine = 0;
  for (int q = 0; q < per; ++q) mine += hist[t * per + q];
  cum[t] = mine;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
    unsigned long long add = t >= off ? cum[t - off] : 0;
    __syncthreads();
    cum[t] += add;
    __syncthreads();
  }
  const unsigned long long k = st->k;
  unsigned long long before = cum[t] - mine;
  if (k >= before && k < cum[t]) {
    unsigned long long c = before;
    for (int q = 0; q < per; ++q) {
      const unsigned int h = hist[t * per + q];
      if (k < c + h) {
        const uint32_t bin = (uint32_t)(t * per + q);
        st->prefix |= bin << shift;
        st->mask |= (uint32_t)(nb - 1) << shift;
        st->k = k - c;
        if (shift == 0) st->result = key_float(st->prefix);
        break;
      }
      c += h;
    }
  }
  __syncthreads();
  for (int q = 0; q < per; ++q) hist[t * per + q] = 0;
}

// ------------------------------------------------------ compaction users
// Edges the search can expand: free edge to a free node (PUMP.cu:52-53).
struct OpenEdgePred {
  const uint8_t *free_e, *free_s;
  const int *dst;
  __device__ bool operator()(long long e) const { return free_e[e] && free_s[dst[e]]; }
};
struct OpenEdgeEmit {
  const int *src, *dst;
  const float *copt, *topt;
  int *f_id, *f_src, *f_dst;
  float *f_copt, *f_topt;
  __device__ void operator()(long long e, long long pos) const {
    f_id[pos] = (int)e;
    f_src[pos] = src[e];
    f_dst[pos] = dst[e];
    f_copt[pos] = copt[e];
    f_topt[pos] = topt[e];
  }
};
struct PairEdgePred {
  PairView pv;
  float rn;
  __device__ bool operator()(long long idx) const {
    int i, j;
    pv.pair(idx, &i, &j);
    return pv.copt(i, j) < rn;
  }
};
struct PairEdgeEmit {
  PairView pv;
  long long cap;
  int *src, *dst;
  float *copt, *topt;
  __device__ void operator()(long long idx, long long pos) const {
    if (pos >= cap) return;
    int i, j;
    pv.pair(idx, &i, &j);
    src[pos] = i;
    dst[pos] = j;
    copt[pos] = pv.copt(i, j);
    topt[pos] = pv.topt(i, j);
  }
};
struct FlagPred {
  const uint8_t *flags;
  __device__ bool operator()(long long i) const { return flags[i] != 0; }
};
struct IndexEmit {
  int *out;
  __device__ void operator()(long long idx, long long pos) const { out[pos] = (int)idx; }
};

// go_start[i] = first edge whose source is >= i (edges sorted by source).
__global__ void go_start_kernel(const int *__restrict__ src, long long E, int N,
                                int *__restrict__ go_start) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > N) return;
  long long lo = 0, hi = E;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (src[mid] < i) lo = mid + 1; else hi = mid;
  }
  go_start[i] = (int)lo;
}

__global__ void copy_count_kernel(const unsigned long long *total, int *out) { *out = (int)*total; }

// Device-side k-th smallest of src(0 .. n-1): the result lands in the ctx
// select state; *d_result points at it (device).
template <class Src>
pump_status_t select_kth_src(Ctx *ctx, Src src, long long n, long long k, const float **d_result,
                             cudaStream_t stream) {
  if (n <= 0 || k < 0 || k >= n) return set_error(PUMP_ERR_BAD_INPUT, "select_kth: k=%lld n=%lld", k, n);
  char *scratch = nullptr;
  const size_t bytes = sizeof(SelectState) + 2048 * sizeof(unsigned int);
  PUMP_TRY(ctx->scratch(Ctx::kSelect, bytes, (void **)&scratch));
  SelectState *st = (SelectState *)scratch;
  unsigned int *hist = (unsigned int *)(scratch + sizeof(SelectState));
  select_init_kernel<<<1, 1024, 0, stream>>>(st, (unsigned long long)k, hist);
  PUMP_TRY(launch_status("select_init_kernel"));
  long long blocks = (n + 1023) / 1024;
  if (blocks > kNumSMs * 8) blocks = kNumSMs * 8;
  const int shifts[3] = {21, 10, 0}, bits[3] = {11, 11, 10};
  for (int pass = 0; pass < 3; ++pass) {
    select_hist_kernel<<<(unsigned)blocks, 1024, 0, stream>>>(src, n, st, shifts[pass], bits[pass], hist);
    PUMP_TRY(launch_status("select_hist_kernel"));
    select_pick_kernel<<<1, 1024, 0, stream>>>(st, shifts[pass], bits[pass], hist);
    PUMP_TRY(launch_status("select_pick_kernel"));
  }
  *d_result = &st->result;
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

pump_status_t build_edges_device(Ctx *ctx, const float *d_copts, const float *d_topts, int N, float rn,
                                 long long max_edges, int *d_src, int *d_dst, float *d_copt,
                                 float *d_topt, int *d_go_start, long long *h_num_edges,
                                 cudaStream_t stream) {
  const long long npairs = (long long)N * (N - 1);
  TileScratch ts{};
  {
    const long long ntiles = npairs > 0 ? (npairs + kTile - 1) / kTile : 1;
    const size_t bytes = sizeof(unsigned long long) * (ntiles + 2) + sizeof(unsigned int) * 4;
    char *scratch = nullptr;
    PUMP_TRY(ctx->scratch(Ctx::kCompact, bytes, (void **)&scratch));
    ts.total = (unsigned long long *)scratch;
    ts.status = ts.total + 1;
    ts.tile_counter = (unsigned int *)(ts.status + ntiles + 1);
    ts.error = (int *)(ts.tile_counter + 1);
    PUMP_CUDA_TRY(cudaMemsetAsync(scratch, 0, bytes, stream));
    if (npairs > 0) {
      if (ntiles > 2147483647LL) return set_error(PUMP_ERR_CAPACITY, "build_edges: too many tiles");
      edge_compact_kernel<<<(unsigned)ntiles, kCompactThreads, 0, stream>>>(
          npairs, N, d_copts, d_topts, rn, max_edges, d_src, d_dst, d_copt, d_topt, ts);
      PUMP_TRY(launch_status("edge_compact_kernel"));
    }
  }
  unsigned long long total = 0;
  PUMP_TRY(finish_compact(ts, &total, stream));
  *h_num_edges = (long long)total;
  if ((long long)total > max_edges)
    return set_error(PUMP_ERR_CAPACITY, "build_edges: %llu edges exceed capacity %lld", total, max_edges);
  if (d_go_start) {
    go_start_kernel<<<grid_for(N + 1, 256), 256, 0, stream>>>(d_src, (long long)total, N, d_go_start);
    PUMP_TRY(launch_status("go_start_kernel"));
  }
  return PUMP_OK;
}

// The expandable edges in (source, destination) order with their row starts
// per source node: the adjacency the search walks, without the edges it
// would skip.
pump_status_t open_edges_device(Ctx *ctx, const uint8_t *d_free_e, const uint8_t *d_free_s,
                                const int *d_src, const int *d_dst, const float *d_copt,
                                const float *d_topt, long long E, int N, int *d_fid, int *d_fsrc,
                                int *d_fdst, float *d_fcopt, float *d_ftopt, int *d_fgo,
                                long long *h_count, cudaStream_t stream) {
  TileScratch ts{};
  PUMP_TRY(run_compact(ctx, E, OpenEdgePred{d_free_e, d_free_s, d_dst},
                       OpenEdgeEmit{d_src, d_dst, d_copt, d_topt, d_fid, d_fsrc, d_fdst, d_fcopt,
                                    d_ftopt},
                       stream, &ts));
  unsigned long long total = 0;
  PUMP_TRY(finish_compact(ts, &total, stream));
  *h_count = (long long)total;
  go_start_kernel<<<grid_for(N + 1, 256), 256, 0, stream>>>(d_fsrc, (long long)total, N, d_fgo);
  return launch_status("go_start_kernel");
}

// Device-side frontier compaction; *d_error_out (device) is nonzero when a
// look-back wait gave up.
// Edges of one query of a batch from its pair view (same order and values as
// build_edges_device on the query's own pair arrays).
pump_status_t build_edges_pairs(Ctx *ctx, const PairView &pv, float rn, long long max_edges,
                                int *d_src, int *d_dst, float *d_copt, float *d_topt,
                                int *d_go_start, long long *h_num_edges, cudaStream_t stream) {
  const int N = pv.N;
  const long long npairs = (long long)N * (N - 1);
  TileScratch ts{};
  PUMP_TRY(run_compact(ctx, npairs, PairEdgePred{pv, rn},
                       PairEdgeEmit{pv, max_edges, d_src, d_dst, d_copt, d_topt}, stream, &ts));
  unsigned long long total = 0;
  PUMP_TRY(finish_compact(ts, &total, stream));
  *h_num_edges = (long long)total;
  if ((long long)total > max_edges)
    return set_error(PUMP_ERR_CAPACITY, "build_edges: %llu edges exceed capacity %lld", total, max_edges);
  if (d_go_start) {
    go_start_kernel<<<grid_for(N + 1, 256), 256, 0, stream>>>(d_src, (long long)total, N, d_go_start);
    PUMP_TRY(launch_status("go_start_kernel"));
  }
  return PUMP_OK;
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
// device address, so the address is looked up once per device with
// cudaGetSymbolAddress (with that device current) on the first call made on
// it; make that first call before any stream capture.  Each call clears the
// words that must start at zero before its kernel runs; two calls that
// overlap on the GPU (for example on two streams) share the array and race,
// so serialise them.
namespace pump {
namespace {

constexpr long long kNoAllocMaxTiles = 8192;                   // 8192 tiles of 4096 flags
constexpr long long kNoAllocMaxFlags = kNoAllocMaxTiles * kTile;  // 33,554,432
// word 0: selected count; words 1 .. tiles: tile status; the word after the
// last status slot: tile counter (4 B) and error word (4 B)
constexpr int kNoAllocWords = 1 + (int)kNoAllocMaxTiles + 1 + 1;

static __device__ __align__(256) unsigned long long g_frontier_scratch[kNoAllocWords];

std::mutex g_scratch_mutex;
unsigned long long *g_scratch_addr[64] = {nullptr};

pump_status_t frontier_scratch_address(unsigned long long **out) {
  int dev = 0;
  PUMP_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(PUMP_ERR_BAD_INPUT, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_frontier_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_frontier_scratch)");
    g_scratch_addr[dev] = static_cast<unsigned long long *>(p);
  }
  *out = g_scratch_addr[dev];
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
                                                                IndexEmit{d_active}, ts);
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
