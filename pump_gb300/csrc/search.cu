// Device-resident exploration: the steps of one iteration of the reference's
// search loop (PUMP.cu:39-290) as kernels over device state.  Paths are
// numbered, stored and bucketed exactly as the host loop numbers them:
// expansion follows the bucket order and each node's edge order (an
// exclusive scan of out-degrees), survivors keep wavefront order (stable
// compaction), and bucket appends keep survivor order.  Dominance only asks
// whether some path dominates, so the per-node lists it walks may be in any
// order.
#include "search.h"

#include "collide.cuh"
#include "common.cuh"
#include "compact.cuh"
#include "ctx.h"
#include "pathpoint.cuh"

namespace pump {
namespace {

__device__ __forceinline__ void search_init_body(const SearchDev &sd) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < sd.N; i += gridDim.x * blockDim.x)
    sd.node_head[i] = -1;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sd.path_prev[0] = -2;
    sd.path_node[0] = 0;
    sd.path_cost[0] = 0.0f;
    sd.path_time[0] = 0.0f;
    sd.path_cp[0] = 0.0f;
    sd.node_next[0] = -1;
    sd.g_list[0][0] = 0;
    sd.ctl->num_new = 0;
    sd.ctl->num_valid = 0;
    sd.ctl->g_count[0] = 1;
    sd.ctl->g_count[1] = 0;
    sd.ctl->goal_found = 0;
    sd.ctl->g_base[0] = 0;
    sd.ctl->g_base[1] = 0;
    sd.ctl->wait_error = 0;
    sd.ctl->overflow = 0;
    // the initial node is listed for its edge checks unless its edges were
    // checked up front
    const bool listed = sd.open_cnt[0] == -1;
    if (listed) {
      sd.open_cnt[0] = 0;
      sd.todo[0] = 0;
    }
    sd.ctl->todo = listed ? 1 : 0;
  }
}

__global__ void search_init_kernel(SearchDev sd) { search_init_body(sd); }

// node_head[0] = path 0 after the per-node reset (separate launch: the
// reset above is grid-strided).
__global__ void search_init_head_kernel(SearchDev sd) { sd.node_head[0] = 0; }


// Work items (listed node, chunk of kChkEdges out-edges), chunks per node
// up to the roadmap's largest degree, taken by blocks in turn so a node's
// edges are spread over many blocks.  Per chunk the waypoints
// (discretize_kernel's arithmetic) are computed one thread per (edge,
// waypoint) and stored to disc (the chunk's records are contiguous), their
// positions kept in shared memory.  Then kChkLanes threads share each edge:
// box o goes to lane o % kChkLanes, which tests it against every segment of
// the edge (the reference's (segment, box) test), skipping first a box that
// is broadphase-disjoint from the whole edge's bounding box (an exact filter;
// none skipped when a waypoint is NaN).  The edge is free when no lane found
// a hit: the reference's result is the AND over its (segment, box) pairs, so
// the split changes no result, and a search iteration that reaches few nodes
// runs a short chain of box tests per thread instead of all of them.  Each
// chunk adds its count of free edges to free nodes to the node's count.
// The wide form, for iterations that list many nodes: 256-edge chunks, and
// each warp tests its 32 edges with the pair queue of warp_queue_hits (the
// eager edge check's test), which keeps the lanes busy where the narrow
// form's box split leaves them waiting on the longest box list.
constexpr int kChkThreads = 256;
constexpr int kChkLanes = 8;
constexpr int kChkEdges = kChkThreads / kChkLanes;  // 32
constexpr int kChkWideEdges = kChkThreads;          // 256

size_t check_smem(int numObs, int numDisc, bool wide) {
  return sizeof(float) * ((size_t)((numObs * 12 + 3) & ~3) +
                          (size_t)(wide ? kChkWideEdges : kChkEdges) * (numDisc + 1) * 3);
}

template <int Mode, bool Wide>
__device__ __forceinline__ void check_body(const SearchDev &sd, const CheckArgs &ca) {
  constexpr int kEdges = Wide ? kChkWideEdges : kChkEdges;
  extern __shared__ float4 s_dyn4[];
  __shared__ int s_open[kChkThreads / 32];
  __shared__ int s_off[kEdges + 1];  // ragged layout: the chunk's edges' first records
  float *s_obs = reinterpret_cast<float *>(s_dyn4);
  const int numDisc = ca.numDisc, W = numDisc + 1;
  const long long *off = ca.disc_off;
  float *s_wp = s_obs + ((ca.numObs * 12 + 3) & ~3);  // kEdges x W x 3 positions
  const int n_todo = sd.ctl->todo;
  const int chunks = ca.max_degree > kEdges ? (ca.max_degree + kEdges - 1) / kEdges : 1;
  const long long items = (long long)n_todo * chunks;
  if (blockIdx.x >= items) return;  // no item: leave before staging (block-uniform)
  stage_obstacles(ca.obs, ca.numObs, s_obs);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int el = threadIdx.x / kChkLanes, part = threadIdx.x % kChkLanes;
  for (long long j = blockIdx.x; j < items; j += gridDim.x) {
    const int t = (int)(j / chunks), c = (int)(j - (long long)t * chunks);
    const int node = sd.todo[t];
    const int e1 = sd.go[node + 1];
    const int c0 = sd.go[node] + c * kEdges;
    if (c0 >= e1) continue;  // block-uniform: this node has fewer chunks
    const int ne = e1 - c0 < kEdges ? e1 - c0 : kEdges;
    // the chunk's records: ne * W, or the edges' own ranges (ragged layout)
    long long rbase = (long long)c0 * W;
    int total = ne * W;
    if (off) {
      for (int k = threadIdx.x; k <= ne; k += kChkThreads) s_off[k] = (int)(off[c0 + k] - off[c0]);
      __syncthreads();
      rbase = off[c0];
      total = s_off[ne];
      if (total > kEdges * W) {  // a count past the staged capacity (never from disc_offsets)
        __syncthreads();
        continue;
      }
    }
    for (int q = threadIdx.x; q < total; q += kChkThreads) {
      int eq, i, nd = numDisc;
      if (off) {  // the chunk edge holding record q
        int lo = 0, hi = ne;
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (s_off[mid] <= q) lo = mid;
          else hi = mid;
        }
        eq = lo;
        i = q - s_off[eq];
        nd = s_off[eq + 1] - s_off[eq] - 1;
      } else {
        eq = q / W;
        i = q - eq * W;
      }
      const int e = c0 + eq;
      const int b = sd.dst[e];
      float x0[kDim], x1[kDim], x[kDim];
#pragma unroll
      for (int d = 0; d < kDim; ++d) {
        x0[d] = __ldg(&ca.samples[node * kDim + d]);
        x1[d] = __ldg(&ca.samples[b * kDim + d]);
      }
      if (i == 0) {
#pragma unroll
        for (int d = 0; d < kDim; ++d) x[d] = x0[d];
      } else if (i == nd) {
#pragma unroll
        for (int d = 0; d < kDim; ++d) x[d] = x1[d];
      } else {
        const float topt = ca.wp_topt[e];
        const float dt = topt / nd;
        if (Mode == PUMP_BVP_PARITY) path_point_fast(dt * i, topt, x0, x1, x);
        else path_point_f32(dt * i, topt, x0, x1, x);
      }
      // consecutive threads write consecutive 24-byte records: a warp's
      // stores cover one contiguous range
      float2 *out = reinterpret_cast<float2 *>(ca.disc + (rbase + q) * kDim);
      out[0] = make_float2(x[0], x[1]);
      out[1] = make_float2(x[2], x[3]);
      out[2] = make_float2(x[4], x[5]);
#pragma unroll
      for (int d = 0; d < 3; ++d) s_wp[q * 3 + d] = x[d];
    }
    __syncthreads();
    if constexpr (Wide) {
      __shared__ int s_q[kChkThreads / 32][kQueueSlots];
      __shared__ uint8_t s_h[kChkThreads];
      const bool active = (int)threadIdx.x < ne;
      const bool h = off ? warp_queue_hits(s_wp + (warp * 32 < ne ? s_off[warp * 32] : 0) * 3,
                                           OffsetLanes{s_off + warp * 32}, s_obs, ca.numObs, active,
                                           s_q[warp], s_h + warp * 32)
                         : warp_queue_hits(s_wp + warp * 32 * W * 3, W, s_obs, ca.numObs, active,
                                           s_q[warp], s_h + warp * 32);
      int open = 0;
      if (active) {
        const int e = c0 + threadIdx.x;
        sd.free_e[e] = h ? 0 : 1;
        open = (!h && sd.free_s[sd.dst[e]]) ? 1 : 0;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) open += __shfl_xor_sync(0xffffffffu, open, o);
      if (lane == 0) s_open[warp] = open;
      __syncthreads();  // also: every lane is done with s_wp
      if (threadIdx.x == 0) {
        int tot = 0;
        for (int q = 0; q < kChkThreads / 32; ++q) tot += s_open[q];
        if (tot) atomicAdd(&sd.open_cnt[node], tot);
      }
      __syncthreads();  // s_open and s_wp are rewritten by the next item
      continue;
    }
    bool hit = false;
    if (el < ne) {
      constexpr int kPos = 3;  // floats per staged waypoint
      const float *wp = s_wp + (off ? s_off[el] : el * W) * kPos;
      const int We = off ? s_off[el + 1] - s_off[el] : W, nde = We - 1;
      float emin[3], emax[3];
      bool nan = false;
#pragma unroll
      for (int d = 0; d < 3; ++d) emin[d] = emax[d] = wp[d];
      for (int i = 0; i < We; ++i)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const float x = wp[i * kPos + d];
          nan = nan || x != x;
          emin[d] = fminf(emin[d], x);
          emax[d] = fmaxf(emax[d], x);
        }
      for (int o = part; o < ca.numObs && !hit; o += kChkLanes) {
        const float *ob = &s_obs[o * 12];
        if (!nan && broadphase_valid(emin, emax, ob)) continue;
        float v[3], w[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) v[d] = wp[d];
        for (int i = 0; i < nde && !hit; ++i) {
#pragma unroll
          for (int d = 0; d < 3; ++d) w[d] = wp[(i + 1) * kPos + d];
          hit = segment_box_hit(v, w, ob);
#pragma unroll
          for (int d = 0; d < 3; ++d) v[d] = w[d];
        }
      }
    }
    // the edge's lanes are kChkLanes consecutive lanes of one warp
    const unsigned int hits = __ballot_sync(0xffffffffu, hit);
    int open = 0;
    if (el < ne && part == 0) {
      const int e = c0 + el;
      const bool ok = ((hits >> (lane & ~(kChkLanes - 1))) & ((1u << kChkLanes) - 1u)) == 0u;
      sd.free_e[e] = ok ? 1 : 0;
      open = (ok && sd.free_s[sd.dst[e]]) ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) open += __shfl_xor_sync(0xffffffffu, open, o);
    if (lane == 0) s_open[warp] = open;
    __syncthreads();  // also: every lane is done with s_wp
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int q = 0; q < kChkThreads / 32; ++q) tot += s_open[q];
      if (tot) atomicAdd(&sd.open_cnt[node], tot);
    }
    __syncthreads();  // s_open and s_wp are rewritten by the next item
  }
}

template <int Mode, bool Wide>
__global__ void __launch_bounds__(kChkThreads) check_kernel(SearchDev sd, CheckArgs ca) {
  check_body<Mode, Wide>(sd, ca);
}

// One warp per node: open_cnt[node] = its free edges to free nodes.
__global__ void count_open_kernel(SearchDev sd) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  for (long long n = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / 32; n < sd.N; n += warps) {
    int c = 0;
    for (int e = sd.go[n] + lane; e < sd.go[n + 1]; e += 32) c += (sd.free_e[e] && sd.free_s[sd.dst[e]]) ? 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) sd.open_cnt[n] = c;
  }
}

__global__ void max_degree_kernel(const int *__restrict__ go, int N, int *out) {
  __shared__ int s_max[32];
  int m = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) m = max(m, go[i + 1] - go[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    int r = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r = max(r, s_max[q]);
    *out = r;
  }
}

// Zeroes a tile-scratch region (grid-stride).
__device__ __forceinline__ void zero_tiles(const LoopTiles &t) {
  const long long n = loop_tile_words(t.cap);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    t.total[i] = 0ull;
}

// The expansion in one pass (PUMP.cu:47-66): the bucket's paths in tiles
// of kExpTile, taken in order from the tile counter.  A path's offset in the
// wavefront is its exclusive prefix of expandable-edge counts (in-tile scan,
// then the tile's prefix by look-back), and one warp per path writes its
// free edges to free nodes in edge order, clearing the per-node lists of new
// paths at their nodes.  The last tile writes the wavefront size and flags
// an iteration that would overflow: a wavefront larger than max_paths, or
// one that would bring the stored paths to max_paths (PUMP.cu:62-64, 73-76).
// The kernels after it then see an empty wavefront, and writes past the
// wavefront's capacity (max_paths + 1) are dropped.  The same kernel empties
// the bucket, records the bucket sizes the appends start from, and zeroes
// the store pass's tile scratch for this iteration.
constexpr int kExpTile = 32;       // paths per tile: one per lane of the scanning warp
constexpr int kExpThreads = 1024;  // one warp writes each of the tile's paths
constexpr int kExpChunks = 4;      // 32-edge chunks of a path loaded together
static_assert(kLoopScanTile == kExpTile, "expansion tile size");

__device__ __forceinline__ void expand_body(const SearchDev &sd, const int *g, int n_g, int g_idx,
                                            int num_paths, int max_paths, const TileScratch &ts,
                                            const LoopTiles &store) {
  {
    const long long nb = loop_tile_words(store.cap);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nb; i += stride)
      store.total[i] = 0ull;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    SearchCtl *c = sd.ctl;
    c->g_count[g_idx] = 0;
    c->g_base[g_idx] = 0;
    c->g_base[1 - g_idx] = c->g_count[1 - g_idx];
    c->num_valid = 0;
    c->todo = 0;  // this iteration's checks have run
  }
  __shared__ unsigned int s_off[kExpTile];
  __shared__ int s_prev[kExpTile], s_node[kExpTile];
  __shared__ int s_timeout;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned int lt = (1u << lane) - 1u;
  const long long ntiles = ((long long)n_g + kExpTile - 1) / kExpTile;
  const unsigned long long cap = (unsigned long long)max_paths + 1ull;
  while (true) {
    const long long tile = next_tile(ts);  // synchronises the block
    if (tile >= ntiles) break;             // block-uniform
    if (warp == 0) {
      const long long i = tile * kExpTile + lane;
      unsigned int cnt = 0u;
      if (i < n_g) {
        const int prev = g[i];
        const int node = sd.path_node[prev];
        s_prev[lane] = prev;  // the path warps start from these
        s_node[lane] = node;
        cnt = (unsigned int)sd.open_cnt[node];
      }
      unsigned int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
      }
      const unsigned int agg = __shfl_sync(0xffffffffu, incl, 31);
      bool to = false;
      const unsigned long long ex = lookback_warp(ts, tile, agg, &to);
      s_off[lane] = (unsigned int)(ex + (incl - cnt));
      if (lane == 0) {
        s_timeout = to ? 1 : 0;
        if (to) {
          atomicExch(ts.error, 1);
          atomicExch(&sd.ctl->wait_error, 1);
        }
        if (!to && tile == ntiles - 1) {
          const unsigned long long nn = ex + agg;
          sd.ctl->num_new = nn;
          sd.ctl->overflow =
              nn > (unsigned long long)max_paths
                  ? 1
                  : ((unsigned long long)num_paths + nn >= (unsigned long long)max_paths ? 2 : 0);
        }
      }
    }
    __syncthreads();
    if (s_timeout) break;  // block-uniform
    const long long rest = (long long)n_g - tile * kExpTile;
    const int in_tile = (int)(rest < kExpTile ? rest : kExpTile);
    for (int p = warp; p < in_tile; p += kExpThreads / 32) {
      const int prev = s_prev[p];
      const int node = s_node[p];
      const int e0 = __ldg(&sd.go[node]), e1 = __ldg(&sd.go[node + 1]);
      unsigned int off = s_off[p];
      // the node's expandable edges in edge order (PUMP.cu:52-53), kExpChunks
      // chunks of 32 edges at a time: their loads are issued together (the
      // roadmap arrays are read-only here), then the chunks are written in
      // order
      for (int b0 = e0; b0 < e1; b0 += 32 * kExpChunks) {
        int dst[kExpChunks];
        bool open[kExpChunks];
#pragma unroll
        for (int c = 0; c < kExpChunks; ++c) {
          const int e = b0 + 32 * c + lane;
          dst[c] = e < e1 ? __ldg(&sd.dst[e]) : 0;
          open[c] = e < e1 && __ldg(&sd.free_e[e]) != 0;
        }
#pragma unroll
        for (int c = 0; c < kExpChunks; ++c) open[c] = open[c] && __ldg(&sd.free_s[dst[c]]) != 0;
#pragma unroll
        for (int c = 0; c < kExpChunks; ++c) {
          const int e = b0 + 32 * c + lane;
          const unsigned int bal = __ballot_sync(0xffffffffu, open[c]);
          const unsigned int q = off + __popc(bal & lt);
          if (open[c] && q < cap) {
            sd.wf_prev[q] = prev;
            sd.wf_node[q] = dst[c];
            sd.wf_edge[q] = e;
            sd.wf_open[q] = e;
            sd.new_head[dst[c]] = -1;
          }
          off += __popc(bal);
        }
      }
    }
    __syncthreads();  // s_off is rewritten by the next tile
  }
}

__global__ void __launch_bounds__(kExpThreads) expand_kernel(SearchDev sd, const int *g, int n_g,
                                                          int g_idx, int num_paths, int max_paths,
                                                          TileScratch ts, LoopTiles store) {
  expand_body(sd, g, n_g, g_idx, num_paths, max_paths, ts, store);
}


// PUMP.cu:188-218: a new path (not at the goal) dies if a stored path at its
// node, or another new path there that passed the cut-off, epsilon-dominates
// it; co-dominant paths keep the lower path number.  Tested inside the store
// pass, which prepends its survivors to the stored lists meanwhile: the walk
// reads the lists through L2 and skips entries stored in this pass (index
// num_paths or above), so it sees each list as it was when the pass began (a
// survivor is published only after its link is written).
__device__ __forceinline__ bool dominated_in_store(const SearchDev &sd, int i, int node,
                                                   int num_paths, float eps_cp, float eps_cost) {
  const int path_idx = num_paths + i;
  const float cp = sd.new_cp[i], cost = sd.new_cost[i];
  auto dominated_by = [&](float cp_c, float cost_c, int idx_c) {
    if (cp_c < eps_cp + cp && cost_c < eps_cost + cost) {
      if (cp_c + eps_cp >= cp && cost_c + eps_cost >= cost && path_idx < idx_c) return false;
      return true;
    }
    return false;
  };
  for (int c = __ldcg(&sd.node_head[node]); c >= 0; c = __ldcg(&sd.node_next[c])) {
    if (c >= num_paths) continue;
    if (dominated_by(sd.path_cp[c], sd.path_cost[c], c)) return true;
  }
  for (int j = sd.new_head[node]; j >= 0; j = sd.new_next[j])
    if (j != i && dominated_by(sd.new_cp[j], sd.new_cost[j], num_paths + j)) return true;
  return false;
}

// PUMP.cu:188-282 in one pass.  A survivor (alive, not dominated, not at the
// initial node) becomes stored path num_paths + r, r = its rank among the
// survivors in wavefront order, and is appended to bucket b at
// g_base[b] + r_b, r_b = its rank among the survivors of bucket b (the
// reference appends survivors to the buckets in the order it stores them).
// Both ranks come from one stable compaction: a tile's count is the pair
// (survivors, survivors of bucket 1) packed into one word (31 bits each in
// the look-back value, 16 bits each within a tile), so the look-back adds
// both at once.  The last tile writes the survivor count and the bucket
// sizes.  Each survivor also moves its particle mask from the stage.
// A wavefront is typically a few thousand paths, so tiles are small (256
// paths, one per thread, whose dominance walks run side by side) to spread
// it over many blocks, and each thread issues all loads of its path before
// any node-list push or store.
constexpr int kStoreRows = 1;
constexpr int kStoreTile = kCompactThreads * kStoreRows;  // 256 items
constexpr int kStoreWarps = kCompactThreads / 32;
constexpr int kStoreCounts = kStoreRows * kStoreWarps;
static_assert(kStoreCounts <= 32, "one (row, warp) count per lane of the scan");
constexpr unsigned long long kLow31 = (1ull << 31) - 1ull;
static_assert(kLoopStoreTile == kStoreTile, "store tile size");

__device__ __forceinline__ void store_tiles(
    const SearchDev &sd, int num_paths, int g_idx, float cost_threshold, float dr, float cp_min_soln,
    float eps_cp, float eps_cost, const uint32_t *__restrict__ stage, uint32_t *__restrict__ valid,
    int words, const TileScratch &ts) {
  // per (row, warp): survivors | survivors of bucket 1 << 16, then their
  // exclusive offsets within the tile; entry r * kStoreWarps + warp
  __shared__ unsigned int s_cnt[kStoreRows * kStoreWarps];
  __shared__ unsigned long long s_excl;
  __shared__ int s_timeout;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long n = wave_size(sd.ctl);
  const long long ntiles = (n + kStoreTile - 1) / kStoreTile;
  const unsigned int lt = (1u << lane) - 1u;
  // blocks take tiles in order from the counter until none is left
  while (true) {
    const long long tile = next_tile(ts);
    if (tile >= ntiles) return;  // block-uniform
    const long long base = tile * kStoreTile;
    bool surv[kStoreRows];
    int node[kStoreRows];
    float cost[kStoreRows];
#pragma unroll
    for (int r = 0; r < kStoreRows; ++r) {
      const long long i = base + r * kCompactThreads + threadIdx.x;
      uint8_t al = 0;
      node[r] = 0;
      cost[r] = 0.0f;
      if (i < n) {
        al = sd.alive[i];
        node[r] = sd.wf_node[i];
        cost[r] = sd.new_cost[i];
      }
      // dominance is tested only for live paths not at the goal (or at the
      // initial node, which stores nothing)
      bool dead = false;
      if (al && node[r] != sd.goal && node[r] != 0)
        dead = dominated_in_store(sd, (int)i, node[r], num_paths, eps_cp, eps_cost);
      surv[r] = al && !dead && node[r] != 0;
    }
    uint8_t bkt[kStoreRows];
#pragma unroll
    for (int r = 0; r < kStoreRows; ++r) {
      bkt[r] = 0;
      if (surv[r]) {
        float dcost = (cost[r] + sd.h[node[r]] - cost_threshold);
        dcost = (0.0f < dcost) ? dcost : 0.0f;  // std::max((float)0, dCost)
        bkt[r] = (uint8_t)((((int)(dcost / dr)) + g_idx + 1) % 2);
      }
    }
    unsigned int bs[kStoreRows], b1[kStoreRows];
#pragma unroll
    for (int r = 0; r < kStoreRows; ++r) {
      bs[r] = __ballot_sync(0xffffffffu, surv[r]);
      b1[r] = __ballot_sync(0xffffffffu, surv[r] && bkt[r] == 1);
      if (lane == 0)
        s_cnt[r * kStoreWarps + warp] = (unsigned int)__popc(bs[r]) | ((unsigned int)__popc(b1[r]) << 16);
    }
    __syncthreads();
    if (warp == 0) {
      // (row, warp) order is lane order: one warp scan of the packed pairs
      // (each half at most kStoreTile < 2^16, so the halves never carry)
      const unsigned int v = lane < kStoreCounts ? s_cnt[lane] : 0u;
      unsigned int incl = v;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const unsigned int o = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += o;
      }
      if (lane < kStoreCounts) s_cnt[lane] = incl - v;
      const unsigned int tt = __shfl_sync(0xffffffffu, incl, 31);
      const unsigned long long agg =
          (unsigned long long)(tt & 0xFFFFu) | ((unsigned long long)(tt >> 16) << 31);
      bool to = false;
      const unsigned long long ex_tile = lookback_warp(ts, tile, agg, &to);
      if (lane == 0) {
        s_excl = ex_tile;
        s_timeout = to ? 1 : 0;
        if (to) {
          atomicExch(ts.error, 1);
          atomicExch(&sd.ctl->wait_error, 1);
        }
        if (!to && tile == ntiles - 1) {
          const unsigned long long tot = ex_tile + agg;
          const int n_s = (int)(tot & kLow31), n_1 = (int)(tot >> 31);
          *ts.total = (unsigned long long)n_s;
          SearchCtl *c = sd.ctl;
          c->num_valid = (unsigned long long)n_s;
          c->g_count[0] = c->g_base[0] + (n_s - n_1);
          c->g_count[1] = c->g_base[1] + n_1;
        }
      }
    }
    __syncthreads();
    if (s_timeout) return;  // block-uniform
    const long long ex_s = (long long)(s_excl & kLow31), ex_1 = (long long)(s_excl >> 31);
    const int gb0 = sd.ctl->g_base[0], gb1 = sd.ctl->g_base[1];
    // loads of every survivor row first
    int st[kStoreRows], slot[kStoreRows], prev[kStoreRows];
    float tm[kStoreRows], cp[kStoreRows];
    uint4 mk[kStoreRows];
#pragma unroll
    for (int r = 0; r < kStoreRows; ++r) {
      st[r] = slot[r] = prev[r] = 0;
      tm[r] = cp[r] = 0.0f;
      mk[r] = make_uint4(0u, 0u, 0u, 0u);
      if (!surv[r]) continue;
      const long long i = base + r * kCompactThreads + threadIdx.x;
      const unsigned int in_tile = s_cnt[r * kStoreWarps + warp];
      const long long rank = ex_s + (in_tile & 0xFFFFu) + __popc(bs[r] & lt);
      const long long rank1 = ex_1 + (in_tile >> 16) + __popc(b1[r] & lt);
      st[r] = num_paths + (int)rank;
      slot[r] = bkt[r] == 1 ? gb1 + (int)rank1 : gb0 + (int)(rank - rank1);
      prev[r] = sd.wf_prev[i];
      tm[r] = sd.new_time[i];
      cp[r] = sd.new_cp[i];
      if (words == 4) mk[r] = reinterpret_cast<const uint4 *>(stage)[i];
    }
    // then the survivors pushed onto their nodes' stored lists: the link is
    // written (through L2) before the entry is published, so a concurrent
    // dominance walk never follows an unset link; and the nodes reached for
    // the first time listed for their edge checks (the thread that moves a
    // node's count from -1 to 0 lists it)
#pragma unroll
    for (int r = 0; r < kStoreRows; ++r) {
      if (!surv[r]) continue;
      int h = __ldcg(&sd.node_head[node[r]]);
      while (true) {
        __stcg(&sd.node_next[st[r]], h);
        __threadfence();
        const int seen = atomicCAS(&sd.node_head[node[r]], h, st[r]);
        if (seen == h) break;
        h = seen;
      }
    }
#pragma unroll
    for (int r = 0; r < kStoreRows; ++r)
      if (surv[r] && sd.open_cnt[node[r]] == -1 && atomicCAS(&sd.open_cnt[node[r]], -1, 0) == -1)
        sd.todo[atomicAdd(&sd.ctl->todo, 1)] = node[r];
    // then the stores
#pragma unroll
    for (int r = 0; r < kStoreRows; ++r) {
      if (!surv[r]) continue;
      const int p = st[r];
      sd.path_prev[p] = prev[r];
      sd.path_node[p] = node[r];
      sd.path_cost[p] = cost[r];
      sd.path_time[p] = tm[r];
      sd.path_cp[p] = cp[r];
      (bkt[r] == 1 ? sd.g_list[1] : sd.g_list[0])[slot[r]] = p;
      if (node[r] == sd.goal && cp[r] <= cp_min_soln) atomicOr(&sd.ctl->goal_found, 1);
      uint32_t *dst = valid + (long long)p * words;
      if (words == 4) {
        *reinterpret_cast<uint4 *>(dst) = mk[r];
      } else {
        const long long i = base + r * kCompactThreads + threadIdx.x;
        const uint32_t *src = stage + i * words;
        for (int q = 0; q < words; ++q) dst[q] = src[q];
      }
    }
    __syncthreads();  // s_cnt, s_excl and the tile index are reused by the next tile
  }
}

__device__ __forceinline__ void store_body(
    const SearchDev &sd, int num_paths, int g_idx, float cost_threshold, float dr, float cp_min_soln,
    float eps_cp, float eps_cost, const uint32_t *__restrict__ stage, uint32_t *__restrict__ valid,
    int words, const TileScratch &ts, unsigned int *done, SearchCtl *host_ctl, unsigned int seq) {
  store_tiles(sd, num_paths, g_idx, cost_threshold, dr, cp_min_soln, eps_cp, eps_cost, stage, valid,
              words, ts);
  if (!host_ctl) return;
  // the last block to finish copies the counters to the host
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(done, 1u) == gridDim.x - 1) {
      __threadfence();
      const volatile SearchCtl *c = sd.ctl;
      host_ctl->num_new = c->num_new;
      host_ctl->num_valid = c->num_valid;
      host_ctl->g_count[0] = c->g_count[0];
      host_ctl->g_count[1] = c->g_count[1];
      host_ctl->goal_found = c->goal_found;
      host_ctl->g_base[0] = c->g_base[0];
      host_ctl->g_base[1] = c->g_base[1];
      host_ctl->wait_error = c->wait_error;
      host_ctl->overflow = c->overflow;
      host_ctl->todo = c->todo;
      __threadfence_system();
      *reinterpret_cast<volatile unsigned int *>(&host_ctl->seq) = seq;
    }
  }
}

__global__ void __launch_bounds__(kCompactThreads) store_kernel(
    SearchDev sd, int num_paths, int g_idx, float cost_threshold, float dr, float cp_min_soln,
    float eps_cp, float eps_cost, const uint32_t *__restrict__ stage, uint32_t *__restrict__ valid,
    int words, TileScratch ts, unsigned int *done, SearchCtl *host_ctl, unsigned int seq,
    LoopTiles scan) {
  zero_tiles(scan);  // for the next iteration's expansion
  store_body(sd, num_paths, g_idx, cost_threshold, dr, cp_min_soln, eps_cp, eps_cost, stage, valid,
             words, ts, done, host_ctl, seq);
}

// ------------------------------------------- the search loop on the device
// Graph form of the loop: every kernel reads its arguments from its query's
// LoopArgs block (blockIdx.y of the group); the per-iteration values come
// from the loop state, which the control step updates after each iteration.

// The argument block of this block's query, or null when the block has no
// query or the query's loop has ended (block-uniform).
__device__ __forceinline__ LoopArgs *loop_query(const LoopGroup *g) {
  if ((int)blockIdx.y >= g->nq) return nullptr;
  LoopArgs *a = g->args[blockIdx.y];
  return *reinterpret_cast<const volatile int *>(&a->L.active) ? a : nullptr;
}

__device__ __forceinline__ TileScratch tiles_of(const LoopTiles &t) {
  TileScratch ts{};
  ts.status = t.status;
  ts.tile_counter = t.tile_counter;
  ts.total = t.total;
  ts.error = t.error;
  return ts;
}

// search_init_kernel, the particle-table error word and path 0's particle
// mask (all P particles valid), per query of the group.
__global__ void loop_init_kernel(LoopGroup *g) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) g->store_done = 0u;
  if ((int)blockIdx.y >= g->nq) return;
  const LoopArgs *a = g->args[blockIdx.y];
  const SearchDev sd = a->sd;
  search_init_body(sd);
  if (blockIdx.x == 0 && threadIdx.x == 0) *a->err = 0;
  {  // the first iteration's tile scratch
    const long long na = loop_tile_words(a->scan.cap), nb = loop_tile_words(a->store.cap);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < na + nb; i += stride) {
      if (i < na) a->scan.total[i] = 0ull;
      else a->store.total[i - na] = 0ull;
    }
  }
  const int words = a->words, P = a->P;
  uint32_t *valid = a->valid;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < words; q += gridDim.x * blockDim.x) {
    const int rem = P - q * 32;
    valid[q] = rem >= 32 ? 0xFFFFFFFFu : ((1u << rem) - 1u);
  }
}

// search_init_head_kernel, then the while node's first iteration (one block
// per query).
__global__ void loop_arm_kernel(LoopGroup *g, cudaGraphConditionalHandle h) {
  if ((int)blockIdx.y < g->nq) {
    LoopArgs *a = g->args[blockIdx.y];
    a->sd.node_head[0] = 0;
    a->L.active = 1;
  }
  if (blockIdx.y == 0) cudaGraphSetConditional(h, g->nq > 0 ? 1u : 0u);
}

template <int Mode>
__global__ void __launch_bounds__(kChkThreads, 4) check_loop_kernel(const LoopGroup *g) {
  const LoopArgs *a = loop_query(g);
  if (!a) return;
  const SearchDev sd = a->sd;
  const CheckArgs ca = a->ca;
  check_body<Mode, false>(sd, ca);
}

__global__ void __launch_bounds__(kExpThreads, 1) expand_loop_kernel(const LoopGroup *g) {
  const LoopArgs *a = loop_query(g);
  if (!a) return;
  const SearchDev &sd = a->sd;  // fields read from the argument block as used
  const int g_idx = a->L.g_idx;
  const TileScratch ts = tiles_of(a->scan);
  expand_body(sd, g_idx ? sd.g_list[1] : sd.g_list[0], a->L.n_g, g_idx, a->L.num_paths,
              a->L.max_paths, ts, a->store);
}


// The host loop's bookkeeping after an iteration's counters are back
// (PUMP.cu:259-288), then whether the query's loop goes on; run by the
// store pass's last block of the query to finish.  A guard ends the loop
// after 64 iterations whatever the state says.
__device__ void loop_control(LoopArgs *a) {
  LoopState &L = a->L;
  SearchCtl c;
  {  // written by other blocks of this iteration's kernels
    const volatile SearchCtl *v = a->sd.ctl;
    c.num_new = v->num_new;
    c.num_valid = v->num_valid;
    c.g_count[0] = v->g_count[0];
    c.g_count[1] = v->g_count[1];
    c.goal_found = v->goal_found;
    c.wait_error = v->wait_error;
    c.overflow = v->overflow;
  }
  const int scan_error = *reinterpret_cast<const volatile int *>(a->scan.error);
  int cont = 0;
  ++L.guard;
  if (c.overflow == 1) {
    L.status = kLoopWavefrontOverflow;
  } else {
    const int num_new = (int)c.num_new;
    if (L.itrs <= 32) L.wavefront_sizes[L.itrs - 1] = num_new;
    if (num_new == 0) {
    } else if (c.overflow == 2) {
      L.status = kLoopPathsWouldOverflow;
    } else {
      L.considered += num_new;
      if (c.wait_error || scan_error) {
        L.status = kLoopWaitError;
      } else {
        L.num_paths += (int)c.num_valid;
        L.g_count[0] = c.g_count[0];
        L.g_count[1] = c.g_count[1];
        if (!c.goal_found && !(c.g_count[0] == 0 && c.g_count[1] == 0)) {
          L.g_idx = (L.g_idx + 1) % 2;
          L.cost_threshold += L.dr;
          if (L.num_paths >= L.max_paths) {
            L.status = kLoopPathsFull;
          } else if (L.itrs < L.max_itrs) {
            ++L.itrs;
            L.n_g = L.g_count[L.g_idx];
            if (L.n_g == 0) {
              if (L.itrs <= 32) L.wavefront_sizes[L.itrs - 1] = 0;
            } else {
              cont = 1;
            }
          }
        }
      }
    }
  }
  if (L.guard >= 64) cont = 0;
  L.active = cont;
}

__global__ void __launch_bounds__(kCompactThreads, 2) store_loop_kernel(
    LoopGroup *g, cudaGraphConditionalHandle h) {
  __shared__ bool s_last;
  LoopArgs *a = loop_query(g);
  if (a) {
    const SearchDev sd = a->sd;
    const TileScratch ts = tiles_of(a->store);
    zero_tiles(a->scan);  // for the next iteration's expansion
    store_tiles(sd, a->L.num_paths, a->L.g_idx, a->L.cost_threshold, a->L.dr, a->cp_min_soln,
                a->eps_cp, a->eps_cost, a->stage, a->valid, a->words, ts);
    // the query's last block to finish runs its control step
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      s_last = atomicAdd(a->store.done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
      __threadfence();
      loop_control(a);
    }
  }
  // the launch's last block to finish (every query's control step is done)
  // sets the while node's condition: another iteration while any query goes on
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&g->store_done, 1u) == gridDim.x * gridDim.y - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    unsigned int any = 0u;
    for (int q = 0; q < g->nq; ++q)
      any |= *reinterpret_cast<const volatile int *>(&g->args[q]->L.active) ? 1u : 0u;
    g->store_done = 0u;
    cudaGraphSetConditional(h, any);
  }
}


}  // namespace

pump_status_t search_init(const SearchDev &sd, cudaStream_t s) {
  search_init_kernel<<<grid_for(sd.N, 256), 256, 0, s>>>(sd);
  PUMP_TRY(launch_status("search_init"));
  search_init_head_kernel<<<1, 1, 0, s>>>(sd);
  return launch_status("search_init_head");
}

pump_status_t search_check(const SearchDev &sd, int max_todo, const CheckArgs &ca, cudaStream_t s) {
  if (max_todo <= 0) return PUMP_OK;
  // the wide form when its items alone fill the GPU twice over (and its
  // stage fits): few listed nodes keep the narrow form's short chains
  const long long wide_items =
      (long long)max_todo * ((ca.max_degree + kChkWideEdges - 1) / kChkWideEdges);
  const bool wide = wide_items >= 2LL * kNumSMs && ca.numObs <= 0xFFFF &&
                    check_smem(ca.numObs, ca.numDisc, true) <= 200 * 1024;
  const size_t smem = check_smem(ca.numObs, ca.numDisc, wide);
  if (smem > 220 * 1024)
    return set_error(PUMP_ERR_CAPACITY, "%d obstacles and %d waypoints exceed the check stage",
                     ca.numObs, ca.numDisc + 1);
  // at most one block per (listed node, chunk), no more than the GPU holds
  const int edges = wide ? kChkWideEdges : kChkEdges;
  const long long chunks = ca.max_degree > edges ? (ca.max_degree + edges - 1) / edges : 1;
  const long long want = (long long)max_todo * chunks;
  const unsigned blocks = (unsigned)(want < kNumSMs * 8 ? want : kNumSMs * 8);
  const void *fn = ca.mode == PUMP_BVP_PARITY
                       ? (wide ? (const void *)check_kernel<PUMP_BVP_PARITY, true>
                               : (const void *)check_kernel<PUMP_BVP_PARITY, false>)
                       : (wide ? (const void *)check_kernel<PUMP_BVP_PRECISION, true>
                               : (const void *)check_kernel<PUMP_BVP_PRECISION, false>);
  PUMP_TRY(smem_attr(fn, smem));
  if (ca.mode == PUMP_BVP_PARITY) {
    if (wide) check_kernel<PUMP_BVP_PARITY, true><<<blocks, kChkThreads, smem, s>>>(sd, ca);
    else check_kernel<PUMP_BVP_PARITY, false><<<blocks, kChkThreads, smem, s>>>(sd, ca);
  } else {
    if (wide) check_kernel<PUMP_BVP_PRECISION, true><<<blocks, kChkThreads, smem, s>>>(sd, ca);
    else check_kernel<PUMP_BVP_PRECISION, false><<<blocks, kChkThreads, smem, s>>>(sd, ca);
  }
  return launch_status("check_kernel");
}

pump_status_t search_count_open(const SearchDev &sd, cudaStream_t s) {
  long long blocks = ((long long)sd.N * 32 + 255) / 256;
  if (blocks > kNumSMs * 16) blocks = kNumSMs * 16;
  count_open_kernel<<<(unsigned)(blocks > 0 ? blocks : 1), 256, 0, s>>>(sd);
  return launch_status("count_open_kernel");
}

pump_status_t max_degree_async(const int *d_go, int N, int *d_out, cudaStream_t s) {
  max_degree_kernel<<<1, 1024, 0, s>>>(d_go, N, d_out);
  return launch_status("max_degree_kernel");
}

pump_status_t search_expand(const SearchDev &sd, int g_idx, int n_g, int num_paths, int max_paths,
                           const LoopTiles &scan, const LoopTiles &store, cudaStream_t s) {
  if (n_g <= 0) return PUMP_OK;
  TileScratch ts{};
  ts.status = scan.status;
  ts.tile_counter = scan.tile_counter;
  ts.total = scan.total;
  ts.error = scan.error;
  const long long ntiles = ((long long)n_g + kExpTile - 1) / kExpTile;
  if (ntiles > scan.cap) return set_error(PUMP_ERR_CAPACITY, "expansion: %lld tiles", ntiles);
  const unsigned blocks = (unsigned)(ntiles < kNumSMs * 2 ? ntiles : kNumSMs * 2);
  expand_kernel<<<blocks, kExpThreads, 0, s>>>(sd, sd.g_list[g_idx], n_g, g_idx, num_paths,
                                               max_paths, ts, store);
  return launch_status("expand_kernel");
}

HsmcEpilogue search_hsmc_epilogue(const SearchDev &sd, float cp_cutoff) {
  HsmcEpilogue e{};
  e.wf_open = sd.wf_open;
  e.wf_node = sd.wf_node;
  e.path_time = sd.path_time;
  e.path_cost = sd.path_cost;
  e.topt = sd.topt;
  e.copt = sd.copt;
  e.new_time = sd.new_time;
  e.new_cost = sd.new_cost;
  e.alive = sd.alive;
  e.new_head = sd.new_head;
  e.new_next = sd.new_next;
  e.cp_cutoff = cp_cutoff;
  return e;
}


pump_status_t search_store(const SearchDev &sd, int max_new, int num_paths, int g_idx,
                           float cost_threshold, float dr, float cp_min_soln, float eps_cp,
                           float eps_cost, const uint32_t *stage,
                           uint32_t *valid, int words, const LoopTiles &store,
                           const LoopTiles &scan, SearchCtl *host_ctl, unsigned int seq,
                           cudaStream_t s) {
  TileScratch ts{};
  ts.status = store.status;
  ts.tile_counter = store.tile_counter;
  ts.total = store.total;
  ts.error = store.error;
  const long long ntiles = ((long long)(max_new > 0 ? max_new : 1) + kStoreTile - 1) / kStoreTile;
  if (ntiles > store.cap) return set_error(PUMP_ERR_CAPACITY, "store pass: %lld tiles", ntiles);
  const unsigned blocks = (unsigned)(ntiles < kNumSMs * 4 ? ntiles : kNumSMs * 4);
  store_kernel<<<blocks, kCompactThreads, 0, s>>>(sd, num_paths, g_idx, cost_threshold, dr,
                                                  cp_min_soln, eps_cp, eps_cost, stage, valid,
                                                  words, ts, store.done, host_ctl, seq, scan);
  return launch_status("store_kernel");
}

pump_status_t search_loop_graph(LoopGroup *d_group, int gcap, bool lazy, int mode, int numObs,
                                int numDisc, int maxHS, int P, cudaStream_t capture_stream,
                                cudaGraphExec_t *out) {
  *out = nullptr;
  if (gcap < 1 || gcap > kLoopGroupMax)
    return set_error(PUMP_ERR_BAD_INPUT, "search loop graph: %d queries per group", gcap);
  const size_t chk_smem = check_smem(numObs, numDisc, false);
  if (chk_smem > 220 * 1024)
    return set_error(PUMP_ERR_CAPACITY, "%d obstacles and %d waypoints exceed the check stage",
                     numObs, numDisc + 1);
  const void *chk = mode == PUMP_BVP_PARITY ? (const void *)check_loop_kernel<PUMP_BVP_PARITY>
                                            : (const void *)check_loop_kernel<PUMP_BVP_PRECISION>;
  if (lazy) PUMP_TRY(smem_attr(chk, chk_smem));
  PUMP_TRY(hsmc_loop_prepare(numObs, numDisc + 1, maxHS, P));
  // each query's share of a kernel's grid (the whole grid for one query)
  auto share = [gcap](int whole, int least) {
    const int b = whole / gcap;
    return (unsigned)(b > least ? b : least);
  };
  cudaGraph_t g = nullptr;
  PUMP_CUDA_TRY(cudaGraphCreate(&g, 0));
  // the while node's condition starts at 0 and is set by the arm kernel
  // upstream of it, so the body runs only if the device sets it
  pump_status_t st = PUMP_OK;
  cudaGraphConditionalHandle h{};
  cudaGraphNode_t n_init = nullptr, n_arm = nullptr, n_loop = nullptr;
  cudaGraphNodeParams cp{};
  st = cuda_status(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault),
                   "cudaGraphConditionalHandleCreate");
  if (st == PUMP_OK) {
    cudaKernelNodeParams kp{};
    void *init_args[1] = {&d_group};
    kp.func = (void *)loop_init_kernel;
    kp.gridDim = dim3(share(kNumSMs * 2, 2), gcap);
    kp.blockDim = dim3(256);
    kp.kernelParams = init_args;
    st = cuda_status(cudaGraphAddKernelNode(&n_init, g, nullptr, 0, &kp), "cudaGraphAddKernelNode");
  }
  if (st == PUMP_OK) {
    cudaKernelNodeParams kp{};
    void *arm_args[2] = {&d_group, &h};
    kp.func = (void *)loop_arm_kernel;
    kp.gridDim = dim3(1, gcap);
    kp.blockDim = dim3(1);
    kp.kernelParams = arm_args;
    st = cuda_status(cudaGraphAddKernelNode(&n_arm, g, &n_init, 1, &kp), "cudaGraphAddKernelNode");
  }
  if (st == PUMP_OK) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    st = cuda_status(cudaGraphAddNode(&n_loop, g, &n_arm, nullptr, 1, &cp), "cudaGraphAddNode");
  }
  if (st == PUMP_OK) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t cs = capture_stream;
    st = cuda_status(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                                   cudaStreamCaptureModeRelaxed),
                     "cudaStreamBeginCaptureToGraph");
    if (st == PUMP_OK) {
      // fixed grids (the kernels loop over the device-side counts)
      const int g_check = kNumSMs * 8, g_wide = kNumSMs * 4;
      if (lazy) {
        const dim3 gd(share(g_check, 8), gcap);
        if (mode == PUMP_BVP_PARITY)
          check_loop_kernel<PUMP_BVP_PARITY><<<gd, kChkThreads, chk_smem, cs>>>(d_group);
        else
          check_loop_kernel<PUMP_BVP_PRECISION><<<gd, kChkThreads, chk_smem, cs>>>(d_group);
      }
      expand_loop_kernel<<<dim3(share(kNumSMs * 2, 2), gcap), kExpThreads, 0, cs>>>(d_group);
      // HSMC's blocks are half as wide (4 warps): twice as many per SM; its
      // grid is not split (blocks take chunks of every query's wavefront)
      hsmc_loop_launch(d_group, numObs, numDisc + 1, maxHS, P, 2 * g_wide, cs);
      store_loop_kernel<<<dim3(share(g_wide, 4), gcap), kCompactThreads, 0, cs>>>(d_group, h);
      cudaGraph_t captured = nullptr;
      const pump_status_t ce = cuda_status(cudaStreamEndCapture(cs, &captured), "cudaStreamEndCapture");
      st = ce == PUMP_OK ? launch_status("search loop capture") : ce;
    }
  }
  if (st == PUMP_OK) st = cuda_status(cudaGraphInstantiate(out, g, 0), "cudaGraphInstantiate");
  cudaGraphDestroy(g);
  return st;
}

}  // namespace pump
