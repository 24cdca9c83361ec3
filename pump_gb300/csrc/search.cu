// Device-resident exploration: the steps of one iteration of the reference's
// search loop (PUMP.cu:39-290) as kernels over device state.  Paths are
// numbered, stored and bucketed exactly as the host loop numbers them:
// expansion follows the bucket order and each node's edge order (an
// exclusive scan of out-degrees), survivors keep wavefront order (stable
// compaction), and bucket appends keep survivor order.  Dominance only asks
// whether some path dominates, so the per-node lists it walks may be in any
// order.
#include "search.h"

#include "common.cuh"
#include "compact.cuh"
#include "ctx.h"

namespace pump {
namespace {

__global__ void search_init_kernel(SearchDev sd) {
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
  }
}

// node_head[0] = path 0 after the per-node reset (separate launch: the
// reset above is grid-strided).
__global__ void search_init_head_kernel(SearchDev sd) { sd.node_head[0] = 0; }

struct ExpandCount {
  const int *g, *path_node, *fgo;
  __device__ unsigned int operator()(long long i) const {
    const int node = path_node[g[i]];
    return (unsigned int)(fgo[node + 1] - fgo[node]);
  }
};

// One warp per bucket entry: its node's expandable edges in order.  The
// wavefront's nodes get empty lists of new paths; thread 0 empties bucket
// g_idx and records the bucket sizes the store pass appends after (the
// expansion reads the bucket through n_g, not through its count).
__global__ void expand_write_kernel(SearchDev sd, const int *g, int n_g, int g_idx,
                                    int num_paths, int max_paths) {
  const unsigned long long nn = sd.ctl->num_new;
  const int ovf = nn > (unsigned long long)max_paths
                      ? 1
                      : ((unsigned long long)num_paths + nn >= (unsigned long long)max_paths ? 2 : 0);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    SearchCtl *c = sd.ctl;
    c->g_count[g_idx] = 0;
    c->g_base[g_idx] = 0;
    c->g_base[1 - g_idx] = c->g_count[1 - g_idx];
    c->num_valid = 0;
    c->overflow = ovf;
  }
  if (ovf) return;
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  for (long long k = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / 32; k < n_g; k += warps) {
    const int prev = g[k];
    const int node = sd.path_node[prev];
    const int f0 = sd.fgo[node], cnt = sd.fgo[node + 1] - f0;
    const unsigned int off = sd.wf_off[k];
    for (int q = lane; q < cnt; q += 32) {
      const int f = f0 + q;
      const int dst = sd.fdst[f];
      sd.wf_prev[off + q] = prev;
      sd.wf_node[off + q] = dst;
      sd.wf_edge[off + q] = sd.fid[f];
      sd.wf_open[off + q] = f;
      sd.new_head[dst] = -1;
    }
  }
}

// PUMP.cu:164-185: time and cost of the new paths and the CP cut-off; the
// survivors of the cut-off are linked into their node's list of new paths
// (emptied by the expansion kernel).
__global__ void new_paths_kernel(SearchDev sd, float cp_cutoff) {
  const int n = wave_size(sd.ctl);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int prev = sd.wf_prev[i], f = sd.wf_open[i];
    sd.new_time[i] = sd.path_time[prev] + sd.ftopt[f];
    sd.new_cost[i] = sd.path_cost[prev] + sd.fcopt[f];
    const bool alive = !(sd.new_cp[i] > cp_cutoff);
    sd.alive[i] = alive ? 1 : 0;
    if (alive) sd.new_next[i] = atomicExch(&sd.new_head[sd.wf_node[i]], i);
  }
}

// PUMP.cu:188-218: a new path (not at the goal) dies if a stored path at its
// node, or another new path there that passed the cut-off, epsilon-dominates
// it; co-dominant paths keep the lower path number.
__device__ void dominance_one(SearchDev sd, int i, int num_paths, float eps_cp, float eps_cost) {
  const int node = sd.wf_node[i];
  uint8_t dead = 0;
  if (sd.alive[i] && node != sd.goal) {
    const int path_idx = num_paths + i;
    const float cp = sd.new_cp[i], cost = sd.new_cost[i];
    auto dominated_by = [&](float cp_c, float cost_c, int idx_c) {
      if (cp_c < eps_cp + cp && cost_c < eps_cost + cost) {
        if (cp_c + eps_cp >= cp && cost_c + eps_cost >= cost && path_idx < idx_c) return false;
        return true;
      }
      return false;
    };
    for (int c = sd.node_head[node]; c >= 0 && !dead; c = sd.node_next[c])
      if (dominated_by(sd.path_cp[c], sd.path_cost[c], c)) dead = 1;
    for (int j = sd.new_head[node]; j >= 0 && !dead; j = sd.new_next[j])
      if (j != i && dominated_by(sd.new_cp[j], sd.new_cost[j], num_paths + j)) dead = 1;
  }
  sd.dominated[i] = dead;
}

__global__ void dominance_kernel(SearchDev sd, int num_paths, float eps_cp, float eps_cost) {
  const int n = wave_size(sd.ctl);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    dominance_one(sd, i, num_paths, eps_cp, eps_cost);
}

// PUMP.cu:221-282 in one pass.  A survivor (alive, not dominated, not at the
// initial node) becomes stored path num_paths + r, r = its rank among the
// survivors in wavefront order, and is appended to bucket b at
// g_base[b] + r_b, r_b = its rank among the survivors of bucket b (the
// reference appends survivors to the buckets in the order it stores them).
// Both ranks come from one stable compaction: a tile's count is the pair
// (survivors, survivors of bucket 1) packed into one word (31 bits each in
// the look-back value, 16 bits each within a tile), so the look-back adds
// both at once.  The last tile writes the survivor count and the bucket
// sizes.  Each survivor also moves its particle mask from the stage.
constexpr unsigned long long kLow31 = (1ull << 31) - 1ull;

__global__ void __launch_bounds__(kCompactThreads) store_kernel(
    SearchDev sd, int num_paths, int g_idx, float cost_threshold, float dr, float cp_min_soln,
    const uint32_t *__restrict__ stage, uint32_t *__restrict__ valid, int words, TileScratch ts) {
  __shared__ TileShared sh;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long n = wave_size(sd.ctl);
  const long long ntiles = (n + kTile - 1) / kTile;
  const unsigned int lt = (1u << lane) - 1u;
  // blocks take tiles in order from the counter until none is left
  while (true) {
    const long long tile = next_tile(ts);
    if (tile >= ntiles) return;  // block-uniform
    const long long base = tile * kTile;
    bool surv[kCompactRows];
    uint8_t bkt[kCompactRows];
#pragma unroll
    for (int r = 0; r < kCompactRows; ++r) {
      const long long i = base + r * kCompactThreads + threadIdx.x;
      surv[r] = false;
      bkt[r] = 0;
      if (i < n && sd.alive[i] && !sd.dominated[i]) {
        const int node = sd.wf_node[i];
        if (node != 0) {
          surv[r] = true;
          float dcost = (sd.new_cost[i] + sd.h[node] - cost_threshold);
          dcost = (0.0f < dcost) ? dcost : 0.0f;  // std::max((float)0, dCost)
          bkt[r] = (uint8_t)((((int)(dcost / dr)) + g_idx + 1) % 2);
        }
      }
    }
    unsigned int bs[kCompactRows], b1[kCompactRows];
#pragma unroll
    for (int r = 0; r < kCompactRows; ++r) {
      bs[r] = __ballot_sync(0xffffffffu, surv[r]);
      b1[r] = __ballot_sync(0xffffffffu, surv[r] && bkt[r] == 1);
      if (lane == 0)
        sh.cnt[r][warp] = (unsigned int)__popc(bs[r]) | ((unsigned int)__popc(b1[r]) << 16);
    }
    // in-tile offsets of both counts (each at most kTile < 2^16), then the
    // tile's pair in the look-back's packing
    __syncthreads();
    if (warp == 0) {
      const unsigned int tt = scan_tile_counts(sh.cnt);
      const unsigned long long agg =
          (unsigned long long)(tt & 0xFFFFu) | ((unsigned long long)(tt >> 16) << 31);
      bool to = false;
      const unsigned long long ex_tile = lookback_warp(ts, tile, agg, &to);
      if (lane == 0) {
        sh.excl = ex_tile;
        sh.timeout = to;
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
    if (sh.timeout) return;
    const long long ex_s = (long long)(sh.excl & kLow31), ex_1 = (long long)(sh.excl >> 31);
    const int gb0 = sd.ctl->g_base[0], gb1 = sd.ctl->g_base[1];
#pragma unroll
    for (int r = 0; r < kCompactRows; ++r) {
      if (!(bs[r] & (1u << lane))) continue;
      const long long i = base + r * kCompactThreads + threadIdx.x;
      const unsigned int in_tile = sh.cnt[r][warp];
      const long long rank = ex_s + (in_tile & 0xFFFFu) + __popc(bs[r] & lt);
      const long long rank1 = ex_1 + (in_tile >> 16) + __popc(b1[r] & lt);
      const int st = num_paths + (int)rank;
      const int node = sd.wf_node[i];
      const float cp = sd.new_cp[i];
      sd.path_prev[st] = sd.wf_prev[i];
      sd.path_node[st] = node;
      sd.path_cost[st] = sd.new_cost[i];
      sd.path_time[st] = sd.new_time[i];
      sd.path_cp[st] = cp;
      if (bkt[r] == 1) sd.g_list[1][gb1 + (int)rank1] = st;
      else sd.g_list[0][gb0 + (int)(rank - rank1)] = st;
      sd.node_next[st] = atomicExch(&sd.node_head[node], st);
      if (node == sd.goal && cp <= cp_min_soln) atomicOr(&sd.ctl->goal_found, 1);
      const uint32_t *src = stage + i * words;
      uint32_t *dst = valid + (long long)st * words;
      if ((words & 3) == 0) {
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
        for (int q = 0; q < words / 4; ++q) d4[q] = s4[q];
      } else {
        for (int q = 0; q < words; ++q) dst[q] = src[q];
      }
    }
    __syncthreads();  // sh and the tile index are reused by the next tile
  }
}

}  // namespace

pump_status_t search_init(const SearchDev &sd, cudaStream_t s) {
  search_init_kernel<<<grid_for(sd.N, 256), 256, 0, s>>>(sd);
  PUMP_TRY(launch_status("search_init"));
  search_init_head_kernel<<<1, 1, 0, s>>>(sd);
  return launch_status("search_init_head");
}

pump_status_t search_expand_scan(Ctx *ctx, const SearchDev &sd, int g_idx, int n_g,
                                 cudaStream_t s) {
  TileScratch ts{};
  return run_scan(ctx, n_g, ExpandCount{sd.g_list[g_idx], sd.path_node, sd.fgo}, sd.wf_off, s, &ts,
                  &sd.ctl->num_new);
}

pump_status_t search_expand_write(const SearchDev &sd, int g_idx, int n_g, int num_paths,
                                  int max_paths, cudaStream_t s) {
  const long long threads = (long long)(n_g > 0 ? n_g : 1) * 32;
  long long blocks = (threads + 255) / 256;
  if (blocks > kNumSMs * 16) blocks = kNumSMs * 16;
  expand_write_kernel<<<(unsigned)blocks, 256, 0, s>>>(sd, sd.g_list[g_idx], n_g, g_idx, num_paths,
                                                      max_paths);
  return launch_status("expand_write");
}

pump_status_t search_prune(const SearchDev &sd, int num_paths, float cp_cutoff, float eps_cp,
                           float eps_cost, cudaStream_t s) {
  new_paths_kernel<<<kNumSMs * 4, 256, 0, s>>>(sd, cp_cutoff);
  PUMP_TRY(launch_status("new_paths"));
  dominance_kernel<<<kNumSMs * 4, 256, 0, s>>>(sd, num_paths, eps_cp, eps_cost);
  return launch_status("dominance");
}

pump_status_t search_store(Ctx *ctx, const SearchDev &sd, int max_new, int num_paths,
                           int g_idx, float cost_threshold, float dr, float cp_min_soln,
                           const uint32_t *stage, uint32_t *valid, int words, cudaStream_t s) {
  TileScratch ts{};
  long long ntiles = 0;
  PUMP_TRY(prepare_tiles(ctx, max_new > 0 ? max_new : 1, s, &ts, &ntiles));
  const unsigned blocks = (unsigned)(ntiles < kNumSMs * 4 ? ntiles : kNumSMs * 4);
  store_kernel<<<blocks, kCompactThreads, 0, s>>>(sd, num_paths, g_idx, cost_threshold, dr,
                                                  cp_min_soln, stage, valid, words, ts);
  return launch_status("store_kernel");
}

}  // namespace pump
