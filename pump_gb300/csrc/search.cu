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

__global__ void copy_total_kernel(const unsigned long long *total, unsigned long long *dst) {
  *dst = *total;
}

// One warp per bucket entry: its node's expandable edges in order.
__global__ void expand_write_kernel(SearchDev sd, const int *g, int n_g) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  for (long long k = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / 32; k < n_g; k += warps) {
    const int prev = g[k];
    const int node = sd.path_node[prev];
    const int f0 = sd.fgo[node], cnt = sd.fgo[node + 1] - f0;
    const unsigned int off = sd.wf_off[k];
    for (int q = lane; q < cnt; q += 32) {
      const int f = f0 + q;
      sd.wf_prev[off + q] = prev;
      sd.wf_node[off + q] = sd.fdst[f];
      sd.wf_edge[off + q] = sd.fid[f];
      sd.wf_open[off + q] = f;
    }
  }
}

__global__ void clear_bucket_kernel(SearchCtl *ctl, int g_idx) { ctl->g_count[g_idx] = 0; }

// PUMP.cu:164-185: time and cost of the new paths, the CP cut-off, and a
// reset of the per-node lists of new paths.
__global__ void new_paths_kernel(SearchDev sd, int num_new, float cp_cutoff) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= num_new) return;
  const int prev = sd.wf_prev[i], f = sd.wf_open[i];
  sd.new_time[i] = sd.path_time[prev] + sd.ftopt[f];
  sd.new_cost[i] = sd.path_cost[prev] + sd.fcopt[f];
  sd.alive[i] = sd.new_cp[i] > cp_cutoff ? 0 : 1;
  sd.new_head[sd.wf_node[i]] = -1;
}

__global__ void link_new_kernel(SearchDev sd, int num_new) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= num_new || !sd.alive[i]) return;
  sd.new_next[i] = atomicExch(&sd.new_head[sd.wf_node[i]], i);
}

// PUMP.cu:188-218: a new path (not at the goal) dies if a stored path at its
// node, or another new path there that passed the cut-off, epsilon-dominates
// it; co-dominant paths keep the lower path number.
__global__ void dominance_kernel(SearchDev sd, int num_new, int num_paths, float eps_cp,
                                 float eps_cost) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= num_new) return;
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

// PUMP.cu:221-256: survivors (alive, not dominated, not at the initial
// node) become stored paths num_paths + rank.
struct StorePred {
  SearchDev sd;
  __device__ bool operator()(long long i) const {
    return sd.alive[i] && !sd.dominated[i] && sd.wf_node[i] != 0;
  }
};
struct StoreEmit {
  SearchDev sd;
  int num_paths, g_idx;
  float cost_threshold, dr, cp_min_soln;
  __device__ void operator()(long long i, long long rank) const {
    const int st = num_paths + (int)rank;
    const int node = sd.wf_node[i];
    const float cost = sd.new_cost[i], cp = sd.new_cp[i];
    sd.path_prev[st] = sd.wf_prev[i];
    sd.path_node[st] = node;
    sd.path_cost[st] = cost;
    sd.path_time[st] = sd.new_time[i];
    sd.path_cp[st] = cp;
    sd.map_src[rank] = (int)i;
    float dcost = (cost + sd.h[node] - cost_threshold);
    dcost = (0.0f < dcost) ? dcost : 0.0f;  // std::max((float)0, dCost)
    sd.bucket[rank] = (uint8_t)((((int)(dcost / dr)) + g_idx + 1) % 2);
    sd.node_next[st] = atomicExch(&sd.node_head[node], st);
    if (node == sd.goal && cp <= cp_min_soln) atomicOr(&sd.ctl->goal_found, 1);
  }
};

struct BucketPred {
  SearchDev sd;
  int b;
  __device__ bool operator()(long long k) const {
    return (unsigned long long)k < sd.ctl->num_valid && sd.bucket[k] == b;
  }
};
struct BucketEmit {
  SearchDev sd;
  int b, num_paths;
  __device__ void operator()(long long k, long long pos) const {
    sd.g_list[b][sd.ctl->g_count[b] + pos] = num_paths + (int)k;
  }
};

__global__ void bucket_count_kernel(const unsigned long long *total, SearchCtl *ctl, int b) {
  ctl->g_count[b] += (int)*total;
}

// Particle masks of the survivors: stage[map_src[k]] -> valid[k].
__global__ void gather_survivors_kernel(const uint32_t *__restrict__ stage,
                                        const int *__restrict__ map_src, const SearchCtl *ctl,
                                        int bound, int words, uint32_t *__restrict__ valid) {
  const long long n = (long long)bound * words;
  const long long num = (long long)ctl->num_valid * words;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n && t < num;
       t += (long long)gridDim.x * blockDim.x) {
    const long long k = t / words;
    valid[t] = stage[(long long)map_src[k] * words + (t - k * words)];
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
  PUMP_TRY(run_scan(ctx, n_g, ExpandCount{sd.g_list[g_idx], sd.path_node, sd.fgo}, sd.wf_off, s,
                    &ts));
  copy_total_kernel<<<1, 1, 0, s>>>(ts.total, &sd.ctl->num_new);
  return launch_status("copy_total");
}

pump_status_t search_expand_write(const SearchDev &sd, int g_idx, int n_g, cudaStream_t s) {
  if (n_g > 0) {
    const long long threads = (long long)n_g * 32;
    long long blocks = (threads + 255) / 256;
    if (blocks > kNumSMs * 16) blocks = kNumSMs * 16;
    expand_write_kernel<<<(unsigned)blocks, 256, 0, s>>>(sd, sd.g_list[g_idx], n_g);
    PUMP_TRY(launch_status("expand_write"));
  }
  clear_bucket_kernel<<<1, 1, 0, s>>>(sd.ctl, g_idx);
  return launch_status("clear_bucket");
}

pump_status_t search_prune(const SearchDev &sd, int num_new, int num_paths, float cp_cutoff,
                           float eps_cp, float eps_cost, cudaStream_t s) {
  const unsigned g = grid_for(num_new, 256);
  new_paths_kernel<<<g, 256, 0, s>>>(sd, num_new, cp_cutoff);
  PUMP_TRY(launch_status("new_paths"));
  link_new_kernel<<<g, 256, 0, s>>>(sd, num_new);
  PUMP_TRY(launch_status("link_new"));
  dominance_kernel<<<g, 256, 0, s>>>(sd, num_new, num_paths, eps_cp, eps_cost);
  return launch_status("dominance");
}

pump_status_t search_store(Ctx *ctx, const SearchDev &sd, int num_new, int num_paths,
                           int g_idx, float cost_threshold, float dr, float cp_min_soln,
                           const uint32_t *stage, uint32_t *valid, int words, cudaStream_t s) {
  TileScratch ts{};
  PUMP_TRY(run_compact(ctx, num_new, StorePred{sd},
                       StoreEmit{sd, num_paths, g_idx, cost_threshold, dr, cp_min_soln}, s, &ts));
  copy_total_kernel<<<1, 1, 0, s>>>(ts.total, &sd.ctl->num_valid);
  PUMP_TRY(launch_status("copy_total"));
  for (int b = 0; b < 2; ++b) {
    PUMP_TRY(run_compact(ctx, num_new, BucketPred{sd, b}, BucketEmit{sd, b, num_paths}, s, &ts));
    bucket_count_kernel<<<1, 1, 0, s>>>(ts.total, sd.ctl, b);
    PUMP_TRY(launch_status("bucket_count"));
  }
  const long long n = (long long)num_new * words;
  long long blocks = (n + 255) / 256;
  if (blocks > kNumSMs * 16) blocks = kNumSMs * 16;
  if (blocks < 1) blocks = 1;
  gather_survivors_kernel<<<(unsigned)blocks, 256, 0, s>>>(stage, sd.map_src, sd.ctl, num_new, words,
                                                           valid + (size_t)num_paths * words);
  return launch_status("gather_survivors");
}

}  // namespace pump
