// Device-resident exploration (the search loop of PUMP.cu:39-290): the
// state and the steps of one iteration, all on the device.  The host keeps
// only the loop control (a few counters read back twice per iteration).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pump.h"

namespace pump {

class Ctx;

// Counters of an iteration, read back by the host.
struct SearchCtl {
  unsigned long long num_new;    // wavefront size (expansion scan total)
  unsigned long long num_valid;  // survivors stored this iteration
  int g_count[2];                // bucket sizes (the reference's G lists)
  int goal_found;                // a stored goal path has CP <= cpTarget / eta
  int g_base[2];                 // bucket sizes before this iteration's appends
  int wait_error;                // 1: a look-back wait of the store pass gave up
  int overflow;                  // 1: wavefront > maxPathCount, 2: paths would reach it
  int todo;                      // nodes claimed for edge checks this iteration
};

// The wavefront size the kernels after the expansion work on: 0 when the
// iteration would overflow the path store.
__device__ __forceinline__ int wave_size(const SearchCtl *ctl) {
  return ctl->overflow ? 0 : (int)ctl->num_new;
}

// Device arrays of one search (capacities: M + 1 paths and new paths, N nodes).
struct SearchDev {
  int N, goal;
  // the roadmap's edges (row starts per node, destination, cost, time), the
  // free-sample mask, and the edges' free mask and each node's count of
  // expandable edges (free edges to a free node; -1: not checked yet), both
  // filled when the search first reaches the node (0 from its claim on,
  // counted up by the checks)
  const int *go, *dst;
  const float *copt, *topt, *h;
  const uint8_t *free_s;
  uint8_t *free_e;
  int *open_cnt;
  int *todo;  // nodes whose out-edges this iteration checks (capacity N)
  // stored paths
  int *path_prev, *path_node;
  float *path_cost, *path_time, *path_cp;
  int *g_list[2];
  int *node_head, *node_next;  // stored paths per node (linked lists)
  // the wavefront of the current iteration
  int *wf_prev, *wf_node, *wf_edge, *wf_open;
  unsigned int *wf_off;          // expansion offsets per bucket entry
  float *new_cost, *new_time;
  const float *new_cp;           // HSMC output
  uint8_t *alive, *dominated;
  int *new_head, *new_next;      // new paths per node passing the CP cut-off
  SearchCtl *ctl;
};

// What the edge checks of search_check need: the samples and the edges'
// waypoint layout (disc[e][W][6], written here), the obstacles and the BVP
// mode of the waypoints.
struct CheckArgs {
  const float *samples;
  float *disc;
  int numDisc, mode;
  const float *obs;
  int numObs;
  int max_degree;  // largest out-degree of the roadmap
};

// What the HSMC kernel writes for the search after a new path's CP (the
// first half of PUMP.cu:164-185): its time and cost, whether it survives the
// CP cut-off, and each survivor linked into its node's list of new paths
// (emptied by the expansion).
struct HsmcEpilogue {
  const int *wf_open, *wf_node;
  const float *path_time, *path_cost, *topt, *copt;
  float *new_time, *new_cost;
  uint8_t *alive;
  int *new_head, *new_next;
  float cp_cutoff;
};

// Path 0 at the initial node in bucket 0 (PUMP.cu:19-34).
pump_status_t search_init(const SearchDev &sd, cudaStream_t s);
// The nodes listed in todo (the initial node, then the nodes of stored
// paths as the store pass reaches them for the first time) get their
// out-edges checked (freeEdges, collisionCheck.cu:5-37, with the waypoints
// of findDiscretizedPath written on the way) and their count of expandable
// edges, before any path at them is expanded.  The reference checks every
// edge up front; the search reads only these, so the wavefronts are the
// same.  max_todo bounds the listed count (sizes the grid).
pump_status_t search_check(const SearchDev &sd, int max_todo, const CheckArgs &ca, cudaStream_t s);
// Every node's count of expandable edges from the full free-edge mask (the
// eager form: all edges checked up front).
pump_status_t search_count_open(const SearchDev &sd, cudaStream_t s);
// Largest out-degree of a CSR with row starts go[0..N] into *d_out (device).
pump_status_t max_degree_async(const int *d_go, int N, int *d_out, cudaStream_t s);
// Expansion offsets of the n_g paths of bucket g_idx; the wavefront size
// lands in ctl->num_new (n_g > 0).
pump_status_t search_expand_scan(Ctx *ctx, const SearchDev &sd, int g_idx, int n_g,
                                 cudaStream_t s);
// Writes the wavefront (PUMP.cu:47-66), empties bucket g_idx (recording the
// bucket sizes the appends start from) and clears the per-node lists of new
// paths at the wavefront's nodes.  The wavefront size is read from
// ctl->num_new; a wavefront larger than max_paths, or one that would bring
// the stored paths to max_paths, sets ctl->overflow and is not written
// (PUMP.cu:62-64, 73-76).
pump_status_t search_expand_write(const SearchDev &sd, int g_idx, int n_g, int num_paths,
                                  int max_paths, cudaStream_t s);
// New paths' time and cost, the CP cut-off (PUMP.cu:164-185) with per-node
// lists of the survivors of the cut-off (unless the HSMC kernel wrote them:
// new_paths_done), then epsilon dominance (PUMP.cu:188-218); wavefront size
// from the device (wave_size), at most max_new (sizes the grids).
pump_status_t search_prune(const SearchDev &sd, int max_new, int num_paths, float cp_cutoff,
                           float eps_cp, float eps_cost, bool new_paths_done, cudaStream_t s);
// The search's part of the HSMC kernel for this search state.
HsmcEpilogue search_hsmc_epilogue(const SearchDev &sd, float cp_cutoff);
// One pass over the wavefront (PUMP.cu:221-282): survivors become stored
// paths num_paths + rank in wavefront order, each is appended to its bucket
// in the same order, linked into its node's list, goal-tested, and its
// particle mask moves from the stage to its stored slot.
// Wavefront size from the device (wave_size); max_new bounds it (sizes the
// tile status words).
pump_status_t search_store(Ctx *ctx, const SearchDev &sd, int max_new, int num_paths,
                           int g_idx, float cost_threshold, float dr, float cp_min_soln,
                           const uint32_t *stage, uint32_t *valid, int words, cudaStream_t s);

}  // namespace pump
