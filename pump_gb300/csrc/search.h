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
  unsigned int seq;              // host copy: written last, after the fields above
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
  uint8_t *alive;
  int *new_head, *new_next;      // new paths per node passing the CP cut-off
  SearchCtl *ctl;
};

// What the edge checks of search_check need: the samples and the edges'
// waypoint layout (disc[e][W][6], written here), the obstacles and the BVP
// mode of the waypoints.
struct CheckArgs {
  const float *samples;
  float *disc;
  int numDisc, mode;       // mode: PUMP_BVP_PARITY or PUMP_BVP_PRECISION waypoints
  const float *wp_topt;    // per edge, the optimal time its waypoints are evaluated at
  // the ragged waypoint layout (may be null: numDisc + 1 records per edge):
  // edge e's records disc_off[e] .. disc_off[e+1]-1, at most numDisc + 1
  const long long *disc_off;
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

// Arguments of the HSMC kernel (hsmc.cu).
struct HsmcParams {
  int num_new, W;
  // with num_new_dev the path count is *num_new_dev (0 when *skip_dev is set)
  const unsigned long long *num_new_dev;
  const int *skip_dev;
  const int *wf_edge, *wf_prev;
  long long num_edges;
  int num_prev;
  // cached half-spaces
  const float *as, *bs;
  const uint8_t *hs_count;
  // half-spaces from the boxes; disc_off (may be null): the ragged waypoint
  // layout, edge e's waypoints at records disc_off[e] .. disc_off[e+1]-1
  // (2 .. W of them), otherwise W records per edge
  const float *obs, *disc;
  const long long *disc_off;
  int numObs;
  float maxd2;
  int maxHS;
  const float *times, *topts;
  float dt;
  const float *offsets_t;
  int Pmc, T_rows;
  float offset_mult;
  const uint32_t *valid_in;
  uint32_t *valid_out;
  int P;
  float *cp_out;
  int *error;
  // the search's new-path step after each CP (when epi_on)
  HsmcEpilogue epi;
  int epi_on;
};

// The search loop run on the device: a CUDA graph whose conditional while
// node repeats one iteration's kernels.  The iteration's kernels read the
// values the host loop passes as arguments from this state, and the control
// kernel at the end of each iteration updates it exactly as the host loop
// does (PUMP.cu:39-290), then sets the while node's condition.
struct LoopState {
  // per query
  int max_itrs, max_paths;
  float dr;
  // the loop
  int itrs, g_idx, n_g, num_paths, status, guard;
  int active;  // 1 while the loop goes on (the graph's kernels skip a finished query)
  float cost_threshold;
  long long considered;
  int g_count[2];
  int wavefront_sizes[32];
};
enum LoopStatus {
  kLoopOk = 0,
  kLoopWavefrontOverflow,  // wavefront larger than maxPathCount
  kLoopPathsWouldOverflow, // stored paths would reach maxPathCount
  kLoopWaitError,          // a look-back wait of the store pass gave up
  kLoopPathsFull           // stored paths reached maxPathCount
};

// Items per look-back tile of the loop's expansion and store passes.
constexpr int kLoopScanTile = 32;
constexpr int kLoopStoreTile = 256;

// Tile scratch of one look-back pass of the loop (zeroed before each pass):
// total, status words (one per tile, from status[0]), tile counter, error
// word, and the count of blocks that finished the pass.
struct LoopTiles {
  unsigned long long *total, *status;
  unsigned int *tile_counter;
  int *error;
  unsigned int *done;
  long long cap;  // tiles
};
// 8-byte words of a LoopTiles region for cap tiles (total, cap + 1 status
// words, tile counter and error word, done count).
__host__ __device__ inline long long loop_tile_words(long long cap) { return cap + 4; }

// Everything the loop's kernels read, at one device address per context.
struct LoopArgs {
  SearchDev sd;
  CheckArgs ca;
  HsmcParams hp;
  LoopState L;
  LoopTiles scan, store;
  // the store pass
  float cp_min_soln, eps_cp, eps_cost, cp_cutoff;
  const uint32_t *stage;
  uint32_t *valid;
  int words, P;
  int *err;  // the particle-table error word (zeroed at the start)
};

// The searches one loop graph runs side by side: query y of a launch is
// args[y] (y < nq).  The graph's kernels give each query a share of their
// grid (blockIdx.y), except HSMC, whose blocks take the chunks of all the
// queries' wavefronts in turn; every kernel skips a query whose loop has
// ended.  The while node repeats the iteration while any query goes on.
constexpr int kLoopGroupMax = 16;
struct LoopGroup {
  LoopArgs *args[kLoopGroupMax];
  int nq;
  unsigned int store_done;  // store-pass blocks (all queries) done with this iteration
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
// The expansion (PUMP.cu:47-66) in one pass over the n_g paths of bucket
// g_idx (n_g > 0): writes the wavefront in order, its size to ctl->num_new,
// and flags (ctl->overflow) a wavefront larger than max_paths, or one that
// would bring the stored paths to max_paths (PUMP.cu:62-64, 73-76); the
// kernels after it then see an empty wavefront.  Empties bucket g_idx,
// records the bucket sizes the appends start from, clears the per-node lists
// of new paths at the wavefront's nodes and zeroes the store pass's tile
// scratch.  Its own tile scratch (scan) must be zeroed (the store pass
// zeroes it for the next iteration).
pump_status_t search_expand(const SearchDev &sd, int g_idx, int n_g, int num_paths, int max_paths,
                           const LoopTiles &scan, const LoopTiles &store, cudaStream_t s);
// The search's part of the HSMC kernel for this search state.
HsmcEpilogue search_hsmc_epilogue(const SearchDev &sd, float cp_cutoff);
// One pass over the wavefront (PUMP.cu:188-282): a new path survives if it
// passed the CP cut-off, is not epsilon-dominated (PUMP.cu:188-218, tested
// here against the lists as they were when the pass began) and is not at
// the initial node; survivors become stored
// paths num_paths + rank in wavefront order, each is appended to its bucket
// in the same order, linked into its node's list, goal-tested, and its
// particle mask moves from the stage to its stored slot.
// Wavefront size from the device (wave_size); max_new bounds it (sizes the
// grid).  The store's tile scratch must be zeroed; it zeroes the
// expansion's (scan) for the next iteration.  With host_ctl (pinned
// host memory), the last block to finish copies the iteration's counters
// there and then writes seq to host_ctl->seq, so the host can wait for that
// word instead of synchronising the stream.
pump_status_t search_store(const SearchDev &sd, int max_new, int num_paths, int g_idx,
                           float cost_threshold, float dr, float cp_min_soln, float eps_cp,
                           float eps_cost, const uint32_t *stage,
                           uint32_t *valid, int words, const LoopTiles &store,
                           const LoopTiles &scan, SearchCtl *host_ctl, unsigned int seq,
                           cudaStream_t s);

// The graph of the search loop for the group at d_group (device; at most
// gcap queries): init, then a while node over {[lazy: edge checks],
// expansion, HSMC, store with the dominance test and the control step}.
// Launch shapes are fixed (grid-stride and tile-counter loops); dynamic
// shared memory is sized for numObs boxes, numDisc waypoints per edge,
// maxHS half-spaces and P particles, each at least the group's largest.
// Kernel attributes are set here, before the capture.
pump_status_t search_loop_graph(LoopGroup *d_group, int gcap, bool lazy, int mode, int numObs,
                                int numDisc, int maxHS, int P, cudaStream_t capture_stream,
                                cudaGraphExec_t *out);

// HSMC in the loop graph (hsmc.cu): all active queries of the group.
pump_status_t hsmc_loop_prepare(int numObs, int W, int maxHS, int P);
pump_status_t hsmc_loop_launch(const LoopGroup *d_group, int numObs, int W, int maxHS, int P,
                               int blocks, cudaStream_t stream);
pump_status_t hsmc_boxes_fill(int num_new, int W, const int *d_edge, const int *d_prev,
                              long long num_edges, int num_prev, const float *d_obs, int numObs,
                              const float *d_disc, float maxd2, int maxHS, const float *d_times,
                              const float *d_topt, float dt, const float *d_offsets_t, int Pmc,
                              int T_rows, float offset_mult, const uint32_t *d_valid_in,
                              uint32_t *d_valid_out, int P, float *d_cp_out, int *d_error,
                              const unsigned long long *d_num_new, const int *d_skip,
                              const HsmcEpilogue *epi, HsmcParams *out,
                              const long long *d_disc_off = nullptr);

}  // namespace pump
