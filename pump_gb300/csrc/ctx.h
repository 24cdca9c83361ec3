// Library context: the device it runs on and grow-only scratch buffers that
// are reused across calls (allocation happens only when a call needs more
// than any earlier call on the same context did).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include <functional>
#include <vector>

#include "pump.h"

namespace pump {

struct PairView;

class Ctx {
 public:
  enum Slot {
    kSelect = 0,   // radix-select state + histogram
    kCompact,      // compaction tile status words
    kPlanA,        // planner buffers (see plan.cpp)
    kRefine,       // refinement descent state (refine.cu)
    kSuperset,     // rn bracket bound and the pairs below it (select.cu)
    kLoop,         // the search loop graph's argument block and tile scratch
    kPairStage,    // per warp of the pair pass: the mask of its rn superset pairs
    kNumSlots
  };
  // Pinned host staging buffers (uploads, read-backs of small results).
  enum PinSlot { kPinIn = 0, kPinOut, kPinOptIn, kPinOptOut, kPinPaths, kPinCtl, kPinLoop, kNumPin };
  explicit Ctx(int device) : device_(device) {
    for (int i = 0; i < kNumSlots; ++i) { buf_[i] = nullptr; cap_[i] = 0; }
    for (int i = 0; i < kNumPin; ++i) { pin_[i] = nullptr; pin_cap_[i] = 0; }
  }
  ~Ctx();
  static Ctx *from(pump_ctx *c) { return reinterpret_cast<Ctx *>(c); }
  pump_ctx *handle() { return reinterpret_cast<pump_ctx *>(this); }
  int device() const { return device_; }
  pump_status_t activate();
  // Device buffer of at least `bytes` for `slot` (contents undefined).  A
  // buffer that grows leaves the old one to be freed with the context, so
  // growing never waits for the device.
  pump_status_t scratch(int slot, size_t bytes, void **out);
  // Pinned host buffer of at least `bytes` for `slot` (grow-only; an
  // outgrown buffer is freed with the context).
  pump_status_t pinned(int slot, size_t bytes, void **out);
  // Time-major particle table for (seed, P, T), generated on first use and
  // shared by every context on the device (the reference loads its table
  // once per process); `stream` is ordered after its generation.  The
  // largest |offset| per row and axis (T x 3) follows the table's P x T x 3
  // values in the same allocation.
  pump_status_t particle_table(uint64_t seed, int P, int T, const float **out, cudaStream_t stream);

  // Per-call device arena: the planner's buffers of one call are carved from
  // memory the context keeps across calls, so a call makes no allocation
  // calls once the arena has reached the size its calls need.  arena_begin
  // starts a call on stream s (ordered after the previous call's use of the
  // arena, and with the previous call's chunks merged into one when it
  // needed more than one); arena_take hands out 256-byte aligned regions
  // (adding a chunk when the current one is full); arena_end marks the end
  // of the call's use on s.  One call at a time per context.
  pump_status_t arena_begin(cudaStream_t s);
  pump_status_t arena_take(size_t bytes, void **out);
  void arena_end(cudaStream_t s);

  // The captured refinement loop of the last pump_refine_paths call, replayed
  // while its key (arguments, iterations, output and scratch pointers) is the same.
  struct GraphCache {
    unsigned char key[192];
    size_t key_len = 0;
    cudaGraphExec_t exec = nullptr;
  };
  GraphCache refine_graph;

  // Instantiated graphs of the search loop (search_loop_graph), one per
  // shape class, reused by every query on this context, and the stream they
  // are captured on.
  struct LoopGraph {
    int lazy, mode, obs_cap, num_disc, max_hs, particles;
    long long scan_cap, store_cap;
    void *base;
    cudaGraphExec_t exec;
  };
  std::vector<LoopGraph> loop_graphs;
  cudaStream_t capture_stream = nullptr;
  // recorded after a grouped search loop's argument block (pump_plan_batch)
  cudaEvent_t loop_ready = nullptr;
  // Values of the completion words that kernels write to pinned memory for
  // a host waiting on them (one per wait, never repeated on this context).
  unsigned int seq_counter = 0;

 private:
  int device_;
  void *buf_[kNumSlots];
  size_t cap_[kNumSlots];
  void *pin_[kNumPin];
  size_t pin_cap_[kNumPin];
  // outgrown buffers: queued work may still use them, so they are freed with
  // the context instead of at once (a free would wait for the whole device)
  std::vector<void *> retired_, retired_pinned_;
  // arena chunks in use by the current call (the first is kept across calls)
  struct ArenaChunk {
    char *p;
    size_t cap;
  };
  std::vector<ArenaChunk> arena_;
  size_t arena_used_ = 0;   // bytes taken from the last chunk
  size_t arena_total_ = 0;  // bytes taken by the current call
  cudaStream_t arena_stream_ = nullptr;
  cudaEvent_t arena_done_ = nullptr;  // recorded at the end of each call
  bool arena_pending_ = false;
};

// Internal device-side entry points shared between translation units.
pump_status_t select_kth_device(Ctx *ctx, const float *d_v, long long n, long long k,
                                const float **d_result, cudaStream_t stream);
pump_status_t build_edges_device(Ctx *ctx, const float *d_copts, const float *d_topts, int N,
                                 float rn, long long max_edges, int *d_src, int *d_dst,
                                 float *d_copt, float *d_topt, int *d_go_start,
                                 long long *h_num_edges, cudaStream_t stream);
pump_status_t select_kth_pairs(Ctx *ctx, const PairView &pv, long long k, const float **d_result,
                               cudaStream_t stream);
pump_status_t build_edges_pairs(Ctx *ctx, const PairView &pv, float rn, long long max_edges,
                                int *d_src, int *d_dst, float *d_copt, float *d_topt,
                                int *d_go_start, long long *h_num_edges, cudaStream_t stream);
// rn and the edge count of the one-read rn selection, left on the device
// until the caller's next read-back.  ok = 0: the superset of the pass
// missed rank k or overflowed its buffer; rn_bits and edges are then
// meaningless and the caller runs the matching *_fallback function.  edges
// exceeds max_edges when the edges did not fit (only max_edges were written).
struct RnEdgesPack {
  uint32_t rn_bits;
  int ok;
  unsigned long long edges;
  int error;  // a look-back wait of the pass gave up (PUMP_ERR_TIMEOUT)
  int pad;
};

// rn (the k-th smallest pair cost) and the edges below it in one read of the
// pair costs, from the query's own pair arrays or its pair view.  With
// `deferred`, nothing is read back: *h_num_edges is -1, *deferred points at
// the device pack (read it after a synchronisation) and the row starts are
// already built from the device count.  After the superset pass the rest
// runs as one cooperative launch (`cooperative`, the lower latency for a
// query that has the GPU to itself) or as separate launches that share the
// GPU with concurrent queries (always for a pair view: batch workers).
pump_status_t rn_edges_device(Ctx *ctx, const float *d_copts, const float *d_topts, int N,
                              long long k, long long max_edges, int *d_src, int *d_dst,
                              float *d_copt, float *d_topt, int *d_go_start, float *h_rn,
                              long long *h_num_edges, cudaStream_t stream,
                              const RnEdgesPack **deferred = nullptr, bool cooperative = true);
pump_status_t rn_edges_pairs(Ctx *ctx, const PairView &pv, long long k, long long max_edges,
                             int *d_src, int *d_dst, float *d_copt, float *d_topt,
                             int *d_go_start, float *h_rn, long long *h_num_edges,
                             cudaStream_t stream, const RnEdgesPack **deferred = nullptr);
// A read-back pack: PUMP_ERR_TIMEOUT when a wait gave up, fallback() when
// ok = 0, else rn and the edge count (PUMP_ERR_CAPACITY past max_edges).
pump_status_t rn_edges_unpack(const RnEdgesPack &pk, long long k, long long max_edges, float *h_rn,
                              long long *h_num_edges,
                              const std::function<pump_status_t()> &fallback);
// The exact three-pass select over all pairs and the full compaction
// (synchronises): what a pack with ok = 0 falls back to.
pump_status_t rn_edges_fallback_device(Ctx *ctx, const float *d_copts, const float *d_topts, int N,
                                       long long k, long long max_edges, int *d_src, int *d_dst,
                                       float *d_copt, float *d_topt, int *d_go_start, float *h_rn,
                                       long long *h_num_edges, cudaStream_t stream);
pump_status_t rn_edges_fallback_pairs(Ctx *ctx, const PairView &pv, long long k,
                                      long long max_edges, int *d_src, int *d_dst, float *d_copt,
                                      float *d_topt, int *d_go_start, float *h_rn,
                                      long long *h_num_edges, cudaStream_t stream);
// All N(N-1) pair BVPs of the samples (tmax, arithmetic bvp_mode), then rn
// and the edges as rn_edges_device.  In the precision arithmetic the pair
// kernel also writes the rn superset as it stores the costs (the bracket
// sample's costs are computed first), so the costs are not read again.
// stage_ms (optional, non-deferred only; 3 floats): CUDA-event times of what
// precedes the pair kernel (the samples' preparation and the bracket), the
// pair kernel, and the rest.  cooperative = false: the pair kernel without
// the superset masks and the separate-launch tail (for concurrent queries).
pump_status_t roadmap_pairs_edges(Ctx *ctx, const float *d_samples, int N, float tmax,
                                  int bvp_mode, long long k, long long max_edges, float *d_copts,
                                  float *d_topts, int *d_src, int *d_dst, float *d_copt,
                                  float *d_topt, int *d_go_start, float *h_rn,
                                  long long *h_num_edges, cudaStream_t stream,
                                  const RnEdgesPack **deferred = nullptr, float *stage_ms = nullptr,
                                  bool cooperative = true);
pump_status_t frontier_compact_device(Ctx *ctx, const uint8_t *d_flags, int N, int *d_active,
                                      int *d_count, int **d_error_out, cudaStream_t stream);
pump_status_t particle_rowmax_async(const float *d_table, int P, int T, float *d_rowmax,
                                    cudaStream_t stream);
pump_status_t particle_tables_async(uint64_t seed, int P, int T, float *d_tmajor, float *d_pmajor,
                                    cudaStream_t stream);
pump_status_t bvp_pairs_precision_launch(const float *d_samples, int N, float tmax, float *d_copts,
                                         float *d_topts, cudaStream_t stream);
// The precision pair pass marking the rn superset as it stores the costs.
// One kernel prepares the samples and computes the bracket sample's costs
// (pair numbers floor((2q + 1) n / (2 S)), S = the bracket's sample count)
// and, in its last block, the bracket bound *key_hi for the given rank.
// The pair kernel then stores every pair's cost and time and, per warp of
// 32 consecutive pairs of a row, the mask of those whose cost's order key is
// below *key_hi; *out describes the masks (masks_per_row per row of the
// pair matrix, each covering pairs 32 m .. 32 m + 31 of its row, bits past
// the row's end zero).  N <= 65535; sample_keys holds S words; done is one
// word, zero before the call (the kernel leaves it zero).  `between`
// (optional) is recorded before the pair kernel, after_pairs (optional)
// after it.
struct PairStage {
  const uint32_t *masks;
  long long nmasks;
  int masks_per_row;
};
struct PairSuperset {
  unsigned int rank;
  unsigned long long *key_hi;
  uint32_t *sample_keys;
  unsigned int *done;
  cudaEvent_t after_pairs;
  PairStage *out;
};
pump_status_t bvp_pairs_precision_superset(Ctx *ctx, const float *d_samples, int N, float tmax,
                                           float *d_copts, float *d_topts, const PairSuperset &ps,
                                           cudaStream_t stream, cudaEvent_t between = nullptr);
// Explicit pairs (x0[k], x1[k]), k < n (x1[0] for every k with x1_same),
// each bisected for `jobs` (1 or 2)
// optimal-time limits: job j writes topt[j][k] and cost[j][k] (either may be
// null).  One thread per (job, pair); small batches use 32-thread blocks so
// their binary64 bisections spread over more SMs.
struct BvpJobs {
  const float *x0, *x1;
  int n, jobs;
  float tmax[2];
  float *topt[2], *cost[2];
  int x1_same;  // 1: every pair's end state is x1[0..5]
};
pump_status_t bvp_jobs_launch(const BvpJobs &jb, int mode, cudaStream_t stream);
pump_status_t bvp_jobs_precision_launch(const BvpJobs &jb, cudaStream_t stream);
// the reference GPU kernel's arithmetic (bvp_refgpu.cu)
pump_status_t bvp_pairs_refgpu_launch(const float *d_samples, int N, float tmax, float *d_copts,
                                      float *d_topts, cudaStream_t stream);
pump_status_t bvp_jobs_refgpu_launch(const BvpJobs &jb, cudaStream_t stream);
// Optimal time of every edge (src[e], dst[e]) in the parity arithmetic
// (toptBisection as the reference's host code runs it, tmax 5): the time the
// reference's findDiscretizedPath recomputes for the waypoints.
pump_status_t edge_topts_parity_async(const float *d_samples, const int *d_src, const int *d_dst,
                                      long long E, float *d_topt, cudaStream_t stream);
// Per-edge waypoint counts by edge length and their ragged layout (bvp.cu):
// d_off[E + 1] (the first record of each edge, the total at E) from
// d_scratch of disc_offsets_scratch(E) bytes; the waypoints over that layout
// (*error, when given, records an edge count outside [2, max_disc + 1]).
size_t disc_offsets_scratch(long long E);
pump_status_t disc_offsets_async(const float *d_samples, const int *d_src, const int *d_dst,
                                 long long E, float disc_len, int min_disc, int max_disc,
                                 long long *d_off, long long *d_scratch, cudaStream_t s);
pump_status_t discretize_off_async(const float *d_samples, const int *d_src, const int *d_dst,
                                   const float *d_topt, long long E, const long long *d_off,
                                   int max_disc, int mode, float *d_disc, cudaStream_t s,
                                   int *error = nullptr);
// freeEdges over the ragged layout (collide.cu).
pump_status_t free_edges_off_async(const float *d_obstacles, int numObs, const float *d_disc,
                                   const long long *d_off, long long E, int max_disc,
                                   uint8_t *d_is_free, cudaStream_t s, int *error = nullptr);
// The BVP arithmetic of the reference's host code for a planner mode: the
// parity arithmetic for both parity modes, the precision mode otherwise.
inline int host_bvp_mode(int mode) { return mode == PUMP_BVP_PRECISION ? PUMP_BVP_PRECISION : PUMP_BVP_PARITY; }
// Device buffers of a batch of candidate paths: per path its node count and
// first segment; its segments (node i -> i + 1) as explicit pairs x0, x1,
// paths in order; their optimal times (tmax 5) and smoothing costs (tmax 2),
// the dense path of findOptimalPath per path at a fixed stride of rows_cap
// rows, and per path its length and cost.
struct CandidateBufs {
  const int *node_cnt, *seg_base;
  const float *x0, *x1;
  float *topt, *seg_cost, *states, *cost;
  int *len;
  int *hits;     // zeroed per path when not null (the MC CP counters)
  float *topt2;  // when not null: the segments' optimal times with tmax 2
  unsigned int *done;  // zeroed when not null (the MC CP's finished-block count)
};
// max_segs: the most segments of one path.
pump_status_t candidate_paths_async(const CandidateBufs &cb, int n_paths, int n_seg, int max_segs,
                                    int mode, float dt, bool with_cost, int rows_cap,
                                    cudaStream_t s);
// MC CP hit counts of n_paths dense paths into d_hits (zeroed beforehand):
// the kernels of mc_cp_async without its memset and CP division.  With
// copy_dst (host memory; n_paths <= 65535), the last block to finish copies
// copy_words words from copy_src to it, then writes seq to
// copy_dst[copy_words]; *done must be zero before the launch.
pump_status_t mc_cp_hits_async(const float *d_paths, const int *d_offset, const int *d_len,
                               int n_paths, const float *d_offsets_t, int Pmc, int T_rows,
                               float offset_mult, const float *d_obstacles, int numObs,
                               int *d_hits, cudaStream_t stream, const float *d_rowmax,
                               const int *copy_src = nullptr, int *copy_dst = nullptr,
                               int copy_words = 0, unsigned int *done = nullptr,
                               unsigned int seq = 0);
// Halton samples of a query (sampler.cu:20-41), N x 6, then (goal_row) the
// goal row once more.
pump_status_t halton_samples_async(int N, const float *lo, const float *hi, const float *init,
                                   const float *goal, float *d_out, cudaStream_t stream,
                                   bool goal_row = true);
// The 4N-6 pairs of a query that touch its init or goal sample, as explicit
// (x0, x1) rows: init row (0 -> j, j = 1 .. N-1), init column (i -> 0),
// goal row (N-1 -> j, j = 1 .. N-2), goal column (i -> N-1).
pump_status_t own_pairs_async(const float *d_samples, int N, float *d_x0, float *d_x1,
                              cudaStream_t stream);
pump_status_t bvp_path_states(const float *d_xs, const int *d_seg, const float *d_tsample,
                              const float *d_tau, int total, float *d_out, cudaStream_t stream);

}  // namespace pump
