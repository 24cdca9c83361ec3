// One PUMP planning query on the GPU (reference: mainPUMP.cu:248-687 and
// PUMP(), PUMP.cu:3-607).
//
// Device work: pair BVPs, rn selection, edge compaction, waypoints,
// heuristic, sample/edge collision checks, half-spaces, the particle table,
// the search loop (search.cu: expansion, HSMC, CP cut-off, epsilon
// dominance, survivor compaction, buckets), and the dense paths and Monte
// Carlo CP of goal candidates and smoothing iterates.  The host keeps the
// loop control of the search and the alpha bisection of the smoothing loop.
// Differences in structure, not in results:
//  - the reference copies each survivor's particle mask with one
//    cudaMemcpy (PUMP.cu:236-237); here survivors are gathered by one kernel;
//  - the reference evaluates goal candidates one at a time until one meets
//    the CP target (PUMP.cu:371-405); here all candidates' dense paths and
//    MC CPs are computed in one batch and the first in (cost, index) order
//    that meets the target is taken, which selects the same path;
//  - adjacency is a CSR over edges sorted by (source, target) instead of the
//    N x N nnIdxs table (mainPUMP.cu:315, 338).
// Host arithmetic follows the reference's float expressions and is compiled
// without multiply-add contraction.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <string>
#include <memory>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <utility>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "loopbatch.h"
#include "pairview.cuh"
#include "search.h"

namespace pump {

bool hsmc_boxes_fits(int numObs, int W, int maxHS);
pump_status_t hsmc_boxes_async(int num_new, int W, const int *d_edge, const int *d_prev,
                               long long num_edges, int num_prev, const float *d_obs, int numObs,
                               const float *d_disc, float maxd2, int maxHS, const float *d_times,
                               const float *d_topt, float dt, const float *d_offsets_t, int Pmc,
                               int T_rows, float offset_mult, const uint32_t *d_valid_in,
                               uint32_t *d_valid_out, int P, float *d_cp_out, int *d_error,
                               cudaStream_t stream, const unsigned long long *d_num_new,
                               const int *d_skip, const HsmcEpilogue *epi,
                               const long long *d_disc_off = nullptr);
pump_status_t mc_cp_async(const float *d_paths, const int *d_offset, const int *d_len, int n_paths,
                          const float *d_offsets_t, int Pmc, int T_rows, float offset_mult,
                          const float *d_obstacles, int numObs, int *d_hits, float *d_cp,
                          int *d_error, cudaStream_t stream, const float *d_rowmax);

namespace {

using clk = std::chrono::steady_clock;
double ms_since(clk::time_point t0) {
  return std::chrono::duration<double, std::milli>(clk::now() - t0).count();
}

// Stream that the planner running on this host thread allocates on, and the
// context whose arena its buffers come from (null: stream-ordered pool).
thread_local cudaStream_t t_alloc_stream = nullptr;
thread_local Ctx *t_arena = nullptr;

// Device buffer of a planner call: a region of the context's arena while a
// planner runs on this thread (released with the call), else allocated and
// freed in stream order on the planner's stream (cudaMallocAsync /
// cudaFreeAsync).  Neither synchronises the device, so planners on other
// streams keep running; the arena also makes no allocation call per buffer,
// which matters when many host threads plan at once.
template <class T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  bool arena = false;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { if (p && !arena) cudaFreeAsync(p, s); }
  pump_status_t alloc(size_t count) {
    if (count <= n && p) return PUMP_OK;
    if (p && !arena) PUMP_CUDA_TRY(cudaFreeAsync(p, s));
    p = nullptr;
    n = 0;
    s = t_alloc_stream;
    arena = t_arena != nullptr;
    if (arena) PUMP_TRY(t_arena->arena_take(sizeof(T) * (count ? count : 1), (void **)&p));
    else PUMP_CUDA_TRY(pool_malloc_async((void **)&p, sizeof(T) * (count ? count : 1), s));
    n = count;
    return PUMP_OK;
  }
};

// Which planners run the search loop as a graph (pump_search_graph): 0
// none, 1 single queries (the default), 2 batch workers too; the
// environment variable PUMP_SEARCH_GRAPH sets the starting level.
std::atomic<int> &search_graph_flag() {
  static std::atomic<int> flag([] {
    const char *e = std::getenv("PUMP_SEARCH_GRAPH");
    return (e && e[0] >= '0' && e[0] <= '2') ? e[0] - '0' : 1;
  }());
  return flag;
}

// Grouped search loops of pump_plan_batch (pump_batch_groups): queries per
// group (1: none) and the window in microseconds; the environment variable
// PUMP_BATCH_GROUPS ("max_group" or "max_group,window_us") sets the
// starting values.
std::atomic<int> *batch_group_flags() {
  static std::atomic<int> flags[2];
  static std::once_flag once;
  std::call_once(once, [] {
    int g = 1, w = 100;
    if (const char *e = std::getenv("PUMP_BATCH_GROUPS")) {
      char *end = nullptr;
      const long v = std::strtol(e, &end, 10);
      if (end != e) g = (int)(v < 1 ? 1 : (v > kLoopGroupMax ? kLoopGroupMax : v));
      if (end && *end == ',') {
        const long u = std::strtol(end + 1, nullptr, 10);
        w = (int)(u < 0 ? 0 : (u > 100000 ? 100000 : u));
      }
    }
    flags[0].store(g);
    flags[1].store(w);
  });
  return flags;
}

// The arena of ctx serves this thread's planner buffers while in scope.
struct ArenaScope {
  Ctx *c;
  cudaStream_t s;
  ArenaScope(Ctx *ctx, cudaStream_t stream) : c(ctx), s(stream) { t_arena = ctx; }
  ~ArenaScope() {
    t_arena = nullptr;
    c->arena_end(s);
  }
};

// sampler.cu:43-57
float halton(int n, int b) {
  float hn = 0;
  int n0 = n;
  float f = 1 / ((float)b);
  while (n0 > 0) {
    float n1 = (float)(n0 / b);
    int r = (int)(n0 - n1 * b);
    hn += f * r;
    f = f / b;
    n0 = (int)n1;
  }
  return hn;
}

// sampler.cu:20-41 (bases 2, 3, 5, 7, 11, 13 with skip 0)
void halton_samples(const pump_problem &pb, std::vector<float> &s) {
  static const int bases[6] = {2, 3, 5, 7, 11, 13};
  const int N = pb.N;
  s.assign((size_t)N * kDim, 0.0f);
  for (int d = 0; d < kDim; ++d)
    for (int n = 0; n < N; ++n)
      s[(size_t)n * kDim + d] = halton(n, bases[d]) * (pb.hi[d] - pb.lo[d]) + pb.lo[d];
  for (int d = 0; d < kDim; ++d) {
    s[d] = pb.init[d];
    s[(size_t)(N - 1) * kDim + d] = pb.goal[d];
  }
}

// Device buffers of one batch of candidate paths and the pinned slots of its
// upload and read-back.  A planner keeps two, so the unconstrained optimal
// path is evaluated in the same round trip as the goal candidates.
struct CandSet {
  int pin_in, pin_out;
  DevBuf<float> in, segcost, states;
  DevBuf<int> out;  // hits | lengths | costs | optimal times (tmax 5, then 2)
  // the batch launched last (read back by eval_read after a synchronisation)
  int n = 0, segs = 0, states_rows = 0, table_rows = 0, num_mc = 0;
  bool with_cost = false, with_cp = false, with_topts = false;
  const char *hout = nullptr;
  size_t head_bytes = 0;  // results before the completion word
  unsigned int seq = 0;   // completion word value (0: none, wait on the stream)
  CandSet(int in_slot, int out_slot) : pin_in(in_slot), pin_out(out_slot) {}
};

// What eval_read returns: per path the dense length, the smoothing's cost and
// the MC CP (-1 when the dense path has more states than the table has rows);
// per segment (paths in order) the optimal times with tmax 5 and with tmax 2
// when asked for; the first rows of path 0's dense states when asked for.
struct CandResult {
  std::vector<int> len;
  std::vector<float> cost, cp, t5, t2, states;
};

// Pair BVPs of Halton points 1 .. M shared by a batch's queries (see
// pairview.cuh); key = the BVP mode and the state bounds that scale the points.
struct SharedRoadmap {
  int mode;
  float lo[6], hi[6];
  long long M;
  const float *d_copt, *d_topt;  // pump_bvp_pairs layout over the M points
  bool matches(const pump_problem &pb) const {
    if (pb.samples || pb.bvp_mode != mode || pb.N - 2 > M || pb.N < 4) return false;
    for (int d = 0; d < 6; ++d)
      if (pb.lo[d] != lo[d] || pb.hi[d] != hi[d]) return false;
    return true;
  }
};


class Planner {
 public:
  // lazy: check each node's out-edges when the search first reaches it (the
  // batch's throughput form); otherwise all edges are checked up front (the
  // latency form).  Results are the same.  batcher: the search loop runs in
  // a group of the batch's queries (one graph launch for the group).
  Planner(Ctx *ctx, const pump_problem &pb, pump_plan_result *res, cudaStream_t s,
          const SharedRoadmap *shared = nullptr, bool lazy = false,
          LoopBatcher *batcher = nullptr)
      : ctx_(ctx), pb_(pb), res_(res), s_(s), shared_(shared), lazy_(lazy), batcher_(batcher) {}
  pump_status_t run();
  // CP (dense path + MC over the table), smoothing cost and dense length of
  // explicit candidate paths (pump_path_cp).
  pump_status_t evaluate_paths(const std::vector<std::vector<float>> &xs, const float *d_table,
                               const float *d_obs, int nobs, float *cp, float *cost, int *len);

 private:
  pump_status_t roadmap();
  pump_status_t pair_costs_shared(long long rnIdx, long long cap);
  pump_status_t online();
  pump_status_t explore();
  // The search loop as one launch of the context's loop graph; fills the
  // counters the host loop keeps (iterations, stored and considered paths,
  // wavefront sizes) and the loop's status.
  // The context's loop region for M paths: the graph's argument block, then
  // the tile scratch of the expansion scan and of the store pass.
  pump_status_t loop_region(int M, char **base, size_t *args_b, LoopTiles *scan, LoopTiles *store);
  pump_status_t explore_graph(const SearchDev &sd, const CheckArgs &ca, const HsmcEpilogue &epi,
                              int M, float cpCutoff, float cpMinSoln, float dr, int *itrs,
                              long long *considered, pump_status_t *status);
  // The loop's counters and status from the argument block after the loop.
  pump_status_t loop_result(const LoopArgs *d_args, int M, int *itrs, long long *considered,
                            pump_status_t *status);
  pump_status_t search_and_smooth();
  // The controller's discretisation of node states xs; t5 and t2, when not
  // null, are the segments' optimal times with tmax 5 and 2 (else computed
  // here).  control_launch enqueues its work (after a pending read-back of
  // the kept path, if any); control_finish runs after a synchronisation.
  pump_status_t control_launch(const std::vector<float> &xs, const std::vector<float> *t5,
                               const std::vector<float> *t2);
  pump_status_t control_finish();
  pump_status_t refine(const std::vector<float> &xs, float cpTarget, float *lastCP,
                       float *lastCost, std::vector<float> *bestPath, int *bestLen,
                       std::vector<float> *xsFinal);
  // Candidate paths evaluated on the device (candidate_paths_async) with
  // the buffers of c: eval_launch enqueues the upload, the kernels and the
  // read-back into pinned memory (states of path k at c.states + k *
  // rows_cap rows; with_topts: the segments' optimal times with tmax 5 and
  // 2; states_rows: read back that many rows of path 0's states);
  // eval_read parses the read-back after a synchronisation.
  pump_status_t eval_launch(CandSet &c, const std::vector<std::vector<float>> &xs, float dt,
                            int rows_cap, bool with_cost, bool with_cp, bool with_topts,
                            int states_rows);
  void eval_read(const CandSet &c, CandResult *r) const;
  // eval_launch, synchronisation and eval_read on the first buffer set
  pump_status_t eval_candidates(const std::vector<std::vector<float>> &xs, float dt, int rows_cap,
                                bool with_cost, bool with_cp, std::vector<int> &len,
                                std::vector<float> &cost, std::vector<float> &cp);
  pump_status_t topts_of(const std::vector<float> &x0, const std::vector<float> &x1, float tmax,
                         std::vector<float> *topt, std::vector<float> *cost);
  pump_status_t sync() {
    const auto t = clk::now();
    const pump_status_t st = cuda_status(cudaStreamSynchronize(s_), "cudaStreamSynchronize");
    res_->ms_wait += ms_since(t);
    ++res_->num_waits;
    return st;
  }
  // Waits until the stream's last kernel has written `want` to the pinned
  // completion word (written after the results it guards), without a driver
  // call per wait; every 0.5 ms the stream's status is checked, so a fault,
  // or a stream that finished without writing the word, ends the wait with
  // an error.
  pump_status_t wait_seq(const unsigned int *word, unsigned int want) {
    const auto t = clk::now();
    auto checked = t;
    while (__atomic_load_n(word, __ATOMIC_ACQUIRE) != want) {
      const auto now = clk::now();
      if (now - checked < std::chrono::microseconds(500)) continue;
      checked = now;
      const cudaError_t e = cudaStreamQuery(s_);
      if (e == cudaErrorNotReady) continue;
      if (e != cudaSuccess) return cuda_status(e, "cudaStreamQuery");
      if (__atomic_load_n(word, __ATOMIC_ACQUIRE) == want) break;
      return set_error(PUMP_ERR_CUDA, "stream finished without writing its completion word");
    }
    res_->ms_wait += ms_since(t);
    ++res_->num_waits;
    return PUMP_OK;
  }
  // The next completion word value of this context.
  unsigned int next_seq() { return ++ctx_->seq_counter; }
  // Waits for the candidate batch launched last on c (its completion word,
  // or the stream).
  pump_status_t wait_cand(const CandSet &c) {
    if (c.n == 0) return PUMP_OK;
    if (!c.seq) return sync();
    return wait_seq(reinterpret_cast<const unsigned int *>(c.hout + c.head_bytes), c.seq);
  }
  template <class T>
  pump_status_t h2d(T *d, const T *h, size_t n) {
    if (n == 0) return PUMP_OK;
    res_->h2d_bytes += (long long)(sizeof(T) * n);
    return cuda_status(cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, s_), "H2D");
  }
  template <class T>
  pump_status_t d2h(T *h, const T *d, size_t n) {
    if (n == 0) return PUMP_OK;
    res_->d2h_bytes += (long long)(sizeof(T) * n);
    return cuda_status(cudaMemcpyAsync(h, d, sizeof(T) * n, cudaMemcpyDeviceToHost, s_), "D2H");
  }
  std::vector<float> node_states(int path_idx, std::vector<int> *nodes) const;

  Ctx *ctx_;
  const pump_problem &pb_;
  pump_plan_result *res_;
  cudaStream_t s_;
  const SharedRoadmap *shared_;
  bool lazy_ = false;
  LoopBatcher *batcher_ = nullptr;
  DevBuf<float> d_own_c_, d_own_t_;  // pairs touching init/goal (shared-roadmap path)

  // problem constants (mainPUMP.cu:51-72)
  const float dt_ = (float)0.05;
  const float lambda_ = (float)0.5;
  const int numBuckets_ = 2;
  const float epsCost_ = (float)0.0002, epsCP_ = (float)0.0002;
  const int maxItrs_ = 20;
  int N_ = 0, W_ = 0, P_ = 0, words_ = 0, maxHS_ = 0, nobs_ = 0;
  float maxd2_ = 0;

  std::vector<float> samples_;
  DevBuf<float> d_samples_, d_obs_, d_copts_, d_topts_;
  DevBuf<int> d_src_, d_dst_, d_go_;
  DevBuf<float> d_coptE_, d_toptE_, d_disc_;
  // PUMP_BVP_PARITY_GPU: each edge's optimal time in the host arithmetic, the
  // time the reference's findDiscretizedPath evaluates the waypoints at
  // (d_toptE_ holds the GPU kernel's times, which the search and HSMC use)
  DevBuf<float> d_toptH_;
  // per-edge waypoint counts by edge length (pb_.disc_len > 0): edge e's
  // waypoints are records d_disc_off_[e] .. d_disc_off_[e+1]-1 of d_disc_
  DevBuf<long long> d_disc_off_, d_disc_scratch_;
  const long long *disc_off() const { return pb_.disc_len > 0 ? d_disc_off_.p : nullptr; }
  const float *waypoint_topts() const {
    return pb_.bvp_mode == PUMP_BVP_PARITY_GPU ? d_toptH_.p : d_toptE_.p;
  }
  const float *d_table_ = nullptr;   // context-cached particle table
  const float *d_rowmax_ = nullptr;  // its largest |offset| per row and axis
  const float *obs_p_ = nullptr;    // device obstacles used by the MC CP
  DevBuf<uint8_t> d_free_s_, d_free_e_;
  DevBuf<int> d_open_cnt_;  // per node: expandable edges, -1 until checked
  DevBuf<int> d_todo_;      // nodes checked in an iteration
  DevBuf<int> d_scalar_;    // one int read back with the roadmap
  int max_degree_ = 0;      // largest out-degree of the roadmap
  long long E_ = 0;
  // rn and the edge count left on the device by the roadmap (null when they
  // were read back already), and the pair view of a batched query's costs
  const RnEdgesPack *d_pack_ = nullptr;
  PairView pv_{};
  bool use_pv_ = false;
  float rn_ = 0;
  DevBuf<float> d_h_;  // heuristic per node (cost to the goal)
  float h0_ = 0;

  // exploration state (mainPUMP.cu:623-681)
  int maxPathCount_ = 0;
  std::vector<int> pathPrev_, pathNode_;
  std::vector<float> pathCost_;
  std::vector<std::vector<int>> atNode_;
  DevBuf<uint32_t> d_valid_, d_stage_;
  DevBuf<float> d_pathTime_, d_cpStage_;
  DevBuf<int> d_wfPrev_, d_wfEdge_, d_err_;
  int numPaths_ = 0;
  // reusable scratch of the batched BVP / dense-path / MC CP helpers
  DevBuf<float> d_bx0_, d_bx1_, d_bt_, d_bc_, d_xs_;
  // candidate batches: the search's and the unconstrained optimal path's;
  // the dense path kept by the smoothing
  CandSet cs_{Ctx::kPinIn, Ctx::kPinOut}, co_{Ctx::kPinOptIn, Ctx::kPinOptOut};
  DevBuf<float> d_best_;
  // the controller path being assembled (control_launch .. control_finish)
  struct ControlJob {
    int rows = 0, total = 0;
    std::vector<float> out;
    std::vector<int> row;
    const float *pts = nullptr;  // pinned read-back of the sampled states
  } ctrl_;
  DevBuf<float> d_ctrl_;
};

pump_status_t Planner::run() {
  const auto t0 = clk::now();
  t_alloc_stream = s_;
  N_ = pb_.N;
  W_ = pb_.num_disc + 1;
  P_ = pb_.num_hsmc;
  words_ = (P_ + 31) / 32;
  nobs_ = pb_.num_obstacles;
  maxHS_ = nobs_ > 5 ? 5 : nobs_;  // mainPUMP.cu:241
  auto t = clk::now();
  PUMP_TRY(roadmap());
  res_->ms_roadmap = ms_since(t);
  t = clk::now();
  PUMP_TRY(online());
  res_->ms_online = ms_since(t);
  t = clk::now();
  pump_status_t st = explore();
  res_->ms_explore = ms_since(t);
  if (st == PUMP_OK) {
    t = clk::now();
    st = search_and_smooth();
    res_->ms_search = ms_since(t);
  }
  res_->ms_total = ms_since(t0);
  return st;
}

pump_status_t Planner::roadmap() {
  // the samples (then the goal state once more) on the device: Halton points
  // generated there, or the caller's samples uploaded through pinned memory.
  // Pinned read-back (at the roadmap's synchronisation): h[0], the largest
  // out-degree, then the Halton samples for the host's path reconstruction.
  const size_t nsf = (size_t)N_ * kDim;
  PUMP_TRY(d_samples_.alloc(nsf + kDim));
  float *hout = nullptr;
  // (then rn and the edge count when they stay on the device until this
  // read-back; 2 + nsf floats keep the pack 8-byte aligned)
  PUMP_TRY(ctx_->pinned(Ctx::kPinOut, sizeof(float) * (2 + nsf) + sizeof(RnEdgesPack),
                        (void **)&hout));
  if (pb_.samples) {
    samples_.assign(pb_.samples, pb_.samples + nsf);
    float *hin = nullptr;
    PUMP_TRY(ctx_->pinned(Ctx::kPinIn, sizeof(float) * (nsf + kDim), (void **)&hin));
    std::memcpy(hin, samples_.data(), sizeof(float) * nsf);
    for (int d = 0; d < kDim; ++d) hin[nsf + d] = pb_.goal[d];
    PUMP_CUDA_TRY(cudaMemcpyAsync(d_samples_.p, hin, sizeof(float) * (nsf + kDim),
                                  cudaMemcpyHostToDevice, s_));
  } else {
    PUMP_TRY(halton_samples_async(N_, pb_.lo, pb_.hi, pb_.init, pb_.goal, d_samples_.p, s_));
    PUMP_CUDA_TRY(cudaMemcpyAsync(hout + 2, d_samples_.p, sizeof(float) * nsf,
                                  cudaMemcpyDeviceToHost, s_));
  }
  // heuristic h (mainPUMP.cu:351-355): cost of the optimal connection of
  // node i to the goal (h[N-1] = 0), kept on the device for the search; h[0]
  // is read back with the roadmap's next synchronisation
  PUMP_TRY(d_h_.alloc(N_));
  PUMP_CUDA_TRY(cudaMemsetAsync(d_h_.p + (N_ - 1), 0, sizeof(float), s_));
  {
    BvpJobs jb{};
    jb.x0 = d_samples_.p;
    jb.x1 = d_samples_.p + nsf;
    jb.x1_same = 1;
    jb.n = N_ - 1;
    jb.jobs = 1;
    jb.tmax[0] = 5.0f;
    jb.cost[0] = d_h_.p;
    PUMP_TRY(bvp_jobs_launch(jb, host_bvp_mode(pb_.bvp_mode), s_));
  }
  PUMP_CUDA_TRY(cudaMemcpyAsync(hout, d_h_.p, sizeof(float), cudaMemcpyDeviceToHost, s_));
  const long long npairs = (long long)N_ * (N_ - 1);
  // mainPUMP.cu:261-262: (int)((NUM-1)*(NUM)*rnPerc) with rnPerc a float
  const long long rnIdx = (long long)((float)((long long)(N_ - 1) * N_) * (float)0.05);
  const long long cap = rnIdx > 0 ? rnIdx : 1;
  PUMP_TRY(d_src_.alloc(cap));
  PUMP_TRY(d_dst_.alloc(cap));
  PUMP_TRY(d_coptE_.alloc(cap));
  PUMP_TRY(d_toptE_.alloc(cap));
  PUMP_TRY(d_go_.alloc(N_ + 1));
  use_pv_ = false;
  if (shared_ && shared_->matches(pb_)) {
    PUMP_TRY(pair_costs_shared(rnIdx, cap));
  } else {
    PUMP_TRY(d_copts_.alloc(npairs));
    PUMP_TRY(d_topts_.alloc(npairs));
    // a batch worker (shared pairs or the lazy throughput form) shares the
    // GPU with the others: no cooperative launch
    PUMP_TRY(roadmap_pairs_edges(ctx_, d_samples_.p, N_, 5.0f, pb_.bvp_mode, rnIdx, cap, d_copts_.p,
                                 d_topts_.p, d_src_.p, d_dst_.p, d_coptE_.p, d_toptE_.p, d_go_.p,
                                 &rn_, &E_, s_, &d_pack_, nullptr, shared_ == nullptr && !lazy_));
  }
  // the edges' waypoints (findDiscretizedPath) are written by the edge
  // checks; with the edge count still on the device, sized for the capacity
  PUMP_TRY(d_disc_.alloc((size_t)(E_ >= 0 ? E_ : cap) * W_ * kDim));
  PUMP_TRY(d_scalar_.alloc(1));
  PUMP_TRY(max_degree_async(d_go_.p, N_, d_scalar_.p, s_));
  PUMP_CUDA_TRY(cudaMemcpyAsync(hout + 1, d_scalar_.p, sizeof(int), cudaMemcpyDeviceToHost, s_));
  RnEdgesPack *hpack = reinterpret_cast<RnEdgesPack *>(hout + 2 + nsf);
  if (d_pack_)
    PUMP_CUDA_TRY(cudaMemcpyAsync(hpack, d_pack_, sizeof(RnEdgesPack), cudaMemcpyDeviceToHost, s_));
  PUMP_TRY(sync());
  if (d_pack_) {
    const RnEdgesPack pk = *hpack;
    d_pack_ = nullptr;
    // the bracket sample misled the one-read pass: the exact select over all
    // pairs and the full compaction (rebuilding the row starts), then the
    // largest out-degree again
    auto fallback = [&]() -> pump_status_t {
      if (use_pv_)
        PUMP_TRY(rn_edges_fallback_pairs(ctx_, pv_, rnIdx, cap, d_src_.p, d_dst_.p, d_coptE_.p,
                                         d_toptE_.p, d_go_.p, &rn_, &E_, s_));
      else
        PUMP_TRY(rn_edges_fallback_device(ctx_, d_copts_.p, d_topts_.p, N_, rnIdx, cap, d_src_.p,
                                          d_dst_.p, d_coptE_.p, d_toptE_.p, d_go_.p, &rn_, &E_,
                                          s_));
      PUMP_TRY(max_degree_async(d_go_.p, N_, d_scalar_.p, s_));
      PUMP_CUDA_TRY(cudaMemcpyAsync(hout + 1, d_scalar_.p, sizeof(int), cudaMemcpyDeviceToHost, s_));
      return sync();
    };
    PUMP_TRY(rn_edges_unpack(pk, rnIdx, cap, &rn_, &E_, fallback));
  }
  res_->rn = rn_;
  res_->num_edges = E_;
  if (pb_.bvp_mode == PUMP_BVP_PARITY_GPU) {
    PUMP_TRY(d_toptH_.alloc(E_ > 0 ? E_ : 1));
    PUMP_TRY(edge_topts_parity_async(d_samples_.p, d_src_.p, d_dst_.p, E_, d_toptH_.p, s_));
  }
  if (pb_.disc_len > 0) {  // the waypoint array (sized for num_disc per edge) holds the ragged layout
    PUMP_TRY(d_disc_off_.alloc(E_ + 1));
    PUMP_TRY(d_disc_scratch_.alloc(disc_offsets_scratch(E_) / sizeof(long long) + 1));
    PUMP_TRY(disc_offsets_async(d_samples_.p, d_src_.p, d_dst_.p, E_, pb_.disc_len, pb_.disc_min,
                                pb_.num_disc, d_disc_off_.p, d_disc_scratch_.p, s_));
  }
  h0_ = hout[0];
  std::memcpy(&max_degree_, hout + 1, sizeof(int));
  if (!pb_.samples) samples_.assign(hout + 2, hout + 2 + nsf);
  return PUMP_OK;
}

// The query's pair costs from the batch's shared Halton pairs plus its own
// 4N-6 pairs touching init or goal (tmax 5, as pump_bvp_pairs): rn and the
// edges come out exactly as from the query's own N(N-1) pair arrays.
pump_status_t Planner::pair_costs_shared(long long rnIdx, long long cap) {
  const int N = N_;
  const size_t own = (size_t)(4 * N - 6);
  PUMP_TRY(d_bx0_.alloc(own * kDim));
  PUMP_TRY(d_bx1_.alloc(own * kDim));
  PUMP_TRY(own_pairs_async(d_samples_.p, N, d_bx0_.p, d_bx1_.p, s_));
  PUMP_TRY(d_own_c_.alloc(own));
  PUMP_TRY(d_own_t_.alloc(own));
  PUMP_TRY(pump_bvp_batch(d_bx0_.p, d_bx1_.p, (int)own, 5.0f, pb_.bvp_mode, d_own_t_.p, d_own_c_.p,
                          (pump_stream_t)s_));
  PairView &pv = pv_;
  pv.N = N;
  pv.M = shared_->M;
  pv.sc = shared_->d_copt;
  pv.st = shared_->d_topt;
  pv.irc = d_own_c_.p;
  pv.irt = d_own_t_.p;
  pv.icc = d_own_c_.p + (N - 1);
  pv.ict = d_own_t_.p + (N - 1);
  pv.grc = d_own_c_.p + 2 * (N - 1);
  pv.grt = d_own_t_.p + 2 * (N - 1);
  pv.gcc = d_own_c_.p + 2 * (N - 1) + (N - 2);
  pv.gct = d_own_t_.p + 2 * (N - 1) + (N - 2);
  use_pv_ = true;
  return rn_edges_pairs(ctx_, pv, rnIdx, cap, d_src_.p, d_dst_.p, d_coptE_.p, d_toptE_.p, d_go_.p,
                        &rn_, &E_, s_, &d_pack_);
}

pump_status_t Planner::online() {
  PUMP_TRY(d_obs_.alloc((size_t)nobs_ * 12));
  PUMP_TRY(h2d(d_obs_.p, pb_.obstacles, (size_t)nobs_ * 12));
  obs_p_ = d_obs_.p;
  PUMP_TRY(d_free_s_.alloc(N_));
  PUMP_TRY(pump_sample_free(d_obs_.p, nobs_, d_samples_.p, N_, d_free_s_.p, (pump_stream_t)s_));
  // freeEdges (mainPUMP.cu:364) and the waypoints it tests
  // (findDiscretizedPath, mainPUMP.cu:339).  Lazy: the search checks the
  // out-edges of each node when it first reaches it (search_check), so edges
  // it never expands are not checked and nothing it reads differs.  Eager:
  // all edges here, then every node's count of expandable edges.
  PUMP_TRY(d_free_e_.alloc(E_));
  PUMP_TRY(d_open_cnt_.alloc(N_));
  PUMP_TRY(d_todo_.alloc(N_));
  PUMP_CUDA_TRY(cudaMemsetAsync(d_open_cnt_.p, 0xFF, sizeof(int) * (size_t)N_, s_));  // -1
  if (!lazy_ && disc_off()) {
    PUMP_TRY(discretize_off_async(d_samples_.p, d_src_.p, d_dst_.p, waypoint_topts(), E_, disc_off(),
                                  pb_.num_disc, host_bvp_mode(pb_.bvp_mode), d_disc_.p, s_));
    PUMP_TRY(free_edges_off_async(d_obs_.p, nobs_, d_disc_.p, disc_off(), E_, pb_.num_disc,
                                  d_free_e_.p, s_));
  } else if (!lazy_) {
    PUMP_TRY(pump_discretize_edges(d_samples_.p, d_src_.p, d_dst_.p, waypoint_topts(), E_,
                                   pb_.num_disc, host_bvp_mode(pb_.bvp_mode), d_disc_.p,
                                   (pump_stream_t)s_));
    PUMP_TRY(pump_free_edges(d_obs_.p, nobs_, d_disc_.p, E_, pb_.num_disc, d_free_e_.p,
                             (pump_stream_t)s_));
  }
  if (!lazy_) {
    SearchDev sd{};
    sd.N = N_;
    sd.go = d_go_.p;
    sd.dst = d_dst_.p;
    sd.free_s = d_free_s_.p;
    sd.free_e = d_free_e_.p;
    sd.open_cnt = d_open_cnt_.p;
    PUMP_TRY(search_count_open(sd, s_));
  }
  // maxd2 = 0.1*offsetMult*offsetMult evaluated in double (mainPUMP.cu:201)
  maxd2_ = (float)(0.1 * (double)pb_.offset_mult * (double)pb_.offset_mult);
  // The half-spaces of cacheHalfspaces (mainPUMP.cu:366-374) are derived by
  // the HSMC kernel for the edges each wavefront propagates along
  if (!hsmc_boxes_fits(nobs_, W_, maxHS_))
    return set_error(PUMP_ERR_CAPACITY,
                     "%d boxes or %d waypoints x %d half-spaces exceed the HSMC shared-memory stage",
                     nobs_, W_, maxHS_);
  PUMP_TRY(ctx_->particle_table(pb_.seed, pb_.num_mc, pb_.table_rows, &d_table_, s_));
  d_rowmax_ = d_table_ + 3 * (size_t)pb_.num_mc * pb_.table_rows;
  return PUMP_OK;
}

// The search loop (PUMP.cu:39-290) with its state on the device
// (search.cu): per iteration the host launches the expansion scan, reads the
// wavefront size, launches expansion, HSMC, pruning and storing, and reads
// the iteration's counters back.
pump_status_t Planner::explore() {
  maxPathCount_ = pb_.max_paths > 0 ? pb_.max_paths
                                    : (int)(2 * N_ * std::sqrt((double)N_));  // mainPUMP.cu:623
  const int M = maxPathCount_;
  const size_t cap = (size_t)M + 1;
  PUMP_TRY(d_valid_.alloc((size_t)M * words_));
  PUMP_TRY(d_stage_.alloc(cap * words_));
  PUMP_TRY(d_cpStage_.alloc(cap));
  PUMP_TRY(d_pathTime_.alloc(cap));
  PUMP_TRY(d_wfPrev_.alloc(cap));
  PUMP_TRY(d_wfEdge_.alloc(cap));
  PUMP_TRY(d_err_.alloc(1));
  DevBuf<int> d_prev, d_node, d_g0, d_g1, d_nhead, d_nnext, d_wnode, d_wopen, d_newhead, d_newnext;
  DevBuf<float> d_cost, d_cp, d_ncost, d_ntime;
  DevBuf<unsigned int> d_off;
  DevBuf<uint8_t> d_alive;
  DevBuf<SearchCtl> d_ctl;
  PUMP_TRY(d_prev.alloc(cap));
  PUMP_TRY(d_node.alloc(cap));
  PUMP_TRY(d_cost.alloc(cap));
  PUMP_TRY(d_cp.alloc(cap));
  PUMP_TRY(d_g0.alloc(cap));
  PUMP_TRY(d_g1.alloc(cap));
  PUMP_TRY(d_nhead.alloc(N_));
  PUMP_TRY(d_nnext.alloc(cap));
  PUMP_TRY(d_wnode.alloc(cap));
  PUMP_TRY(d_wopen.alloc(cap));
  PUMP_TRY(d_off.alloc(cap));
  PUMP_TRY(d_ncost.alloc(cap));
  PUMP_TRY(d_ntime.alloc(cap));
  PUMP_TRY(d_alive.alloc(cap));
  PUMP_TRY(d_newhead.alloc(N_));
  PUMP_TRY(d_newnext.alloc(cap));
  PUMP_TRY(d_ctl.alloc(1));
  // The loop runs on the device as one graph launch (search_loop_graph)
  // unless the wavefront trace is wanted (the host reads it between the
  // expansion and the rest of each iteration).  Batch workers (lazy edge
  // checks) run it in groups of queries (batcher_), or drive it from the
  // host: with 12 workers each launching its own query's graph, the loops
  // took 1.6 ms per query against 0.95 ms host-driven (alone: 0.36 against
  // 0.39 ms).
  const int graph_level = search_graph_flag().load();
  const bool graph_loop =
      !res_->wf_trace && (batcher_ || graph_level >= 2 || (graph_level == 1 && !lazy_));
  if (!graph_loop) {
    PUMP_CUDA_TRY(cudaMemsetAsync(d_err_.p, 0, sizeof(int), s_));
    // setupValidParticles (PUMP.cu:766-777) for path 0: all particles valid
    PUMP_CUDA_TRY(cudaMemsetAsync(d_valid_.p, 0xFF, sizeof(uint32_t) * words_, s_));
    if (P_ % 32) {
      const uint32_t last = (1u << (P_ % 32)) - 1u;
      PUMP_TRY(h2d(d_valid_.p + words_ - 1, &last, 1));
    }
  }
  SearchDev sd{};
  sd.N = N_;
  sd.goal = N_ - 1;
  sd.go = d_go_.p;
  sd.dst = d_dst_.p;
  sd.copt = d_coptE_.p;
  sd.topt = d_toptE_.p;
  sd.free_s = d_free_s_.p;
  sd.free_e = d_free_e_.p;
  sd.open_cnt = d_open_cnt_.p;
  sd.todo = d_todo_.p;
  sd.h = d_h_.p;
  sd.path_prev = d_prev.p;
  sd.path_node = d_node.p;
  sd.path_cost = d_cost.p;
  sd.path_time = d_pathTime_.p;
  sd.path_cp = d_cp.p;
  sd.g_list[0] = d_g0.p;
  sd.g_list[1] = d_g1.p;
  sd.node_head = d_nhead.p;
  sd.node_next = d_nnext.p;
  sd.wf_prev = d_wfPrev_.p;
  sd.wf_node = d_wnode.p;
  sd.wf_edge = d_wfEdge_.p;
  sd.wf_open = d_wopen.p;
  sd.wf_off = d_off.p;
  sd.new_cost = d_ncost.p;
  sd.new_time = d_ntime.p;
  sd.new_cp = d_cpStage_.p;
  sd.alive = d_alive.p;
  sd.new_head = d_newhead.p;
  sd.new_next = d_newnext.p;
  sd.ctl = d_ctl.p;
  if (!graph_loop) PUMP_TRY(search_init(sd, s_));
  CheckArgs ca{};
  ca.samples = d_samples_.p;
  ca.disc = d_disc_.p;
  ca.numDisc = pb_.num_disc;
  ca.mode = host_bvp_mode(pb_.bvp_mode);
  ca.wp_topt = waypoint_topts();
  ca.disc_off = disc_off();
  ca.obs = d_obs_.p;
  ca.numObs = nobs_;
  ca.max_degree = max_degree_;

  // PUMP.cu:10-35
  const float cpTarget = pb_.cp_target;
  const float dr = lambda_ * rn_;
  const float cpMinSoln = cpTarget / pb_.cp_factor;
  const float cpCutoff = cpTarget * pb_.cp_factor;
  int Gidx = 0;
  int gCount[2] = {1, 0};
  numPaths_ = 1;
  float costThreshold = h0_;
  const int maxItrs = maxItrs_;
  int itrs = 0;
  long long considered = 0;
  std::vector<int> trace_prev, trace_edge;
  pump_status_t status = PUMP_OK;
  const HsmcEpilogue epi = search_hsmc_epilogue(sd, cpCutoff);
  // nodes listed for edge checks: the initial node, then at most the paths
  // the last iteration stored
  int maxTodo = 1;
  SearchCtl ctl{};
  SearchCtl *hctl = nullptr;  // pinned read-back of the iteration's counters
  PUMP_TRY(ctx_->pinned(Ctx::kPinCtl, sizeof(SearchCtl), (void **)&hctl));
  LoopTiles scanT{}, storeT{};
  if (graph_loop) {
    const auto tw = clk::now();
    PUMP_TRY(explore_graph(sd, ca, epi, M, cpCutoff, cpMinSoln, dr, &itrs, &considered, &status));
    res_->ms_explore_wait += ms_since(tw);
  } else {
    // the tile scratch of the scan and the store pass, zeroed once here and
    // then by each iteration's expansion kernel
    char *base = nullptr;
    size_t args_b = 0;
    PUMP_TRY(loop_region(M, &base, &args_b, &scanT, &storeT));
    PUMP_CUDA_TRY(cudaMemsetAsync(base + args_b, 0,
                                  sizeof(unsigned long long) * (size_t)(loop_tile_words(scanT.cap) +
                                                                        loop_tile_words(storeT.cap)),
                                  s_));
  }
  while (!graph_loop && itrs < maxItrs) {
    ++itrs;
    const int nG = gCount[Gidx];
    const auto tw = clk::now();
    if (nG == 0) {  // nothing to expand: an empty wavefront (PUMP.cu:66-70)
      if (itrs <= 32) res_->wavefront_sizes[itrs - 1] = 0;
      break;
    }
    // expansion (PUMP.cu:47-66).  The wavefront size stays on the device:
    // HSMC, pruning and storing read it there (and do nothing when the
    // iteration would overflow the path store), so the host waits once per
    // iteration, for the counters.
    // edge checks of the nodes listed so far (the initial node, then the
    // nodes first reached by the last iteration's stored paths)
    if (lazy_) PUMP_TRY(search_check(sd, maxTodo, ca, s_));
    PUMP_TRY(search_expand(sd, Gidx, nG, numPaths_, M, scanT, storeT, s_));
    if (res_->wf_trace) {
      unsigned long long nn = 0;
      PUMP_TRY(d2h(&nn, &d_ctl.p->num_new, 1));
      PUMP_TRY(sync());
      const int nt = nn <= (unsigned long long)M && numPaths_ + (long long)nn < M ? (int)nn : 0;
      trace_prev.resize(nt);
      trace_edge.resize(nt);
      PUMP_TRY(d2h(trace_prev.data(), d_wfPrev_.p, nt));
      PUMP_TRY(d2h(trace_edge.data(), d_wfEdge_.p, nt));
      PUMP_TRY(sync());
      for (int i = 0; i < nt && res_->wf_trace_len + 2 <= res_->wf_trace_cap; ++i) {
        res_->wf_trace[res_->wf_trace_len++] = trace_prev[i];
        res_->wf_trace[res_->wf_trace_len++] = trace_edge[i];
      }
    }
    // HSMC of the wavefront (PUMP.cu:82-160).  The wavefront holds at most
    // the bucket's paths times the largest out-degree (and at most M).
    const unsigned long long *d_nn = &d_ctl.p->num_new;
    const int *d_ovf = &d_ctl.p->overflow;
    const long long bound = (long long)nG * (max_degree_ > 0 ? max_degree_ : 1);
    const int maxNew = bound < M ? (int)bound : M;
    PUMP_TRY(hsmc_boxes_async(maxNew, W_, d_wfEdge_.p, d_wfPrev_.p, E_, numPaths_, d_obs_.p, nobs_,
                              d_disc_.p, maxd2_, maxHS_, d_pathTime_.p, d_toptE_.p, dt_, d_table_,
                              pb_.num_mc, pb_.table_rows, pb_.offset_mult, d_valid_.p, d_stage_.p,
                              P_, d_cpStage_.p, d_err_.p, s_, d_nn, d_ovf, &epi, disc_off()));
    // cut-off (written by the HSMC kernel), dominance and storing, buckets
    // (PUMP.cu:164-256)
    // the store pass's last block leaves the counters in hctl (pinned)
    const unsigned int sq = next_seq();
    *reinterpret_cast<volatile unsigned int *>(&hctl->seq) = sq - 1u;
    PUMP_TRY(search_store(sd, maxNew, numPaths_, Gidx, costThreshold, dr, cpMinSoln, epsCP_,
                          epsCost_, d_stage_.p,
                          d_valid_.p, words_, storeT, scanT, hctl, sq, s_));
    res_->d2h_bytes += (long long)sizeof(SearchCtl);
    PUMP_TRY(wait_seq(&hctl->seq, sq));
    ctl = *hctl;
    res_->ms_explore_wait += ms_since(tw);
    if (ctl.overflow == 1) {
      status = set_error(PUMP_ERR_CAPACITY, "wavefront exceeds maxPathCount %d", M);
      break;
    }
    const int numNew = (int)ctl.num_new;
    if (itrs <= 32) res_->wavefront_sizes[itrs - 1] = numNew;
    if (numNew == 0) break;
    if (ctl.overflow == 2) {
      status = set_error(PUMP_ERR_CAPACITY, "paths exceed maxPathCount %d", M);
      break;
    }
    considered += numNew;
    if (ctl.wait_error) {
      status = set_error(PUMP_ERR_TIMEOUT, "search store: look-back wait exceeded its bound");
      break;
    }
    numPaths_ += (int)ctl.num_valid;
    maxTodo = (int)ctl.num_valid;
    gCount[0] = ctl.g_count[0];
    gCount[1] = ctl.g_count[1];
    // goal and open-set conditions (PUMP.cu:259-288)
    if (ctl.goal_found) break;
    if (gCount[0] == 0 && gCount[1] == 0) break;
    Gidx = (Gidx + 1) % numBuckets_;
    costThreshold += dr;
    if (numPaths_ >= M) {
      status = set_error(PUMP_ERR_CAPACITY, "paths reached maxPathCount %d", M);
      break;
    }
  }
  // stored paths back to the host for the solution search, in one pinned
  // read-back: prev | node | cost | the particle-table error word
  const size_t np = (size_t)numPaths_;
  int *hp = nullptr;
  PUMP_TRY(ctx_->pinned(Ctx::kPinPaths, sizeof(int) * (3 * np + 1), (void **)&hp));
  res_->d2h_bytes += (long long)(sizeof(int) * (3 * np + 1));
  PUMP_CUDA_TRY(cudaMemcpyAsync(hp, d_prev.p, sizeof(int) * np, cudaMemcpyDeviceToHost, s_));
  PUMP_CUDA_TRY(cudaMemcpyAsync(hp + np, d_node.p, sizeof(int) * np, cudaMemcpyDeviceToHost, s_));
  PUMP_CUDA_TRY(cudaMemcpyAsync(hp + 2 * np, d_cost.p, sizeof(float) * np, cudaMemcpyDeviceToHost, s_));
  PUMP_CUDA_TRY(cudaMemcpyAsync(hp + 3 * np, d_err_.p, sizeof(int), cudaMemcpyDeviceToHost, s_));
  // the stored paths' times and particle masks, when the caller asked for them
  if (np > 0 && res_->path_state_cap >= (int)np) {
    if (res_->path_time) {
      PUMP_CUDA_TRY(cudaMemcpyAsync(res_->path_time, d_pathTime_.p, sizeof(float) * np,
                                    cudaMemcpyDeviceToHost, s_));
      res_->d2h_bytes += (long long)(sizeof(float) * np);
    }
    if (res_->path_valid) {
      PUMP_CUDA_TRY(cudaMemcpyAsync(res_->path_valid, d_valid_.p, sizeof(uint32_t) * np * words_,
                                    cudaMemcpyDeviceToHost, s_));
      res_->d2h_bytes += (long long)(sizeof(uint32_t) * np * words_);
    }
  }
  PUMP_TRY(sync());
  pathPrev_.assign(hp, hp + np);
  pathNode_.assign(hp + np, hp + 2 * np);
  pathCost_.resize(np);
  std::memcpy(pathCost_.data(), hp + 2 * np, sizeof(float) * np);
  const int err = hp[3 * np];
  atNode_.assign(N_, std::vector<int>());
  for (int p = 0; p < numPaths_; ++p)
    if (pathNode_[p] == N_ - 1) atNode_[N_ - 1].push_back(p);
  res_->iterations = itrs;
  res_->num_paths = numPaths_;
  res_->num_considered = (int)considered;
  res_->goal_paths = (int)atNode_[N_ - 1].size();
  if (err) return set_error((pump_status_t)err, "particle table has too few rows for a path time");
  return status;
}

pump_status_t Planner::loop_region(int M, char **base, size_t *args_b, LoopTiles *scan,
                                   LoopTiles *store) {
  // tile capacities of the scan (over a bucket) and the store pass (over a
  // wavefront), both at most M + 1 items, in power-of-two classes
  auto pow2 = [](long long v) {
    long long c = 64;
    while (c < v) c <<= 1;
    return c;
  };
  const long long scan_cap = pow2((M + 1 + kLoopScanTile - 1) / kLoopScanTile + 1);
  const long long store_cap = pow2((M + 1 + kLoopStoreTile - 1) / kLoopStoreTile + 1);
  auto round256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
  // the argument block, then the one-query group of this context's graphs
  *args_b = round256(sizeof(LoopArgs)) + round256(sizeof(LoopGroup));
  const size_t scan_b = sizeof(unsigned long long) * (size_t)loop_tile_words(scan_cap);
  const size_t store_b = sizeof(unsigned long long) * (size_t)loop_tile_words(store_cap);
  PUMP_TRY(ctx_->scratch(Ctx::kLoop, *args_b + scan_b + store_b, (void **)base));
  auto tiles_at = [](char *p, long long cap) {
    LoopTiles t{};
    t.total = reinterpret_cast<unsigned long long *>(p);
    t.status = t.total + 1;
    t.tile_counter = reinterpret_cast<unsigned int *>(t.status + cap + 1);
    t.error = reinterpret_cast<int *>(t.tile_counter + 1);
    t.done = reinterpret_cast<unsigned int *>(t.error + 1);
    t.cap = cap;
    return t;
  };
  *scan = tiles_at(*base + *args_b, scan_cap);
  *store = tiles_at(*base + *args_b + scan_b, store_cap);
  return PUMP_OK;
}

pump_status_t Planner::explore_graph(const SearchDev &sd, const CheckArgs &ca,
                                     const HsmcEpilogue &epi, int M, float cpCutoff,
                                     float cpMinSoln, float dr, int *itrs, long long *considered,
                                     pump_status_t *status) {
  char *base = nullptr;
  size_t args_b = 0;
  LoopTiles scan{}, store{};
  PUMP_TRY(loop_region(M, &base, &args_b, &scan, &store));
  const long long scan_cap = scan.cap, store_cap = store.cap;
  // pinned staging of the argument block and of the one-query group
  const size_t group_off = (sizeof(LoopArgs) + 255) & ~(size_t)255;
  LoopArgs *la = nullptr;
  PUMP_TRY(ctx_->pinned(Ctx::kPinLoop, group_off + sizeof(LoopGroup), (void **)&la));
  std::memset(la, 0, group_off + sizeof(LoopGroup));
  la->sd = sd;
  la->ca = ca;
  la->scan = scan;
  la->store = store;
  la->cp_min_soln = cpMinSoln;
  la->eps_cp = epsCP_;
  la->eps_cost = epsCost_;
  la->cp_cutoff = cpCutoff;
  la->stage = d_stage_.p;
  la->valid = d_valid_.p;
  la->words = words_;
  la->P = P_;
  la->err = d_err_.p;
  PUMP_TRY(hsmc_boxes_fill(M, W_, d_wfEdge_.p, d_wfPrev_.p, E_, 1, d_obs_.p, nobs_, d_disc_.p,
                           maxd2_, maxHS_, d_pathTime_.p, d_toptE_.p, dt_, d_table_, pb_.num_mc,
                           pb_.table_rows, pb_.offset_mult, d_valid_.p, d_stage_.p, P_,
                           d_cpStage_.p, d_err_.p, &sd.ctl->num_new, &sd.ctl->overflow, &epi,
                           &la->hp, disc_off()));
  LoopState &L = la->L;
  L.max_itrs = maxItrs_;
  L.max_paths = M;
  L.dr = dr;
  L.itrs = 1;
  L.g_idx = 0;
  L.n_g = 1;
  L.num_paths = 1;
  L.cost_threshold = h0_;
  L.g_count[0] = 1;
  LoopArgs *d_args = reinterpret_cast<LoopArgs *>(base);
  // shared memory sized for the box count rounded up to 32 (exact for large
  // maps, which sit close to the shared-memory limit)
  const int obs_cap = nobs_ > 1024 ? nobs_ : (nobs_ <= 32 ? 32 : ((nobs_ + 31) / 32) * 32);
  const int lazy = lazy_ ? 1 : 0, mode = host_bvp_mode(pb_.bvp_mode), num_disc = pb_.num_disc;
  if (batcher_) {
    // the loop runs in the group the batcher launches, after this stream's
    // work up to the argument block
    res_->h2d_bytes += (long long)sizeof(LoopArgs);
    PUMP_CUDA_TRY(cudaMemcpyAsync(base, la, sizeof(LoopArgs), cudaMemcpyHostToDevice, s_));
    if (!ctx_->loop_ready)
      PUMP_CUDA_TRY(cudaEventCreateWithFlags(&ctx_->loop_ready, cudaEventDisableTiming));
    PUMP_CUDA_TRY(cudaEventRecord(ctx_->loop_ready, s_));
    const LoopShape shape{lazy, mode, obs_cap, num_disc, maxHS_, pb_.num_hsmc};
    PUMP_TRY(batcher_->run(d_args, shape, ctx_->loop_ready));
    return loop_result(d_args, M, itrs, considered, status);
  }
  LoopGroup *hg = reinterpret_cast<LoopGroup *>(reinterpret_cast<char *>(la) + group_off);
  hg->args[0] = d_args;
  hg->nq = 1;
  LoopGroup *d_group = reinterpret_cast<LoopGroup *>(base + group_off);
  res_->h2d_bytes += (long long)(group_off + sizeof(LoopGroup));
  PUMP_CUDA_TRY(cudaMemcpyAsync(base, la, group_off + sizeof(LoopGroup), cudaMemcpyHostToDevice, s_));
  // the context's graph for this shape class (built on first use)
  std::vector<Ctx::LoopGraph> &gs = ctx_->loop_graphs;
  for (size_t i = 0; i < gs.size();) {  // graphs of an outgrown argument block
    if (gs[i].base != base) {
      cudaGraphExecDestroy(gs[i].exec);
      gs.erase(gs.begin() + (long)i);
    } else {
      ++i;
    }
  }
  cudaGraphExec_t exec = nullptr;
  for (const Ctx::LoopGraph &g : gs)
    if (g.lazy == lazy && g.mode == mode && g.obs_cap == obs_cap && g.num_disc == num_disc &&
        g.max_hs == maxHS_ && g.particles == pb_.num_hsmc && g.scan_cap == scan_cap &&
        g.store_cap == store_cap)
      exec = g.exec;
  if (!exec) {
    if (!ctx_->capture_stream)
      PUMP_CUDA_TRY(cudaStreamCreateWithFlags(&ctx_->capture_stream, cudaStreamNonBlocking));
    PUMP_TRY(search_loop_graph(d_group, 1, lazy_, mode, obs_cap, num_disc, maxHS_, pb_.num_hsmc,
                               ctx_->capture_stream, &exec));
    gs.push_back({lazy, mode, obs_cap, num_disc, maxHS_, pb_.num_hsmc, scan_cap, store_cap, base,
                  exec});
  }
  PUMP_CUDA_TRY(cudaGraphLaunch(exec, s_));
  return loop_result(d_args, M, itrs, considered, status);
}

pump_status_t Planner::loop_result(const LoopArgs *d_args, int M, int *itrs,
                                   long long *considered, pump_status_t *status) {
  LoopState *hl = nullptr;
  PUMP_TRY(ctx_->pinned(Ctx::kPinCtl, sizeof(LoopState), (void **)&hl));
  res_->d2h_bytes += (long long)sizeof(LoopState);
  PUMP_CUDA_TRY(cudaMemcpyAsync(hl, &d_args->L, sizeof(LoopState), cudaMemcpyDeviceToHost, s_));
  PUMP_TRY(sync());
  const LoopState r = *hl;
  *itrs = r.itrs;
  *considered = r.considered;
  numPaths_ = r.num_paths;
  for (int k = 0; k < 32 && k < r.itrs; ++k) res_->wavefront_sizes[k] = r.wavefront_sizes[k];
  switch (r.status) {
    case kLoopWavefrontOverflow:
      *status = set_error(PUMP_ERR_CAPACITY, "wavefront exceeds maxPathCount %d", M);
      break;
    case kLoopPathsWouldOverflow:
      *status = set_error(PUMP_ERR_CAPACITY, "paths exceed maxPathCount %d", M);
      break;
    case kLoopWaitError:
      *status = set_error(PUMP_ERR_TIMEOUT, "search store: look-back wait exceeded its bound");
      break;
    case kLoopPathsFull:
      *status = set_error(PUMP_ERR_CAPACITY, "paths reached maxPathCount %d", M);
      break;
    default:
      *status = PUMP_OK;
  }
  return PUMP_OK;
}

std::vector<float> Planner::node_states(int path_idx, std::vector<int> *nodes) const {
  std::vector<int> seq;
  for (int p = path_idx; p != -2; p = pathPrev_[p]) seq.push_back(pathNode_[p]);
  std::reverse(seq.begin(), seq.end());
  std::vector<float> xs(seq.size() * kDim);
  for (size_t k = 0; k < seq.size(); ++k)
    for (int d = 0; d < kDim; ++d) xs[k * kDim + d] = samples_[(size_t)seq[k] * kDim + d];
  if (nodes) *nodes = seq;
  return xs;
}

pump_status_t Planner::topts_of(const std::vector<float> &x0, const std::vector<float> &x1,
                                float tmax, std::vector<float> *topt, std::vector<float> *cost) {
  const int n = (int)(x0.size() / kDim);
  if (topt) topt->assign(n, 0.0f);
  if (cost) cost->assign(n, 0.0f);
  if (n == 0) return PUMP_OK;
  PUMP_TRY(d_bx0_.alloc(x0.size()));
  PUMP_TRY(d_bx1_.alloc(x1.size()));
  PUMP_TRY(d_bt_.alloc(n));
  PUMP_TRY(d_bc_.alloc(n));
  PUMP_TRY(h2d(d_bx0_.p, x0.data(), x0.size()));
  PUMP_TRY(h2d(d_bx1_.p, x1.data(), x1.size()));
  PUMP_TRY(pump_bvp_batch(d_bx0_.p, d_bx1_.p, n, tmax, host_bvp_mode(pb_.bvp_mode), d_bt_.p, d_bc_.p,
                          (pump_stream_t)s_));
  if (topt) PUMP_TRY(d2h(topt->data(), d_bt_.p, n));
  if (cost) PUMP_TRY(d2h(cost->data(), d_bc_.p, n));
  return sync();
}

pump_status_t Planner::eval_launch(CandSet &c, const std::vector<std::vector<float>> &xs,
                                   float dt, int rows_cap, bool with_cost, bool with_cp,
                                   bool with_topts, int states_rows) {
  const int n = (int)xs.size();
  c.n = n;
  c.segs = 0;
  c.states_rows = n > 0 ? states_rows : 0;
  c.with_cost = with_cost;
  c.with_cp = with_cp;
  c.with_topts = with_topts;
  c.table_rows = pb_.table_rows;
  c.num_mc = pb_.num_mc;
  c.hout = nullptr;
  if (n == 0) return PUMP_OK;
  // one upload through pinned memory: the segments' start states | their end
  // states | per path node counts, first segments, dense-path offsets
  int segs = 0, max_segs = 0;
  for (int k = 0; k < n; ++k) {
    const int cnt = (int)(xs[k].size() / kDim);
    const int ns = cnt > 1 ? cnt - 1 : 0;
    segs += ns;
    max_segs = ns > max_segs ? ns : max_segs;
  }
  c.segs = segs;
  const size_t sf = (size_t)segs * kDim;
  const size_t in_bytes = sizeof(float) * 2 * sf + sizeof(int) * 3 * (size_t)n;
  char *hin = nullptr;
  PUMP_TRY(ctx_->pinned(c.pin_in, in_bytes, (void **)&hin));
  float *hx0 = reinterpret_cast<float *>(hin);
  float *hx1 = hx0 + sf;
  int *hints = reinterpret_cast<int *>(hin + sizeof(float) * 2 * sf);
  for (int k = 0, sg = 0; k < n; ++k) {
    const int cnt = (int)(xs[k].size() / kDim);
    hints[k] = cnt;
    hints[n + k] = sg;
    hints[2 * n + k] = k * rows_cap;
    for (int i = 0; i + 1 < cnt; ++i, ++sg) {
      std::memcpy(hx0 + (size_t)sg * kDim, xs[k].data() + (size_t)i * kDim, sizeof(float) * kDim);
      std::memcpy(hx1 + (size_t)sg * kDim, xs[k].data() + (size_t)(i + 1) * kDim,
                  sizeof(float) * kDim);
    }
  }
  PUMP_TRY(c.in.alloc(in_bytes / sizeof(float) + 1));
  PUMP_CUDA_TRY(cudaMemcpyAsync(c.in.p, hin, in_bytes, cudaMemcpyHostToDevice, s_));
  const int *d_ints = reinterpret_cast<const int *>(c.in.p + 2 * sf);
  const size_t sg = segs > 0 ? (size_t)segs : 1;
  PUMP_TRY(c.segcost.alloc(sg));
  // results read back in one copy: MC hit counts | lengths | costs, then the
  // segments' optimal times with tmax 5 and (with_topts) 2
  const size_t seg_f = with_topts ? (size_t)segs : 0;
  PUMP_TRY(c.out.alloc(3 * (size_t)n + sg + seg_f + 1));  // + the MC CP's finished-block count
  PUMP_TRY(c.states.alloc((size_t)n * rows_cap * kDim));
  float *d_topt = reinterpret_cast<float *>(c.out.p + 3 * (size_t)n);
  CandidateBufs cb{};
  cb.node_cnt = d_ints;
  cb.seg_base = d_ints + n;
  cb.x0 = c.in.p;
  cb.x1 = c.in.p + sf;
  cb.topt = d_topt;
  cb.topt2 = with_topts ? d_topt + segs : nullptr;
  cb.seg_cost = c.segcost.p;
  cb.states = c.states.p;
  cb.hits = with_cp ? c.out.p : nullptr;
  // pinned read-back: 3n ints | 2 segs floats (with_topts) | states_rows x 6
  // floats of path 0.  With the MC CP, its last block copies the head (a
  // single launch holds at most 65535 paths).
  // (then the completion word, then the states at a 16-byte boundary)
  const size_t st_f = (size_t)c.states_rows * kDim;
  const size_t head = sizeof(int) * 3 * (size_t)n + sizeof(float) * 2 * seg_f;
  const size_t head_words = head / sizeof(int);
  const size_t st_off = (head + sizeof(unsigned int) + 15) & ~(size_t)15;
  const bool copy_out = with_cp && n <= 65535;
  char *hout = nullptr;
  PUMP_TRY(ctx_->pinned(c.pin_out, st_off + sizeof(float) * st_f, (void **)&hout));
  cb.done = copy_out ? reinterpret_cast<unsigned int *>(c.out.p + head_words) : nullptr;
  c.head_bytes = head;
  c.seq = copy_out ? next_seq() : 0u;
  if (copy_out) *reinterpret_cast<volatile unsigned int *>(hout + head) = c.seq - 1u;
  cb.len = c.out.p + n;
  cb.cost = reinterpret_cast<float *>(c.out.p + 2 * n);
  PUMP_TRY(candidate_paths_async(cb, n, segs, max_segs, pb_.bvp_mode, dt, with_cost, rows_cap, s_));
  if (with_cp)
    PUMP_TRY(mc_cp_hits_async(c.states.p, d_ints + 2 * n, cb.len, n, d_table_, pb_.num_mc,
                              pb_.table_rows, pb_.offset_mult, obs_p_, nobs_, cb.hits, s_,
                              d_rowmax_, copy_out ? c.out.p : nullptr,
                              copy_out ? reinterpret_cast<int *>(hout) : nullptr,
                              (int)head_words, cb.done, c.seq));
  if (!copy_out)
    PUMP_CUDA_TRY(cudaMemcpyAsync(hout, c.out.p, head, cudaMemcpyDeviceToHost, s_));
  if (st_f > 0)
    PUMP_CUDA_TRY(cudaMemcpyAsync(hout + st_off, c.states.p, sizeof(float) * st_f,
                                  cudaMemcpyDeviceToHost, s_));
  c.hout = hout;
  return PUMP_OK;
}

void Planner::eval_read(const CandSet &c, CandResult *r) const {
  const int n = c.n;
  r->len.assign(n, 0);
  r->cost.assign(n, 0.0f);
  r->cp.assign(n, 0.0f);
  r->t5.clear();
  r->t2.clear();
  r->states.clear();
  if (n == 0 || !c.hout) return;
  const int *hi = reinterpret_cast<const int *>(c.hout);
  const float *hf = reinterpret_cast<const float *>(c.hout + sizeof(int) * 3 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    r->len[k] = hi[n + k];
    if (c.with_cost) std::memcpy(&r->cost[k], &hi[2 * n + k], sizeof(float));
    // collisionProbability.cu:89-91: hits / Pmc in binary32; a path longer
    // than the particle table has no CP
    if (c.with_cp)
      r->cp[k] = r->len[k] > c.table_rows ? -1.0f : ((float)hi[k]) / ((float)c.num_mc);
  }
  const size_t seg_f = c.with_topts ? (size_t)c.segs : 0;
  if (seg_f > 0) {
    r->t5.assign(hf, hf + seg_f);
    r->t2.assign(hf + seg_f, hf + 2 * seg_f);
  }
  if (c.states_rows > 0) {
    const float *hs = reinterpret_cast<const float *>(
        c.hout + ((c.head_bytes + sizeof(unsigned int) + 15) & ~(size_t)15));
    r->states.assign(hs, hs + (size_t)c.states_rows * kDim);
  }
}

pump_status_t Planner::eval_candidates(const std::vector<std::vector<float>> &xs, float dt,
                                      int rows_cap, bool with_cost, bool with_cp,
                                      std::vector<int> &len, std::vector<float> &cost,
                                      std::vector<float> &cp) {
  PUMP_TRY(eval_launch(cs_, xs, dt, rows_cap, with_cost, with_cp, false, 0));
  PUMP_TRY(wait_cand(cs_));
  CandResult r;
  eval_read(cs_, &r);
  len.swap(r.len);
  cost.swap(r.cost);
  cp.swap(r.cp);
  return PUMP_OK;
}

pump_status_t Planner::search_and_smooth() {
  const int goalIdx = N_ - 1;
  const float cpTarget = pb_.cp_target;
  // goal candidates in (cost, path index) order (PUMP.cu:355-362)
  std::vector<std::pair<float, int>> goalPaths;
  for (int pi : atNode_[goalIdx]) goalPaths.push_back(std::make_pair(pathCost_[pi], pi));
  std::sort(goalPaths.begin(), goalPaths.end());
  std::vector<std::vector<float>> cand;
  for (auto &g : goalPaths) cand.push_back(node_states(g.second, nullptr));
  const int rowsCap = pb_.table_rows;
  // One round trip for the goal candidates' dense lengths and MC CPs, their
  // segments' optimal times with tmax 2 (the smoothing's split of the chosen
  // path, PUMP.cu:445-450), and the unconstrained optimal path from init to
  // goal at dt / 10 (PUMP.cu:434-441), which depends only on those two
  // states (every goal path runs from the initial node to the goal node).
  const int dtMult = 10;
  const int optCap = pb_.table_rows * dtMult;
  if (!cand.empty()) {
    std::vector<std::vector<float>> two(1);
    two[0].insert(two[0].end(), cand[0].begin(), cand[0].begin() + kDim);
    two[0].insert(two[0].end(), cand[0].end() - kDim, cand[0].end());
    PUMP_TRY(eval_launch(co_, two, dt_ / dtMult, optCap, false, false, false, optCap));
  }
  PUMP_TRY(eval_launch(cs_, cand, dt_, rowsCap, false, true, true, 0));
  // the optimal path's copies precede the candidates' kernels in the stream
  PUMP_TRY(wait_cand(cs_));
  CandResult gr;
  eval_read(cs_, &gr);
  const std::vector<int> &glen = gr.len;
  const std::vector<float> &gcp = gr.cp;
  int sel = -1;
  for (size_t k = 0; k < goalPaths.size(); ++k) {
    if (gcp[k] < 0)
      return set_error(PUMP_ERR_CAPACITY, "goal path of %d states exceeds the %d-row particle table",
                       glen[k], pb_.table_rows);
    if (gcp[k] < cpTarget) { sel = (int)k; break; }
  }
  const int last = sel >= 0 ? sel : (int)goalPaths.size() - 1;
  const bool success = sel >= 0;
  res_->success = success ? 1 : 0;
  res_->soln_path_idx = last >= 0 ? goalPaths[last].second : -1;
  float solnPathCP = last >= 0 ? gcp[last] : 0.0f;
  float solnPathCost = last >= 0 ? pathCost_[goalPaths[last].second] : 0.0f;
  std::vector<int> nodes;
  std::vector<float> xs = last >= 0 ? node_states(goalPaths[last].second, &nodes) : std::vector<float>();
  res_->num_nodes = (int)nodes.size();
  if (res_->nodes)
    for (int k = 0; k < (int)nodes.size() && k < res_->nodes_cap; ++k) res_->nodes[k] = nodes[k];

  // smoothing (PUMP.cu:406-545); xsFinal is the reference's xsSmooth after
  // the loop: the last iterate evaluated, zeros if smoothing did not run.
  // finalT5 / finalT2: its segments' optimal times (tmax 5, 2) from that
  // evaluation, for the controller path.
  std::vector<float> xsFinal(xs.size(), 0.0f);
  std::vector<float> finalT5, finalT2;
  bool haveFinalT = false;
  std::vector<float> xsBest(xs);  // nodes of the path kept so far
  // the dense path kept so far stays on the device (d_best_) until the end
  std::vector<float> bestPath;
  int bestLen = last >= 0 ? glen[last] : 0;
  PUMP_TRY(d_best_.alloc((size_t)rowsCap * kDim));
  auto keep_best = [&](int k, int len) -> pump_status_t {
    PUMP_CUDA_TRY(cudaMemcpyAsync(d_best_.p, cs_.states.p + (size_t)k * rowsCap * kDim,
                                  sizeof(float) * kDim * (size_t)len, cudaMemcpyDeviceToDevice,
                                  s_));
    return PUMP_OK;
  };
  if (last >= 0 && bestLen > 0) PUMP_TRY(keep_best(last, bestLen));
  float lastCP = solnPathCP, lastCost = solnPathCost;
  if (success) {
    const int n = (int)(xs.size() / kDim);
    CandResult orr;
    eval_read(co_, &orr);
    const int optLen = orr.len[0];
    if (optLen > optCap)
      return set_error(PUMP_ERR_CAPACITY, "unconstrained optimal path of %d states exceeds %d",
                       optLen, optCap);
    // splitPathTopts with tmax 2 (PUMP.cu:445-450): the chosen candidate's
    // segments, which follow those of the candidates before it
    size_t sbase = 0;
    for (int k = 0; k < last; ++k) {
      const size_t cnt = cand[k].size() / kDim;
      sbase += cnt > 1 ? cnt - 1 : 0;
    }
    std::vector<float> splitT(n, 0.0f);
    for (int i = 0; i + 1 < n; ++i) splitT[i + 1] = splitT[i] + gr.t2[sbase + i];
    std::vector<float> xsOpt((size_t)n * kDim);
    for (int i = 0; i < n; ++i) {
      const int idx = (int)((optLen - 1) * splitT[i] / splitT[n - 1]);
      for (int d = 0; d < kDim; ++d) xsOpt[(size_t)i * kDim + d] = orr.states[(size_t)idx * kDim + d];
    }
    const float epsSmoothCP = (float)0.0002;
    float alpha = 1.0f, alphaU = 1.0f, alphaL = 0.0f;
    // The alpha bisection is sequential (each step's alpha depends on the
    // previous CP), but every step is a pure function of alpha.  So the 2^D - 1
    // alphas the next D steps can visit are evaluated in one batch (dense
    // paths, costs and MC CPs of all of them), then the reference's decisions
    // are replayed in order over the results: the same sequence of alphas,
    // best-path updates and early exit as PUMP.cu:492-541.  D = 3 (7 paths
    // per batch): deeper batches save round trips but most of their Monte
    // Carlo work is for alphas the bisection never visits.
    const int D = 3, K = (1 << D) - 1;
    int it = 0;
    bool stop = false;
    while (it < 30 && !stop) {
      // tree node k (heap order): children 2k+1 (cp < target) and 2k+2
      std::vector<float> nl(K), nu(K), na(K);
      nl[0] = alphaL; nu[0] = alphaU; na[0] = alpha;
      for (int k = 0; 2 * k + 2 < K; ++k) {
        nl[2 * k + 1] = na[k]; nu[2 * k + 1] = nu[k];
        na[2 * k + 1] = (nl[2 * k + 1] + nu[2 * k + 1]) / 2;
        nl[2 * k + 2] = nl[k]; nu[2 * k + 2] = na[k];
        na[2 * k + 2] = (nl[2 * k + 2] + nu[2 * k + 2]) / 2;
      }
      std::vector<std::vector<float>> cand(K, std::vector<float>(xs.size()));
      for (int k = 0; k < K; ++k)
        for (size_t i = 0; i < xs.size(); ++i) cand[k][i] = (1 - na[k]) * xs[i] + na[k] * xsOpt[i];
      PUMP_TRY(eval_launch(cs_, cand, dt_, rowsCap, true, true, true, 0));
      PUMP_TRY(wait_cand(cs_));
      CandResult sr;
      eval_read(cs_, &sr);
      int k = 0;
      for (int depth = 0; depth < D && it < 30; ++depth, ++it) {
        const float smoothCost = sr.cost[k];
        const float cp = sr.cp[k];
        if (cp < 0)
          return set_error(PUMP_ERR_CAPACITY, "smoothed path of %d states exceeds the %d-row particle table",
                           sr.len[k], pb_.table_rows);
        xsFinal = cand[k];
        // every candidate has n nodes, so candidate k's segments start at k (n - 1)
        finalT5.assign(sr.t5.begin() + (size_t)k * (n - 1), sr.t5.begin() + (size_t)(k + 1) * (n - 1));
        finalT2.assign(sr.t2.begin() + (size_t)k * (n - 1), sr.t2.begin() + (size_t)(k + 1) * (n - 1));
        haveFinalT = true;
        if (cp < cpTarget) alphaL = alpha;
        if (cp >= cpTarget) alphaU = alpha;
        alpha = (alphaL + alphaU) / 2;
        const bool satisfies = cp < cpTarget;
        const bool closer = cp > lastCP;
        const bool eqLower = (cp == lastCP && smoothCost < lastCost);
        if (satisfies && (closer || eqLower)) {
          bestLen = sr.len[k];
          PUMP_TRY(keep_best(k, bestLen));
          lastCost = smoothCost;
          lastCP = cp;
          xsBest = cand[k];
        }
        if (std::fabs(cpTarget - cp) < epsSmoothCP && cpTarget - cp > 0) {
          stop = true;
          break;
        }
        k = 2 * k + (cp < cpTarget ? 1 : 2);
      }
    }
  }
  const bool haveBest = last >= 0 && bestLen > 0;
  if (success && pb_.refine_iters > 0) {
    if (haveBest) {
      bestPath.resize((size_t)bestLen * kDim);
      PUMP_TRY(d2h(bestPath.data(), d_best_.p, bestPath.size()));
      PUMP_TRY(sync());
    }
    PUMP_TRY(refine(xsBest, cpTarget, &lastCP, &lastCost, &bestPath, &bestLen, &xsFinal));
    // the controller path's node states may have changed: its times are
    // computed afresh
    PUMP_TRY(control_launch(xsFinal, nullptr, nullptr));
    PUMP_TRY(sync());
  } else {
    // the kept path's read-back and the controller path in one round trip
    float *hbest = nullptr;
    if (haveBest) {
      PUMP_TRY(ctx_->pinned(Ctx::kPinPaths, sizeof(float) * kDim * (size_t)bestLen, (void **)&hbest));
      res_->d2h_bytes += (long long)(sizeof(float) * kDim * (size_t)bestLen);
      PUMP_CUDA_TRY(cudaMemcpyAsync(hbest, d_best_.p, sizeof(float) * kDim * (size_t)bestLen,
                                    cudaMemcpyDeviceToHost, s_));
    }
    PUMP_TRY(control_launch(xsFinal, haveFinalT ? &finalT5 : nullptr,
                            haveFinalT ? &finalT2 : nullptr));
    PUMP_TRY(sync());
    if (haveBest) bestPath.assign(hbest, hbest + (size_t)bestLen * kDim);
  }
  res_->soln_cp = lastCP;
  res_->soln_cost = lastCost;
  res_->path_len = success ? bestLen : 0;
  if (success && res_->path)
    std::memcpy(res_->path, bestPath.data(),
                sizeof(float) * kDim * (size_t)std::min(bestLen, res_->path_cap));
  PUMP_TRY(control_finish());
  return success ? PUMP_OK : set_error(PUMP_ERR_NO_SOLUTION, "no goal path meets the CP target");
}

pump_status_t Planner::evaluate_paths(const std::vector<std::vector<float>> &xs,
                                      const float *d_table, const float *d_obs, int nobs,
                                      float *cp, float *cost, int *len) {
  d_table_ = d_table;
  obs_p_ = d_obs;
  nobs_ = nobs;
  DevBuf<float> d_rowmax;
  PUMP_TRY(d_rowmax.alloc(3 * (size_t)pb_.table_rows));
  PUMP_TRY(particle_rowmax_async(d_table, pb_.num_mc, pb_.table_rows, d_rowmax.p, s_));
  d_rowmax_ = d_rowmax.p;
  std::vector<int> ln;
  std::vector<float> cs, cps;
  PUMP_TRY(eval_candidates(xs, dt_, pb_.table_rows, true, true, ln, cs, cps));
  for (size_t k = 0; k < xs.size(); ++k) {
    cp[k] = cps[k];
    cost[k] = cs[k];
    len[k] = ln[k];
  }
  return PUMP_OK;
}

// Gradient refinement of the kept path's nodes (pump_refine_paths), judged
// like every candidate of the search: the dense path at dt, its MC CP over
// the particle table and the smoothing's cost (toptBisection tmax 2 + cost
// per segment).  Accepted only if the CP stays <= the target and the cost
// drops; then it replaces the returned path (and feeds the controller path).
pump_status_t Planner::refine(const std::vector<float> &xs, float cpTarget, float *lastCP,
                              float *lastCost, std::vector<float> *bestPath, int *bestLen,
                              std::vector<float> *xsFinal) {
  const int n = (int)(xs.size() / kDim);
  if (n < 3 || n > PUMP_REFINE_MAX_NODES) return PUMP_OK;
  DevBuf<float> d_x, d_out, d_lam, d_J;
  DevBuf<int> d_off, d_cnt;
  DevBuf<double> d_var;
  PUMP_TRY(d_x.alloc(xs.size()));
  PUMP_TRY(d_out.alloc(xs.size()));
  PUMP_TRY(d_lam.alloc(1));
  PUMP_TRY(d_J.alloc(1));
  PUMP_TRY(d_off.alloc(1));
  PUMP_TRY(d_cnt.alloc(1));
  PUMP_TRY(d_var.alloc(pb_.table_rows));
  const int zero = 0;
  const float lam = pb_.refine_lambda;
  PUMP_TRY(h2d(d_x.p, xs.data(), xs.size()));
  PUMP_TRY(h2d(d_off.p, &zero, 1));
  PUMP_TRY(h2d(d_cnt.p, &n, 1));
  PUMP_TRY(h2d(d_lam.p, &lam, 1));
  PUMP_TRY(pump_position_variance(pb_.table_rows, d_var.p, (pump_stream_t)s_));
  pump_refine_args a{};
  a.d_nodes = d_x.p;
  a.n_nodes = n;
  a.d_node_offset = d_off.p;
  a.d_node_count = d_cnt.p;
  a.n_paths = 1;
  a.d_lambda = d_lam.p;
  a.W = pb_.num_disc;
  a.tmax = 5.0f;
  a.d_obstacles = d_obs_.p;
  a.num_obstacles = std::min(nobs_, (int)PUMP_REFINE_MAX_OBSTACLES);
  a.offset_mult = pb_.offset_mult;
  a.d_pos_var = d_var.p;
  a.T_rows = pb_.table_rows;
  a.dt = dt_;
  a.sigma_floor = 1e-3f;
  PUMP_TRY(pump_refine_paths(ctx_->handle(), &a, pb_.refine_iters, d_out.p, d_J.p,
                             (pump_stream_t)s_));
  std::vector<float> xr(xs.size());
  PUMP_TRY(d2h(xr.data(), d_out.p, xr.size()));
  PUMP_TRY(sync());
  std::vector<std::vector<float>> one(1, xr);
  std::vector<int> ln;
  std::vector<float> cs, cps;
  PUMP_TRY(eval_candidates(one, dt_, pb_.table_rows, true, true, ln, cs, cps));
  const float cost = cs[0];
  res_->refine_cp = cps[0];
  res_->refine_cost = cost;
  if (cps[0] >= 0 && cps[0] <= cpTarget && cost < *lastCost) {
    res_->refined = 1;
    *bestLen = ln[0];
    bestPath->resize((size_t)ln[0] * kDim);
    PUMP_TRY(d2h(bestPath->data(), cs_.states.p, bestPath->size()));
    PUMP_TRY(sync());
    *lastCP = cps[0];
    *lastCost = cost;
    *xsFinal = xr;
  }
  return PUMP_OK;
}

// Discretisation for the controller, PUMP.cu:553-569: per segment of the n
// node states, tau = toptBisection(.., 2) sets (int)(tau/0.05 + 1) intervals
// that findDiscretizedPath (tmax 5, 2pBVP.cu:53-69) fills; the row count is
// accumulated as the reference does (an int += float), so trailing rows the
// segments do not reach stay zero.
pump_status_t Planner::control_launch(const std::vector<float> &xs, const std::vector<float> *t5,
                                      const std::vector<float> *t2) {
  const int n = (int)(xs.size() / kDim);
  const float controlDt = 0.05f;
  std::vector<float> tau2, topt5;
  if (t5 && t2 && (int)t5->size() + 1 == n && (int)t2->size() + 1 == n) {
    tau2 = *t2;
    topt5 = *t5;
  } else {
    std::vector<float> a0, a1;
    for (int i = 0; i + 1 < n; ++i) {
      a0.insert(a0.end(), &xs[(size_t)i * kDim], &xs[(size_t)(i + 1) * kDim]);
      a1.insert(a1.end(), &xs[(size_t)(i + 1) * kDim], &xs[(size_t)(i + 2) * kDim]);
    }
    PUMP_TRY(topts_of(a0, a1, 2.0f, &tau2, nullptr));
    PUMP_TRY(topts_of(a0, a1, 5.0f, &topt5, nullptr));
  }
  ControlJob &cj = ctrl_;
  cj.rows = 1;
  for (int i = 0; i + 1 < n; ++i) cj.rows = (int)((float)cj.rows + (tau2[i] / controlDt + 1));
  cj.out.assign((size_t)cj.rows * kDim, 0.0f);
  cj.row.clear();
  cj.pts = nullptr;
  std::vector<int> seg;
  std::vector<float> ts;
  int cur = 0;
  for (int i = 0; i + 1 < n; ++i) {
    const int nw = (int)(tau2[i] / controlDt + 1);
    const float dt = topt5[i] / nw;
    if (cur + nw >= cj.rows)
      return set_error(PUMP_ERR_CAPACITY, "control path: %d rows past %d", cur + nw + 1, cj.rows);
    std::memcpy(&cj.out[(size_t)cur * kDim], &xs[(size_t)i * kDim], sizeof(float) * kDim);
    for (int r = 1; r < nw; ++r) {
      seg.push_back(i);
      cj.row.push_back(cur + r);
      ts.push_back(dt * r);
    }
    cur += nw;
    if (i + 2 == n)
      std::memcpy(&cj.out[(size_t)cur * kDim], &xs[(size_t)(i + 1) * kDim], sizeof(float) * kDim);
  }
  cj.total = (int)seg.size();
  if (cj.total == 0) return PUMP_OK;
  // one upload through pinned memory: node states | sample times | segment
  // times | segment of each sample; the sampled states come back through
  // pinned memory with the caller's synchronisation
  const size_t nx = xs.size(), nt = (size_t)cj.total, nu = topt5.size();
  const size_t in_f = nx + nt + nu + nt;
  float *hin = nullptr;
  PUMP_TRY(ctx_->pinned(Ctx::kPinIn, sizeof(float) * in_f, (void **)&hin));
  std::memcpy(hin, xs.data(), sizeof(float) * nx);
  std::memcpy(hin + nx, ts.data(), sizeof(float) * nt);
  std::memcpy(hin + nx + nt, topt5.data(), sizeof(float) * nu);
  std::memcpy(hin + nx + nt + nu, seg.data(), sizeof(int) * nt);
  PUMP_TRY(d_xs_.alloc(in_f));
  res_->h2d_bytes += (long long)(sizeof(float) * in_f);
  PUMP_CUDA_TRY(cudaMemcpyAsync(d_xs_.p, hin, sizeof(float) * in_f, cudaMemcpyHostToDevice, s_));
  PUMP_TRY(d_ctrl_.alloc(nt * kDim));
  const float *d_x = d_xs_.p;
  const int *d_seg = reinterpret_cast<const int *>(d_xs_.p + nx + nt + nu);
  PUMP_TRY(bvp_path_states(d_x, d_seg, d_x + nx, d_x + nx + nt, cj.total, d_ctrl_.p, s_));
  float *hpts = nullptr;
  PUMP_TRY(ctx_->pinned(Ctx::kPinOut, sizeof(float) * kDim * nt, (void **)&hpts));
  res_->d2h_bytes += (long long)(sizeof(float) * kDim * nt);
  PUMP_CUDA_TRY(cudaMemcpyAsync(hpts, d_ctrl_.p, sizeof(float) * kDim * nt, cudaMemcpyDeviceToHost,
                                s_));
  cj.pts = hpts;
  return PUMP_OK;
}

pump_status_t Planner::control_finish() {
  ControlJob &cj = ctrl_;
  for (int k = 0; k < cj.total && cj.pts; ++k)
    std::memcpy(&cj.out[(size_t)cj.row[k] * kDim], &cj.pts[(size_t)k * kDim], sizeof(float) * kDim);
  res_->ctrl_len = cj.rows;
  if (res_->ctrl_path && res_->ctrl_cap > 0)
    std::memcpy(res_->ctrl_path, cj.out.data(),
                sizeof(float) * kDim * (size_t)std::min(cj.rows, res_->ctrl_cap));
  return PUMP_OK;
}

}  // namespace
}  // namespace pump

using namespace pump;

namespace pump {
namespace {
pump_status_t plan_one(pump_ctx *ctx, const pump_problem *pb, pump_plan_result *res, bool lazy,
                       pump_stream_t stream, const SharedRoadmap *shared,
                       LoopBatcher *batcher = nullptr) {
  if (!ctx || !pb || !res) return set_error(PUMP_ERR_BAD_INPUT, "pump_plan: null argument");
  if (pb->N < 2 || pb->num_disc < 1 || pb->num_hsmc < 1 || pb->num_mc < pb->num_hsmc ||
      pb->table_rows < 2 || pb->num_obstacles < 0 || (pb->num_obstacles > 0 && !pb->obstacles) ||
      !(pb->cp_factor > 0) || pb->max_paths < 0 || !(pb->disc_len >= 0) ||
      (pb->disc_len > 0 && (pb->disc_min < 1 || pb->disc_min > pb->num_disc)) ||
      (pb->bvp_mode != PUMP_BVP_PARITY && pb->bvp_mode != PUMP_BVP_PRECISION &&
       pb->bvp_mode != PUMP_BVP_PARITY_GPU))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_plan: problem out of domain");
  float *path = res->path;
  int path_cap = res->path_cap;
  int *nodes = res->nodes;
  int nodes_cap = res->nodes_cap;
  int *trace = res->wf_trace;
  long long trace_cap = res->wf_trace_cap;
  float *ctrl = res->ctrl_path;
  int ctrl_cap = res->ctrl_cap;
  float *ptime = res->path_time;
  uint32_t *pvalid = res->path_valid;
  const int pstate_cap = res->path_state_cap;
  std::memset(res, 0, sizeof *res);
  res->path_time = ptime;
  res->path_valid = pvalid;
  res->path_state_cap = pstate_cap;
  res->ctrl_path = ctrl;
  res->ctrl_cap = ctrl ? ctrl_cap : 0;
  res->path = path;
  res->path_cap = path_cap;
  res->nodes = nodes;
  res->nodes_cap = nodes_cap;
  res->wf_trace = trace;
  res->wf_trace_cap = trace ? trace_cap : 0;
  res->soln_path_idx = -1;
  Ctx *c = Ctx::from(ctx);
  PUMP_TRY(c->activate());
  PUMP_TRY(c->arena_begin((cudaStream_t)stream));
  ArenaScope scope(c, (cudaStream_t)stream);
  Planner planner(c, *pb, res, (cudaStream_t)stream, shared, lazy, batcher);
  return planner.run();
}
}  // namespace
}  // namespace pump

namespace pump {
namespace {
// Contexts and streams of batch workers, kept across pump_plan_batch calls
// so their scratch and pinned buffers are allocated once per process.
std::mutex g_worker_mu;
std::vector<std::pair<int, std::pair<pump_ctx *, cudaStream_t>>> g_idle_workers;

pump_status_t take_worker(int device, pump_ctx **ctx, cudaStream_t *s) {
  {
    std::lock_guard<std::mutex> lk(g_worker_mu);
    for (size_t i = 0; i < g_idle_workers.size(); ++i)
      if (g_idle_workers[i].first == device) {
        *ctx = g_idle_workers[i].second.first;
        *s = g_idle_workers[i].second.second;
        g_idle_workers.erase(g_idle_workers.begin() + i);
        return Ctx::from(*ctx)->activate();
      }
  }
  *ctx = nullptr;
  *s = nullptr;
  PUMP_TRY(pump_ctx_create(device, ctx));
  return cuda_status(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking),
                     "cudaStreamCreateWithFlags");
}

// A worker goes back to the idle pool only when its stream is idle and its
// last query did not end in a CUDA error or a timed-out device wait: such a
// context or stream may hold queued work or a sticky error, so it is
// destroyed and the next call creates a fresh one.
void give_worker(int device, pump_ctx *ctx, cudaStream_t s, pump_status_t last) {
  const bool healthy = ctx && s && last != PUMP_ERR_CUDA && last != PUMP_ERR_TIMEOUT &&
                       cudaStreamQuery(s) == cudaSuccess;
  if (!healthy) {
    if (s) cudaStreamSynchronize(s);
    if (s) cudaStreamDestroy(s);
    if (ctx) pump_ctx_destroy(ctx);
    cudaGetLastError();
    return;
  }
  std::lock_guard<std::mutex> lk(g_worker_mu);
  g_idle_workers.push_back({device, {ctx, s}});
}
}  // namespace
}  // namespace pump

extern "C" void pump_search_graph(int level) {
  search_graph_flag().store(level < 0 ? 0 : (level > 2 ? 2 : level));
}

extern "C" void pump_batch_groups(int max_group, int window_us) {
  batch_group_flags()[0].store(max_group < 1 ? 1 : (max_group > kLoopGroupMax ? kLoopGroupMax
                                                                                : max_group));
  batch_group_flags()[1].store(window_us < 0 ? 0 : window_us);
}

extern "C" pump_status_t pump_plan_batch(int device, const pump_problem *problems,
                                         pump_plan_result *results, pump_status_t *statuses, int n,
                                         int workers) {
  if (n < 0 || (n > 0 && (!problems || !results || !statuses)) || workers < 1)
    return set_error(PUMP_ERR_BAD_INPUT, "pump_plan_batch: bad arguments");
  if (n == 0) return PUMP_OK;
  if (workers > n) workers = n;
  // Shared roadmaps: one per (BVP mode, bounds) group of Halton queries, with
  // the pair BVPs of Halton points 1 .. max(N) - 2 computed once.
  PUMP_CUDA_TRY(cudaSetDevice(device));
  std::vector<SharedRoadmap> groups;
  std::vector<float *> owned;
  cudaStream_t setup_stream = nullptr;
  PUMP_CUDA_TRY(cudaStreamCreateWithFlags(&setup_stream, cudaStreamNonBlocking));
  auto cleanup = [&]() {
    for (float *p : owned) cudaFree(p);
    cudaStreamDestroy(setup_stream);
  };
  for (int k = 0; k < n; ++k) {
    const pump_problem &pb = problems[k];
    if (pb.samples || pb.N < 4) continue;
    SharedRoadmap *g = nullptr;
    for (auto &x : groups) {
      bool same = x.mode == pb.bvp_mode;
      for (int d = 0; d < 6 && same; ++d) same = x.lo[d] == pb.lo[d] && x.hi[d] == pb.hi[d];
      if (same) g = &x;
    }
    if (!g) {
      SharedRoadmap x{};
      x.mode = pb.bvp_mode;
      for (int d = 0; d < 6; ++d) { x.lo[d] = pb.lo[d]; x.hi[d] = pb.hi[d]; }
      x.M = 0;
      groups.push_back(x);
      g = &groups.back();
    }
    if (pb.N - 2 > g->M) g->M = pb.N - 2;
  }
  for (auto &g : groups) {
    if (g.M < 2) { g.M = -1; continue; }
    pump_problem hp{};
    hp.N = (int)g.M + 2;
    for (int d = 0; d < 6; ++d) { hp.lo[d] = g.lo[d]; hp.hi[d] = g.hi[d]; }
    std::vector<float> all;
    halton_samples(hp, all);  // points 0 .. M+1; the shared set is 1 .. M
    float *d_pts = nullptr, *d_c = nullptr, *d_t = nullptr;
    const long long np = g.M * (g.M - 1);
    pump_status_t st = cuda_status(cudaMalloc(&d_pts, sizeof(float) * kDim * g.M), "cudaMalloc");
    if (st == PUMP_OK) st = cuda_status(cudaMalloc(&d_c, sizeof(float) * np), "cudaMalloc");
    if (st == PUMP_OK) st = cuda_status(cudaMalloc(&d_t, sizeof(float) * np), "cudaMalloc");
    owned.push_back(d_pts);
    owned.push_back(d_c);
    owned.push_back(d_t);
    if (st == PUMP_OK)
      st = cuda_status(cudaMemcpyAsync(d_pts, all.data() + kDim, sizeof(float) * kDim * g.M,
                                       cudaMemcpyHostToDevice, setup_stream), "H2D");
    if (st == PUMP_OK)
      st = pump_bvp_pairs(d_pts, (int)g.M, 5.0f, g.mode, d_c, d_t, (pump_stream_t)setup_stream);
    if (st != PUMP_OK) { cleanup(); return st; }
    g.d_copt = d_c;
    g.d_topt = d_t;
  }
  {
    pump_status_t st = cuda_status(cudaStreamSynchronize(setup_stream), "cudaStreamSynchronize");
    if (st != PUMP_OK) { cleanup(); return st; }
  }
  // grouped search loops (pump_batch_groups): two groups may run at once
  std::unique_ptr<LoopBatcher> batcher;
  const int group_max = batch_group_flags()[0].load();
  if (group_max > 1 && workers > 1) {
    batcher.reset(new LoopBatcher(device, workers, group_max, batch_group_flags()[1].load(), 2));
    if (batcher->status() != PUMP_OK) {
      const pump_status_t st = batcher->status();
      batcher.reset();
      cleanup();
      return st;
    }
  }
  std::atomic<int> next(0);
  std::vector<pump_status_t> setup(workers, PUMP_OK);
  std::vector<std::string> msgs(workers);
  // the message of the first query (in query order) that failed
  std::mutex fail_mu;
  int first_fail = n;
  std::string fail_msg;
  auto worker = [&](int w) {
    // groups stop waiting for this worker once it has no more queries
    struct Leave {
      LoopBatcher *b;
      ~Leave() {
        if (b) b->leave();
      }
    } leave{batcher.get()};
    pump_ctx *ctx = nullptr;
    cudaStream_t s = nullptr;
    pump_status_t st = take_worker(device, &ctx, &s);
    pump_status_t last = st;
    if (st != PUMP_OK) {
      setup[w] = st;
      msgs[w] = pump_last_error();
    } else {
      for (int k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
        const SharedRoadmap *g = nullptr;
        for (const auto &x : groups)
          if (x.M > 0 && x.matches(problems[k])) g = &x;
        statuses[k] = plan_one(ctx, &problems[k], &results[k], true, (pump_stream_t)s, g,
                               batcher.get());
        last = statuses[k];
        if (statuses[k] != PUMP_OK && statuses[k] != PUMP_ERR_NO_SOLUTION) {
          std::lock_guard<std::mutex> lk(fail_mu);
          if (k < first_fail) {
            first_fail = k;
            fail_msg = pump_last_error();
          }
        }
        if (last == PUMP_ERR_CUDA || last == PUMP_ERR_TIMEOUT) {
          // the rest of this worker's queries run on a fresh context and stream
          give_worker(device, ctx, s, last);
          ctx = nullptr;
          s = nullptr;
          last = take_worker(device, &ctx, &s);
          if (last != PUMP_OK) {
            setup[w] = last;
            msgs[w] = pump_last_error();
            break;
          }
        }
      }
    }
    give_worker(device, ctx, s, last);
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < workers; ++w) pool.emplace_back(worker, w);
  worker(0);
  for (auto &t : pool) t.join();
  batcher.reset();
  cleanup();
  for (int w = 0; w < workers; ++w)
    if (setup[w] != PUMP_OK) return set_error(setup[w], "pump_plan_batch worker %d: %s", w, msgs[w].c_str());
  if (first_fail < n) set_error(PUMP_OK, "query %d: %s", first_fail, fail_msg.c_str());
  return PUMP_OK;
}

extern "C" pump_status_t pump_path_cp(pump_ctx *ctx, const float *h_nodes, const int *h_offset,
                                      const int *h_count, int n_paths, int mode,
                                      const float *d_table_t, int Pmc, int T_rows,
                                      float offset_mult, const float *d_obstacles,
                                      int num_obstacles, float *h_cp, float *h_cost, int *h_len,
                                      pump_stream_t stream) {
  if (!ctx || n_paths < 0 || (n_paths > 0 && (!h_nodes || !h_offset || !h_count || !d_table_t ||
                                              !h_cp || !h_cost || !h_len)) ||
      Pmc <= 0 || T_rows < 2 || num_obstacles < 0 || (num_obstacles > 0 && !d_obstacles) ||
      (mode != PUMP_BVP_PARITY && mode != PUMP_BVP_PRECISION && mode != PUMP_BVP_PARITY_GPU))
    return set_error(PUMP_ERR_BAD_INPUT, "pump_path_cp: bad arguments");
  if (n_paths == 0) return PUMP_OK;
  std::vector<std::vector<float>> xs(n_paths);
  for (int k = 0; k < n_paths; ++k) {
    if (h_count[k] < 1 || h_offset[k] < 0)
      return set_error(PUMP_ERR_BAD_INPUT, "pump_path_cp: path %d has %d nodes", k, h_count[k]);
    xs[k].assign(h_nodes + (size_t)h_offset[k] * kDim,
                 h_nodes + (size_t)(h_offset[k] + h_count[k]) * kDim);
  }
  pump_problem pb;
  pump_problem_defaults(&pb);
  pb.bvp_mode = mode;
  pb.num_mc = Pmc;
  pb.table_rows = T_rows;
  pb.offset_mult = offset_mult;
  pump_plan_result res;
  std::memset(&res, 0, sizeof res);
  Ctx *c = Ctx::from(ctx);
  PUMP_TRY(c->activate());
  t_alloc_stream = (cudaStream_t)stream;
  Planner pl(c, pb, &res, (cudaStream_t)stream);
  return pl.evaluate_paths(xs, d_table_t, d_obstacles, num_obstacles, h_cp, h_cost, h_len);
}

extern "C" pump_status_t pump_plan(pump_ctx *ctx, const pump_problem *pb, pump_plan_result *res,
                                   pump_stream_t stream) {
  return plan_one(ctx, pb, res, false, stream, nullptr);
}
