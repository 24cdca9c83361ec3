/*
 * pump.h -- C ABI of pump_gb300, a GB300-native (sm_103a) implementation of
 * the PUMP planner's hot path (Parallel Uncertainty-aware Multiobjective
 * Planning, 3D double integrator, 6D state).
 *
 * Each entry point replaces one function of the reference
 * (StanfordASL/PUMP); the reference file:line is cited beside it.  Device
 * buffers are caller-owned raw pointers; every call takes an explicit CUDA
 * stream (pump_stream_t is cudaStream_t) and returns a pump_status_t instead
 * of exiting the process (the reference calls exit(1) from CUDA_ERROR_CHECK,
 * helper.cuh:22-30).  Calls are asynchronous on the stream unless they return
 * a host value, in which case they synchronise the stream.
 *
 * Arithmetic ("parity" mode): every operation is evaluated in the type the
 * reference's C++ source gives it (binary32, or binary64 where pow() or a
 * double literal promotes it), rounded once, never fused into a
 * multiply-add, and pow(x, n) for n = 2, 3, 4 is correctly rounded.  The
 * reference's own code built for the CPU with that rule reproduces every
 * result of this library bit for bit.  The "precision" BVP mode instead
 * solves the optimal time from the analytic stationarity quartic in binary64.
 *
 * Masks are one byte per item (0/1) as the reference's bool arrays, except
 * the HSMC particle masks, which are bit-packed: bit (p & 31) of word
 * path * ceil(P/32) + p / 32 is particle p of that path.
 *
 * Thread safety: a pump_ctx may be used by one host thread at a time.
 */
#ifndef PUMP_GB300_H
#define PUMP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *pump_stream_t; /* == cudaStream_t */
typedef struct pump_ctx pump_ctx;

typedef enum pump_status_t {
  PUMP_OK = 0,
  PUMP_ERR_BAD_INPUT = 1,   /* argument out of domain (sizes, pointers, file format) */
  PUMP_ERR_CAPACITY = 2,    /* a fixed capacity of the reference would be exceeded */
  PUMP_ERR_TIMEOUT = 3,     /* a bounded device wait or loop gave up */
  PUMP_ERR_CUDA = 4,        /* CUDA runtime error (message in pump_last_error) */
  PUMP_ERR_NO_SOLUTION = 5, /* planner finished without a path meeting the CP target */
  PUMP_ERR_NO_MEMORY = 6
} pump_status_t;

enum { PUMP_DIM = 6 };

/* BVP arithmetic modes for pump_bvp_pairs.
 *  PUMP_BVP_PARITY: the reference's algorithm in the arithmetic of its host
 *    code (every operation rounded once, no contraction, pow(x, n) correctly
 *    rounded), which is also what the reference built for a CPU computes.
 *  PUMP_BVP_PRECISION: the binary64 minimiser of the same cost.
 *  PUMP_BVP_PARITY_GPU: the pair times and costs in the arithmetic of the
 *    reference's own GPU kernel (fillCoptsTopts, 2pBVP.cu:133-150, compiled by
 *    nvcc with its default multiply-add contraction and CUDA's binary64 pow):
 *    bit for bit what that kernel computes on the GB300.  For a planning
 *    query it applies to the pair matrix (rn, the edges, their costs and the
 *    times HSMC and the search use); the waypoints, the heuristic and the
 *    solution search use the parity arithmetic, as the reference's host code
 *    computes them. */
enum { PUMP_BVP_PARITY = 0, PUMP_BVP_PRECISION = 1, PUMP_BVP_PARITY_GPU = 2 };

const char *pump_status_string(pump_status_t s);
/* Last error message of this thread (never NULL). */
const char *pump_last_error(void);
/* Library version string. */
const char *pump_version(void);

/* Context: owns scratch device memory reused across calls on one device. */
pump_status_t pump_ctx_create(int device, pump_ctx **out);
pump_status_t pump_ctx_destroy(pump_ctx *ctx);

/* ------------------------------------------------------------------ 2pBVP */
/* Optimal time and cost of the double-integrator two-point BVP for every
 * ordered pair i != j of N samples (samples: N x 6 floats), written at
 * idx = i*(N-1) + j - (i < j).
 * Replaces fillCoptsTopts (2pBVP.cu:133-150) with toptBisection
 * (2pBVP.cu:71-95) and cost (2pBVP.cu:97-107); mode PUMP_BVP_PRECISION
 * returns the binary64 minimiser of the same cost instead (N <= 65535). */
pump_status_t pump_bvp_pairs(const float *d_samples, int N, float tmax, int mode, float *d_copts,
                             float *d_topts, pump_stream_t stream);

/* Optimal time / cost of the explicit pairs (d_x0[k], d_x1[k]), k < n
 * (6 floats each); replaces host calls of toptBisection + cost
 * (mainPUMP.cu:351-355, PUMP.cu:499-502). */
pump_status_t pump_bvp_batch(const float *d_x0, const float *d_x1, int n, float tmax, int mode,
                             float *d_topt, float *d_cost, pump_stream_t stream);

/* k-th smallest of n floats (0-based), exact: the value the reference reads
 * after thrust::sort (mainPUMP.cu:303-304).  Uses ctx scratch; synchronises
 * the stream and returns the value in *h_kth. */
pump_status_t pump_select_kth(pump_ctx *ctx, const float *d_v, long long n, long long k,
                              float *h_kth, pump_stream_t stream);

/* Roadmap edges: pairs with copt < rn in (i asc, j asc) order
 * (mainPUMP.cu:327-346).  Writes E = *h_num_edges (synchronises), then
 * d_src[E], d_dst[E], d_copt[E], d_topt[E] and the go-adjacency row starts
 * d_go_start[N+1] (edges of node i are [go_start[i], go_start[i+1]), in j
 * order, replacing nnGoEdges/nnIdxs of mainPUMP.cu:379-392).  Capacity
 * max_edges; PUMP_ERR_CAPACITY if more edges qualify. */
pump_status_t pump_build_edges(pump_ctx *ctx, const float *d_copts, const float *d_topts, int N,
                               float rn, long long max_edges, int *d_src, int *d_dst,
                               float *d_copt, float *d_topt, int *d_go_start,
                               long long *h_num_edges, pump_stream_t stream);

/* pump_select_kth(k) followed by pump_build_edges(rn) in one call
 * (mainPUMP.cu:289-346: the thrust::sort of all pair costs, rn at index k,
 * the edges below rn): the same rn (*h_rn), edge count and edge arrays,
 * from one read of the pair costs.  A strided sample bounds rn from above;
 * the pairs below the bound are selected and compacted; a sample that
 * misses rank k falls back to the full passes.  Synchronises. */
pump_status_t pump_roadmap_edges(pump_ctx *ctx, const float *d_copts, const float *d_topts, int N,
                                 long long k, long long max_edges, int *d_src, int *d_dst,
                                 float *d_copt, float *d_topt, int *d_go_start, float *h_rn,
                                 long long *h_num_edges, pump_stream_t stream);

/* The roadmap's device half in one call (mainPUMP.cu:248-346):
 * fillCoptsTopts over all N(N-1) ordered pairs of d_samples[N][6] (tmax,
 * arithmetic bvp_mode, as pump_bvp_pairs) into d_copts/d_topts, then rn =
 * the k-th smallest pair cost and the edges below it, as
 * pump_roadmap_edges.  The outputs are those of the two calls.  In
 * PUMP_BVP_PRECISION the pair kernel counts the rn superset while it stores
 * the costs, so the costs are read once more instead of twice.
 * h_stage_ms (optional, 3 floats): CUDA-event times, in ms, of the work
 * before the pair kernel (sample preparation and the rn bracket's sample),
 * of the pair kernel, and of the rest.  Synchronises. */
pump_status_t pump_roadmap(pump_ctx *ctx, const float *d_samples, int N, float tmax, int bvp_mode,
                           long long k, long long max_edges, float *d_copts, float *d_topts,
                           int *d_src, int *d_dst, float *d_copt, float *d_topt, int *d_go_start,
                           float *h_rn, long long *h_num_edges, float *h_stage_ms,
                           pump_stream_t stream);

/* Edge waypoints disc[E][numDisc+1][6] (findDiscretizedPath, 2pBVP.cu:53-69
 * and pathPoint 2pBVP.cu:117-131, as called at mainPUMP.cu:339).  d_topt
 * is the edge's optimal time (identical to the one toptBisection recomputes
 * there).  mode PUMP_BVP_PARITY evaluates pathPoint's expressions as the
 * reference does (binary64 where they promote); PUMP_BVP_PRECISION
 * evaluates the same cubic in binary32 (FP64 is kept for the time root);
 * PUMP_BVP_PARITY_GPU ignores d_topt (which holds the GPU kernel's times) and
 * recomputes each edge's time with the host arithmetic, as
 * findDiscretizedPath does, then evaluates as PUMP_BVP_PARITY. */
pump_status_t pump_discretize_edges(const float *d_samples, const int *d_src, const int *d_dst,
                                    const float *d_topt, long long E, int numDisc, int mode,
                                    float *d_disc, pump_stream_t stream);

/* Waypoint counts by edge length and the ragged waypoint layout (no
 * counterpart in the reference, whose numDisc is one value per problem,
 * mainPUMP.cu:57).  Edge e (d_src[e] -> d_dst[e]) gets numDisc_e =
 * ceil(L_e / disc_len) clamped to [min_disc, max_disc] (max_disc for every
 * edge when disc_len <= 0), L_e = sqrtf((dx*dx + dy*dy) + dz*dz) of its end
 * positions in binary32.  Writes d_off[E + 1]: edge e's waypoints are
 * records d_off[e] .. d_off[e+1]-1 (numDisc_e + 1 of them) of a waypoint
 * array, and *h_total = d_off[E].  Synchronises. */
pump_status_t pump_disc_offsets(const float *d_samples, const int *d_src, const int *d_dst,
                                long long E, float disc_len, int min_disc, int max_disc,
                                long long *d_off, long long *h_total, pump_stream_t stream);

/* pump_discretize_edges over the ragged layout: numDisc_e + 1 waypoints of
 * edge e at records d_off[e] .. of d_disc (numDisc_e <= max_disc).  An edge
 * whose count lies outside [2, max_disc + 1] is PUMP_ERR_BAD_INPUT (its
 * block writes nothing).  Synchronises. */
pump_status_t pump_discretize_edges_off(const float *d_samples, const int *d_src, const int *d_dst,
                                        const float *d_topt, long long E, const long long *d_off,
                                        int max_disc, int mode, float *d_disc, pump_stream_t stream);

/* -------------------------------------------------------------- tuning */
/* Launch-shape autotuner.  Kernels with several launch shapes that compute
 * the same results (the precision pair BVP's, the waypoints' and the edge
 * check's block sizes; the grid of the large compactions) pick their shape
 * per shape class (a size's power-of-two bucket, the waypoint count, the
 * box count) on the device: the first call of a class runs every candidate
 * twice on its own inputs, on its stream, and keeps the fastest second run.
 * Records are process-wide.  pump_tune_enable(0) (or PUMP_TUNE=0 in the
 * environment) switches tuning off: every kernel then uses its default
 * shape; pump_tune_reset forgets the records.  pump_tune_report writes one
 * line per record (kernel, class, choice, candidate times in ms) into buf
 * (truncated to len - 1 characters) and returns the full length. */
void pump_tune_enable(int on);
void pump_tune_reset(void);
int pump_tune_report(char *buf, size_t len);

/* The reference's Halton samples (createSamplesHalton(0, ...), sampler.cu:20-41,
 * as mainPUMP.cu:250 calls it): sample n, coordinate d = halton(n, base d)
 * scaled into [lo[d], hi[d]] in binary32 as the reference evaluates it,
 * sample 0 = init and sample N-1 = goal; writes d_samples[N][6] on the
 * device (host arrays of 6 floats for lo, hi, init, goal). */
pump_status_t pump_halton_samples(int N, const float *lo, const float *hi, const float *init,
                                  const float *goal, float *d_samples, pump_stream_t stream);

/* ------------------------------------------------------ collision checks */
/* isFree[i] = sample i is not strictly inside any box (sampleFree,
 * sampler.cu:61-88).  obstacles: numObs x 12 floats (lo[6], hi[6]). */
pump_status_t pump_sample_free(const float *d_obstacles, int numObs, const float *d_samples, int N,
                               uint8_t *d_is_free, pump_stream_t stream);

/* isFree[e] = every waypoint segment of edge e misses every box
 * (freeEdges, collisionCheck.cu:5-37, isMotionValid :65-143). */
pump_status_t pump_free_edges(const float *d_obstacles, int numObs, const float *d_disc,
                              long long E, int numDisc, uint8_t *d_is_free, pump_stream_t stream);

/* pump_free_edges over the ragged layout of pump_disc_offsets (each edge's
 * own segments).  PUMP_ERR_BAD_INPUT for an edge count outside
 * [2, max_disc + 1].  Synchronises. */
pump_status_t pump_free_edges_off(const float *d_obstacles, int numObs, const float *d_disc,
                                  const long long *d_off, long long E, int max_disc,
                                  uint8_t *d_is_free, pump_stream_t stream);

/* Half-spaces of every waypoint of free edges: setupAsBs (hsmc.cu:201-211)
 * then cacheHalfspaces (hsmc.cu:10-99).  as[E][W][maxHS][3], bs[E][W][maxHS],
 * count[E][W] (count of non-free edges is written 0). */
pump_status_t pump_cache_halfspaces(const float *d_obstacles, int numObs, const float *d_disc,
                                    const uint8_t *d_is_free_edge, long long E, int W, int maxHS,
                                    float maxd2, float *d_as, float *d_bs, int *d_count,
                                    pump_stream_t stream);

/* The same half-spaces without the defaults: only the stored ones are
 * written (as[e][w][h] for h < count[e][w]; the slots past a waypoint's
 * count keep what the buffers held) and count is one byte per waypoint.
 * What the search reads is the same: pass d_count to pump_hsmc_propagate.
 * maxHS <= 8.  Not a reference function: the reference's arrays are the
 * dense layout above. */
pump_status_t pump_cache_halfspaces_sparse(const float *d_obstacles, int numObs,
                                           const float *d_disc, const uint8_t *d_is_free_edge,
                                           long long E, int W, int maxHS, float maxd2,
                                           float *d_as, float *d_bs, uint8_t *d_count,
                                           pump_stream_t stream);

/* --------------------------------------------------------------- HSMC */
/* Particle tables of the closed-loop tracking-error model (the data of the
 * reference's missing hardCoded.cu, hardCoded.cuh:12-19): position errors
 * tmajor[T][P][3] (xcombTime) and pmajor[P][T][3] (xcomb); either may be
 * NULL.  Philox4x32-10 keyed by seed, Box-Muller, binary64 dynamics.  Uses a
 * temporary of 24 B per (particle, step), allocated and freed in stream
 * order on `stream`. */
pump_status_t pump_particle_tables(uint64_t seed, int P, int T, float *d_tmajor, float *d_pmajor,
                                   pump_stream_t stream);

/* Half-space Monte Carlo propagation of num_new new paths, path base+i
 * extending path prev[i] along edge[i]: propagateValidParticles
 * (PUMP.cu:613-655) with the hit count of calculateCP_HSMC
 * (PUMP.cu:745-758) fused.  valid: bit-packed, ceil(P/32) words per path;
 * times[path] is the start time of each path; topt[edge] the edge time;
 * offsets_t the time-major table with Pmc particles per row and T_rows rows.
 * Device-side checks write *d_error (device, may be NULL): an edge outside
 * [0, num_edges) or a parent outside [0, base) skips that path and records
 * PUMP_ERR_BAD_INPUT; a time row past T_rows records PUMP_ERR_CAPACITY.
 * Writes path_cp[base+i].  d_hs_count (may be NULL): the stored half-spaces
 * per waypoint of pump_cache_halfspaces_sparse; with it only those slots are
 * read, without it every slot is read and b >= 1000 marks an unused one. */
pump_status_t pump_hsmc_propagate(int num_new, int W, const int *d_edge, const int *d_prev,
                                  long long num_edges, int base, const float *d_as, const float *d_bs, int maxHS,
                                  const float *d_times, const float *d_topt, float dt,
                                  const float *d_offsets_t, int Pmc, int T_rows,
                                  float offset_mult, uint32_t *d_valid, int P, float *d_path_cp,
                                  int *d_error, const uint8_t *d_hs_count, pump_stream_t stream);

/* pump_hsmc_propagate with the half-spaces derived inside the kernel from
 * the boxes and the edge's waypoints (disc[edge][W][6]) instead of read from
 * a cache: the same half-spaces pump_cache_halfspaces would store for the
 * edge (first maxHS boxes in index order within the distance gate maxd2 of
 * each waypoint, the reference's arithmetic), so masks and CPs are identical.
 * Every edge named is treated as free (the search only propagates along
 * free edges).  W <= 256 and W * maxHS <= 256; the boxes are staged in
 * shared memory (PUMP_ERR_CAPACITY beyond about 3,800 boxes). */
pump_status_t pump_hsmc_propagate_boxes(int num_new, int W, const int *d_edge, const int *d_prev,
                                        long long num_edges, int base, const float *d_obstacles,
                                        int numObs, const float *d_disc, float maxd2, int maxHS,
                                        const float *d_times, const float *d_topt, float dt,
                                        const float *d_offsets_t, int Pmc, int T_rows,
                                        float offset_mult, uint32_t *d_valid, int P,
                                        float *d_path_cp, int *d_error, pump_stream_t stream);

/* pump_hsmc_propagate_boxes over the ragged layout: each edge's waypoints
 * are records d_disc_off[e] .. d_disc_off[e+1]-1 of d_disc (2 .. max_w of
 * them; an edge outside that range records PUMP_ERR_BAD_INPUT in *d_error
 * and its path is skipped), and its waypoint times are t + i * topt /
 * (W_e - 1).  max_w * maxHS <= 256. */
pump_status_t pump_hsmc_propagate_boxes_off(int num_new, int max_w, const int *d_edge,
                                            const int *d_prev, long long num_edges, int base,
                                            const float *d_obstacles, int numObs,
                                            const float *d_disc, const long long *d_disc_off,
                                            float maxd2, int maxHS, const float *d_times,
                                            const float *d_topt, float dt,
                                            const float *d_offsets_t, int Pmc, int T_rows,
                                            float offset_mult, uint32_t *d_valid, int P,
                                            float *d_path_cp, int *d_error, pump_stream_t stream);

/* Full Monte Carlo collision probability of n_paths dense paths at once
 * (MCCP + thrust::reduce, collisionProbability.cu:4-92).  Path k has
 * d_len[k] states starting at d_paths + d_offset[k]*6.  The particle
 * offsets are read from the time-major table (T_rows rows of Pmc particles;
 * the values equal the reference's particle-major xcomb, the layout only
 * makes a warp's reads contiguous).  Writes d_hits[k] and
 * d_cp[k] = hits / Pmc; a path longer than T_rows states sets *d_error
 * (device, may be NULL) to PUMP_ERR_CAPACITY and counts no hits. */
pump_status_t pump_mc_cp(const float *d_paths, const int *d_offset, const int *d_len, int n_paths,
                         const float *d_offsets_t, int Pmc, int T_rows, float offset_mult,
                         const float *d_obstacles, int numObs, int *d_hits, float *d_cp,
                         int *d_error, pump_stream_t stream);

/* ------------------------------------------------------------- GMT */
/* Stable compaction of a frontier flag array into the ascending list of set
 * indices (thrust::exclusive_scan + fillWavefront, GMT.cu:48-54, 66-76,
 * 166-176).  Writes d_active[0..count) and *d_count (device). */
pump_status_t pump_frontier_compact(pump_ctx *ctx, const uint8_t *d_flags, int N, int *d_active,
                                    int *d_count, pump_stream_t stream);

/* Diagnostic of the bounded device waits (no counterpart in the reference).
 * Every spin of the library's kernels on a word another block publishes (the
 * decoupled look-back of the compactions, the edge lists and the search's
 * store pass) gives up after a bound and records an error that the calling
 * entry point returns as PUMP_ERR_TIMEOUT, leaving the context usable.  This
 * runs that look-back wait, with at most spin_limit polls, on a status word
 * that nothing publishes, and returns what the wait reported: PUMP_ERR_TIMEOUT
 * when the bound ended it (the expected result), PUMP_OK if it did not.
 * Synchronises the stream. */
pump_status_t pump_selftest_wait(pump_ctx *ctx, long long spin_limit, pump_stream_t stream);

/* The same compaction for callers that may not allocate device memory while
 * they run (a real-time loop that reserves all memory at start-up, or a host
 * framework that owns the memory budget and forbids cudaMalloc in plugins).
 * No counterpart in the reference.  Scratch is a fixed 64 KiB array in device
 * memory owned by the library (held by every GPU that loads it until the
 * process exits), so N is limited to 33,554,432 flags (PUMP_ERR_CAPACITY
 * beyond).  The first call on a device (and the first after a device reset,
 * or in another CUDA context) looks up the array's address; make it before
 * any stream capture.  All calls share the array: calls that overlap
 * on the GPU race and must be serialised.  Synchronises the stream. */
pump_status_t pump_frontier_compact_noalloc(const uint8_t *d_flags, int N, int *d_active,
                                            int *d_count, pump_stream_t stream);

/* ------------------------------------------------------ path refinement */
/* Gradient refinement of returned paths, the slot of the reference's
 * alpha-bisection smoothing (PUMP.cu:406-545); no counterpart function in
 * the reference.  For a path of n node states x_0 .. x_{n-1} the objective is
 *   J = sum_i c(tau_i; x_i, x_{i+1}) + lambda * B
 * with c the 2pBVP cost (2pBVP.cu:97-107) at its optimal time tau_i on
 * (0, tmax] (the closed-form binary64 minimiser of the precision mode) and B
 * a smoothed half-space bound of the collision probability: over the
 * waypoints at s = k/W (k < W) of every segment (the cubic of pathPoint,
 * 2pBVP.cu:117-131) and over every box, the sum of
 * Phi(-d / (offset_mult * sigma(T))), where d is the distance from the
 * waypoint to the box's closest point measured perpendicular to the
 * waypoint's velocity (the half-space of cacheHalfspaces, hsmc.cu:70-96,
 * without its distance gate and slot limit) and sigma^2(T) the closed-loop
 * position variance per axis at the waypoint's time T (linear between steps
 * of dt, the last row beyond the table) plus sigma_floor^2.  The gradient is
 * taken with respect to the intermediate nodes x_1 .. x_{n-2}; tau_i enters
 * through the implicit function theorem (dtau/dx = -c'_x / c''_tau; zero
 * when tau_i = tmax).  Arithmetic: binary64 for tau_i, binary32 elsewhere. */
enum { PUMP_REFINE_MAX_NODES = 257, PUMP_REFINE_MAX_W = 64, PUMP_REFINE_MAX_OBSTACLES = 8192 };

typedef struct pump_refine_args {
  const float *d_nodes;       /* node states of all paths, 6 floats each */
  int n_nodes;                /* rows of d_nodes */
  const int *d_node_offset;   /* first node row of path k */
  const int *d_node_count;    /* nodes of path k, 2 .. PUMP_REFINE_MAX_NODES */
  int n_paths;
  const float *d_lambda;      /* bound weight per path */
  int W;                      /* waypoints per segment, 1 .. PUMP_REFINE_MAX_W */
  float tmax;                 /* optimal-time bracket (0, tmax] */
  const float *d_obstacles;   /* num_obstacles x 12 (lo[6], hi[6]) */
  int num_obstacles;          /* 0 .. PUMP_REFINE_MAX_OBSTACLES */
  float offset_mult;          /* position error multiplier (input file line 5) */
  const double *d_pos_var;    /* per-axis position variance per step (pump_position_variance) */
  int T_rows;
  float dt;                   /* table step, 0.05 s */
  float sigma_floor;          /* added to sigma in quadrature (the variance is 0 at T = 0) */
} pump_refine_args;

/* Per-axis position variance of the particle model's closed loop at steps
 * 0 .. T-1 (the covariance of the tracking error behind
 * pump_particle_tables), propagated in binary64 on the device. */
pump_status_t pump_position_variance(int T, double *d_var, pump_stream_t stream);

/* J, the cost sum and B per path (any output may be NULL). */
pump_status_t pump_refine_fwd(const pump_refine_args *a, float *d_J, float *d_cost, float *d_bound,
                              pump_stream_t stream);

/* dJ/dx for every node row of every path (rows of x_0 and x_{n-1} are 0),
 * and J (may be NULL). */
pump_status_t pump_refine_bwd(const pump_refine_args *a, float *d_grad, float *d_J,
                              pump_stream_t stream);

/* `iters` steps of gradient descent with a backtracking (Armijo) step per
 * path, starting from a->d_nodes (not modified) and writing the refined
 * nodes to d_nodes_out (same layout) and their J to d_J (may be NULL).  The
 * loop of 2 launches per step is captured once into a CUDA graph kept in
 * ctx and replayed while the arguments stay the same. */
pump_status_t pump_refine_paths(pump_ctx *ctx, const pump_refine_args *a, int iters,
                                float *d_nodes_out, float *d_J, pump_stream_t stream);

/* Candidate paths given by node states, evaluated as the reference evaluates
 * each goal candidate and smoothing iterate (PUMP.cu:370-385, 492-502), all
 * at once: the dense path at dt = 0.05 of findOptimalPath (2pBVP.cu:5-36;
 * optimal times by toptBisection with tmax 5, or the precision mode), its MC
 * CP over the time-major particle table (collisionProbability,
 * collisionProbability.cu:4-37), and the smoothing's cost (toptBisection
 * with tmax 2 and cost per segment, PUMP.cu:499-502).  Host node arrays;
 * h_cp[k] = -1 when path k's dense path has more states than the table has
 * rows.  Synchronises the stream. */
pump_status_t pump_path_cp(pump_ctx *ctx, const float *h_nodes, const int *h_offset,
                           const int *h_count, int n_paths, int mode, const float *d_table_t,
                           int Pmc, int T_rows, float offset_mult, const float *d_obstacles,
                           int num_obstacles, float *h_cp, float *h_cost, int *h_len,
                           pump_stream_t stream);

/* ---------------------------------------------------------- whole query */
typedef struct pump_problem {
  int N;              /* samples (the reference's compile-time NUM) */
  int num_disc;       /* edge discretisation (mainPUMP.cu:57, default 8) */
  int num_hsmc;       /* HSMC particles (mainPUMP.cu:68, default 128) */
  int num_mc;         /* MC particles = table width (hardCoded.cuh:13, default 2048) */
  int table_rows;     /* particle table rows at dt = 0.05 s (default 400) */
  int num_obstacles;
  const float *obstacles; /* host, num_obstacles x 12 */
  float init[6], goal[6], lo[6], hi[6];
  float offset_mult;  /* noise multiplier (input file line 5) */
  float cp_target;    /* argv[2] */
  float cp_factor;    /* argv[3] (eta) */
  uint64_t seed;      /* particle stream key */
  int bvp_mode;       /* PUMP_BVP_PARITY or PUMP_BVP_PRECISION */
  const float *samples; /* optional host N x 6; NULL = Halton (sampler.cu:20-41) */
  int refine_iters;   /* > 0: refine the returned path (pump_refine_paths), accepted
                         only if its MC CP stays <= cp_target; 0 (default) = the reference */
  float refine_lambda; /* bound weight of the refinement (default 10) */
  int max_paths;      /* stored-path capacity; 0 (default) = the reference's
                         maxPathCount = (int)(2 N sqrt(N)) (mainPUMP.cu:623).  The
                         reference ends the search past it (PUMP.cu:62-76);
                         here the query ends with PUMP_ERR_CAPACITY */
  float disc_len;     /* > 0: waypoints per edge by edge length (no counterpart in
                         the reference, which uses num_disc for every edge):
                         edge e gets numDisc_e = ceil(L_e / disc_len) clamped to
                         [disc_min, num_disc], L_e the binary32 distance of its end
                         positions (pump_disc_offsets); 0 (default): num_disc */
  int disc_min;       /* the smallest per-edge numDisc (default 3, 4 waypoints) */
} pump_problem;

typedef struct pump_plan_result {
  float rn;
  long long num_edges;
  int iterations;       /* exploration iterations */
  int num_paths;        /* stored paths */
  int num_considered;   /* wavefront expansions (sum over iterations) */
  int goal_paths;
  int success;
  int soln_path_idx;
  float soln_cp;        /* MC CP of the returned (smoothed) path */
  float soln_cost;
  int path_len;         /* states written to path (dt = 0.05 s) */
  float *path;          /* host buffer, path_cap x 6 (may be NULL) */
  int path_cap;
  int *nodes;           /* host buffer for the node sequence, init first */
  int nodes_cap;
  int num_nodes;
  /* stage wall times in milliseconds */
  double ms_roadmap, ms_online, ms_explore, ms_search, ms_total;
  /* HSMC expansions per iteration (first 32 iterations) */
  int wavefront_sizes[32];
  /* optional exploration trace: (parent path, edge) of every expansion in
   * launch order; host buffer of wf_trace_cap ints (may be NULL) */
  int *wf_trace;
  long long wf_trace_cap;
  long long wf_trace_len;
  /* bytes copied host->device and device->host by this query */
  long long h2d_bytes, d2h_bytes;
  /* caller buffer (may be NULL): the reference's discretisation for the
   * controller (PUMP.cu:553-579, the rows of discretizedPath.txt) at dt 0.05
   * along the final smoothing iterate; ctrl_len is the row count even when
   * it exceeds ctrl_cap (then the first ctrl_cap rows are written) */
  float *ctrl_path;
  int ctrl_cap;
  int ctrl_len;
  /* refinement (problem.refine_iters > 0): the refined path's MC CP and
   * cost, and whether it replaced the returned path */
  float refine_cp, refine_cost;
  int refined;
  /* of ms_explore: time from each iteration's first launch to its counters
   * back on the host (the iteration's device work and read-backs) */
  double ms_explore_wait;
  /* every stage: time the host spent waiting for the device (stream
   * synchronisations), and how many times it waited */
  double ms_wait;
  int num_waits;
  /* optional caller buffers (either may be NULL): the stored paths' start
   * times (the reference's pathTime, PUMP.cu:185-240) and their HSMC particle
   * masks (bit-packed, ceil(num_hsmc / 32) words per path), written when
   * path_state_cap >= num_paths.  With the exploration trace they give every
   * HSMC launch's inputs. */
  float *path_time;
  uint32_t *path_valid;
  int path_state_cap;
} pump_plan_result;

/* Fills a problem with the reference's defaults (mainPUMP.cu:51-72). */
void pump_problem_defaults(pump_problem *pb);

/* Reads the reference's input file (README.md:10-11, parsed as
 * mainPUMP.cu:152-230) into pb; obstacles are stored in a buffer owned by
 * the library until the next call from this thread. */
pump_status_t pump_read_input(const char *path, pump_problem *pb);

/* One planning query: roadmap, online checks, exploration, solution search
 * and smoothing (mainPUMP.cu:248-687 and PUMP(), PUMP.cu:3-607). */
pump_status_t pump_plan(pump_ctx *ctx, const pump_problem *pb, pump_plan_result *res,
                        pump_stream_t stream);

/* Many independent queries at once.  `workers` host threads each own a
 * context and a non-blocking CUDA stream on `device` and take queries in
 * order from a shared counter, so one query's kernels and copies overlap
 * another's host-side search.  results[k] is filled as pump_plan fills it
 * (its path/nodes buffers are the caller's) and statuses[k] receives query
 * k's status.  Returns PUMP_OK when every query ran, whatever its own status;
 * pump_last_error() then names the first query (in query order) that failed
 * with an error other than PUMP_ERR_NO_SOLUTION, and its message.
 * Queries with Halton samples (samples == NULL) that share a BVP mode and
 * state bounds share one roadmap: Halton point n depends on n and the bounds
 * only, so the pair BVPs of points 1 .. max(N)-2 are computed once per group
 * and each query adds only its 4N-6 pairs touching init or goal.  A query's
 * edges are checked when its search first reaches their source node (its
 * other edges are never checked).  Results are identical to pump_plan's.
 * The reference plans one query per process run (mainPUMP.cu:82-712). */
pump_status_t pump_plan_batch(int device, const pump_problem *problems, pump_plan_result *results,
                              pump_status_t *statuses, int n, int workers);

/* Search loop form (process-wide; no reference counterpart).  As a graph,
 * the whole loop of PUMP.cu:39-290 is one launch of a CUDA graph per query:
 * a conditional while node repeats the iteration's kernels, and a control
 * kernel keeps the loop's counters on the device.  Each context
 * instantiates the graph once per shape class and reuses it.  Otherwise the
 * host drives the loop, one synchronisation per iteration.  Results are the
 * same.  level 0: the host drives every loop; 1 (the default): pump_plan's
 * loops run as graphs, pump_plan_batch's workers drive theirs (many graph
 * loops at once ran slower than host-driven ones); 2: both run as graphs.
 * A result that asks for the wavefront trace is always host-driven.  The
 * environment variable PUMP_SEARCH_GRAPH (0, 1, 2) sets the starting
 * level. */
void pump_search_graph(int level);

/* Grouped search loops of pump_plan_batch (process-wide; no reference
 * counterpart).  With max_group > 1, a worker whose query reaches its
 * search loop joins the group being formed; the group's loop runs as one
 * launch of a loop graph whose kernels serve all of its queries in each
 * iteration (the expansion, edge checks and store pass give each query a
 * share of their grid; HSMC's blocks take the chunks of every query's
 * wavefront in turn), and whose while node repeats the iteration until every
 * query's loop has ended.  A group is launched when it holds max_group
 * queries (at most 16), when every worker still planning is waiting or
 * running a group, or when its first query has waited window_us
 * microseconds; two groups may run at once.  Each query's results are the
 * same as pump_plan's.  max_group 1 (the default): each worker drives its
 * own loop (pump_search_graph).  The environment variable PUMP_BATCH_GROUPS
 * ("max_group" or "max_group,window_us") sets the starting values. */
void pump_batch_groups(int max_group, int window_us);

#ifdef __cplusplus
}
#endif
#endif /* PUMP_GB300_H */
