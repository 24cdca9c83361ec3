/*
 * pump_oracle.h -- CPU restatement of the PUMP hot path (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, the smoke check and bench.py's
 * CPU-baseline leg may load this library, and only as the checker or as the
 * timed CPU baseline; the product (pump_gb300) never links or calls it.
 *
 * Every function restates one piece of the reference (StanfordASL/PUMP,
 * file:line cited beside each declaration) in plain C.  Arithmetic follows
 * the reference's C++ source exactly: each operation is evaluated in the type
 * the C++ promotion rules give it (float, or double where a pow() or a
 * double literal promotes it), rounded once, with no fused multiply-add
 * contraction (build with -ffp-contract=off), and pow(x, n) for n = 2, 3, 4
 * correctly rounded (computed as exact binary64 products of the float x).
 * The reference's own code, built for the CPU with the same integer-power
 * rule (oracle/build_ref.sh), produces bit-identical results; the golden
 * fixtures under tests/golden/ pin this.
 *
 * The state dimension is fixed at 6 (3D double integrator) as in the
 * reference (mainPUMP.cu:84-87).
 */
#ifndef PUMP_ORACLE_H
#define PUMP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_DIM 6

/* ---------------- particle stream (replaces the missing hardCoded.cu) -------- */
/* Philox4x32-10 block (Salmon, Moraes, Dror, Shaw, SC'11). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* ln(x), x > 0, from +,-,*,/ only (atanh series); deterministic across platforms. */
double orc_det_log(double x);
/* sin(2 pi u), cos(2 pi u) for u in [0,1) from +,-,*,/ only (Taylor series). */
void orc_det_sincos_2pi(double u, double *s, double *c);
/* Closed-loop tracking-error particles.  Writes position errors (unscaled;
 * callers multiply by the noise multiplier as the reference does) in the two
 * layouts the reference uses (hardCoded.cuh:15-19):
 *   tmajor[t][p][3]  (xcombTime, used by HSMC)   -- may be NULL
 *   pmajor[p][t][3]  (xcomb, used by MC CP)      -- may be NULL  */
void orc_particle_tables(uint64_t seed, int P, int T, float *tmajor, float *pmajor);
/* FP64 per-axis covariance of the same model: cov[t*3 + {0,1,2}] =
 * (var_pos, cov_pos_vel, var_vel) at step t. */
void orc_particle_cov(int T, double *cov);

/* ---------------- 2pBVP (2pBVP.cu) ---------------- */
float orc_cost(float tau, const float *x0, const float *x1);              /* 2pBVP.cu:97-107 */
float orc_dcost(float tau, const float *x0, const float *x1);             /* 2pBVP.cu:109-115 */
/* 2pBVP.cu:71-95.  *evals (may be NULL) receives the number of cost evaluations. */
float orc_topt_bisection(const float *x0, const float *x1, float tmax, int *evals);
void orc_path_point(float t, float tau, const float *x0, const float *x1, float *x); /* 2pBVP.cu:117-131 */
/* 2pBVP.cu:53-69: writes numDisc+1 states, returns topt (tmax 5). */
float orc_find_discretized_path(float *split, const float *x0, const float *x1, int numDisc);
/* 2pBVP.cu:5-36.  Writes at most cap states; returns total time and sets
 * *len.  *len = -1 if the path needs more than cap states (the reference
 * overflows its stack buffer there). */
float orc_find_optimal_path(float dt, float *split, int cap, const float *xs, int n, int *len);
/* 2pBVP.cu:133-150 over all ordered pairs i != j, idx = i*(N-1)+j-(i<j). */
void orc_bvp_pairs(int N, const float *samples, float tmax, float *copts, float *topts);

/* Precision-mode reference: the global minimiser over (0, tmax] of the same
 * cost function written out as A0/t^3 + A1/t^2 + A2/t + A3 + A4 t, found in
 * long double by scanning c' on a log grid of 4000 points over
 * [1e-4 tmax, tmax], bisecting every -/+ sign change 200 times, and comparing
 * the candidates with tmax.  An independent algorithm for checking the GPU's
 * closed-form root solver. */
void orc_bvp_precise(const float *x0, const float *x1, float tmax, double *topt, double *cost);
/* Exact cost c(t) of a pair in long double (for stating the parity method's
 * cost excess over the optimum). */
double orc_cost_exact(double t, const float *x0, const float *x1);

/* ---------------- sampler (sampler.cu) ---------------- */
float orc_halton(int n, int b);                                           /* sampler.cu:43-57 */
void orc_halton_samples(int N, float *samples, const float *init, const float *goal,
                        const float *lo, const float *hi);                 /* sampler.cu:20-41 */
void orc_sample_free(int N, const float *samples, int nobs, const float *obs,
                     uint8_t *isFree);                                     /* sampler.cu:61-88 */

/* ---------------- roadmap (mainPUMP.cu:258-392) ---------------- */
/* rn = element k of ascending-sorted copts (mainPUMP.cu:303-304). */
float orc_select_kth(long long count, const float *v, long long k);
/* Edges are pairs with copt < rn, numbered in (i asc, j asc) order
 * (mainPUMP.cu:327-346).  Returns the edge count E and fills (when not NULL)
 * src[E], dst[E], coptE[E], toptE[E]. */
long long orc_build_edges(int N, const float *copts, const float *topts, float rn,
                          int *src, int *dst, float *coptE, float *toptE);
/* Waypoints of every edge (mainPUMP.cu:339): disc[E][numDisc+1][6]. */
void orc_discretize_edges(long long E, const int *src, const int *dst, const float *samples,
                          int numDisc, float *disc);
/* Per-edge waypoint counts by edge length (no reference counterpart; the
 * reference uses one numDisc per problem): numDisc_e = ceil(L_e / discLen)
 * clamped to [minDisc, maxDisc] (maxDisc everywhere when discLen <= 0), L_e
 * = sqrtf((dx*dx + dy*dy) + dz*dz) of the end positions in binary32.  off[e]
 * is edge e's first waypoint, off[E] the total (returned). */
long long orc_disc_offsets(long long E, const int *src, const int *dst, const float *samples,
                           float discLen, int minDisc, int maxDisc, long long *off);
/* The waypoint stages over that ragged layout: edge e's waypoints are rows
 * off[e] .. off[e+1]-1 of disc, its half-spaces rows off[e]*maxHS ... */
void orc_discretize_edges_off(long long E, const int *src, const int *dst, const float *samples,
                              const long long *off, float *disc);
void orc_free_edges_off(long long E, const long long *off, const float *disc, int nobs,
                        const float *obs, uint8_t *isFreeEdge);
void orc_cache_halfspaces_off(long long E, const long long *off, const float *disc,
                              const uint8_t *isFreeEdge, int nobs, const float *obs, int maxHS,
                              float maxd2, float *as, float *bs, int *count);
void orc_hsmc_propagate_off(int numNew, const long long *off, const int *wfEdge, const int *wfPrev,
                            int base, const float *as, const float *bs, const float *times,
                            const float *topts, float dt, int maxHS, const float *offsetsT,
                            float offsetMult, int Pmc, uint8_t *valid, int P, float *pathCP);
/* Heuristic h (mainPUMP.cu:351-355). */
void orc_heuristic(int N, const float *samples, const float *goal, float *h);

/* ---------------- collision check (collisionCheck.cu) ---------------- */
int orc_is_motion_valid(const float *v, const float *w, int nobs, const float *obs); /* :65-143 */
void orc_free_edges(long long E, int numDisc, const float *disc, int nobs, const float *obs,
                    uint8_t *isFreeEdge);                                  /* :5-37 */

/* ---------------- half-spaces (hsmc.cu) ---------------- */
/* setupAsBs (hsmc.cu:201-211) followed by cacheHalfspaces (hsmc.cu:10-99).
 * count[] of non-free edges is left as given (the reference leaves it
 * uninitialised). */
void orc_cache_halfspaces(long long E, int W, const float *disc, const uint8_t *isFreeEdge,
                          int nobs, const float *obs, int maxHS, float maxd2,
                          float *as, float *bs, int *count);

/* ---------------- HSMC (PUMP.cu:613-758) ---------------- */
/* propagateValidParticles + calculateCP_HSMC for numNew new paths; valid is
 * one byte per (path, particle) as in the reference. */
void orc_hsmc_propagate(int numNew, int W, const int *wfEdge, const int *wfPrev, int base,
                        const float *as, const float *bs, const float *times, const float *topts,
                        float dt, int maxHS, const float *offsetsT, float offsetMult, int Pmc,
                        uint8_t *valid, int P, float *pathCP);

/* ---------------- full Monte Carlo CP (collisionProbability.cu) ---------------- */
/* MCCP + reduce (collisionProbability.cu:4-92).  pmajor has stride T_stride
 * per particle.  Returns the hit count; *cp = hits / Pmc. */
int orc_mccp(const float *path, int T, const float *pmajor, int T_stride, float offsetMult,
             int nobs, const float *obs, int Pmc, float *cp);

/* ---------------- frontier compaction (GMT.cu:48-76, 166-176) ---------------- */
/* orc_mccp with the collision tests in binary64; returns the hits. */
int orc_mccp64(const float *path, int T, const float *pmajor, int T_stride, float offsetMult,
               int nobs, const float *obs, int Pmc);

/* Exclusive scan of flags then scatter of set indices; returns the count. */
int orc_frontier_compact(int N, const uint8_t *flags, int *active);

/* ---------------- whole query (mainPUMP.cu:248-687, PUMP.cu:3-607) ---------------- */
typedef struct orc_problem {
  int N;                 /* samples (NUM) */
  int numDisc;           /* edge discretisation (mainPUMP.cu:57) */
  int P;                 /* HSMC particles (mainPUMP.cu:68) */
  int Pmc;               /* MC particles = particle table width (hardCoded.cuh:13) */
  int T_table;           /* particle table steps (hardCoded.cuh:12) */
  int numObs;
  const float *obstacles;  /* numObs * 12: lo[6], hi[6] */
  float init[6], goal[6], lo[6], hi[6];
  float offsetMult, cpTarget, cpFactor;
  const float *tmajor;   /* T_table x Pmc x 3 */
  const float *pmajor;   /* Pmc x T_table x 3 */
  const float *samples;  /* optional N x 6; NULL = Halton as the reference */
  float discLen;         /* > 0: per-edge waypoint counts by edge length (orc_disc_offsets,
                            numDisc the largest); 0: numDisc on every edge, as the reference */
  int discMin;           /* the smallest per-edge numDisc */
} orc_problem;

typedef struct orc_result {
  int status;            /* 0 ok, 1 capacity (maxPathCount), 2 output path over table */
  float rn;
  long long numEdges;
  int itrs;              /* exploration iterations run */
  int numPaths;          /* stored paths */
  int numConsidered;     /* sum of wavefront sizes */
  int goalPathCount;
  int success;
  int solnPathIdx;
  float solnCP, solnCost;  /* after smoothing (lastSmoothBelow*) */
  int pathLen;           /* states in the smoothed output path */
  /* caller-provided buffers (may be NULL) */
  float *path;           /* capacity path_cap states x 6 */
  int path_cap;
  int *nodes;            /* node sequence of the solution path, init first */
  int nodes_cap;
  int numNodes;
  /* exploration trace: per iteration, wavefront size (caller buffer of 32) */
  int *wavefront_sizes;
  /* optional full wavefront trace: concatenated (pathPrev, edge) pairs */
  int *wf_trace;
  long long wf_trace_cap;
  long long wf_trace_len;
  /* controller discretisation of the final smoothing iterate (PUMP.cu:553-569) */
  float *ctrl_path;      /* capacity ctrl_cap states x 6 */
  int ctrl_cap;
  int ctrlLen;           /* rows the reference writes to discretizedPath.txt */
} orc_result;

/* The reference's discretisation for the controller (PUMP.cu:553-569): for
 * each segment of the n node states xs, tau = toptBisection(.., 2) gives
 * (int)(tau/0.05 + 1) intervals and findDiscretizedPath (tmax 5) fills them;
 * the row count is accumulated as the reference does (an int += float).
 * Writes min(rows, cap) rows to out (unwritten rows zero) and returns rows. */
int orc_control_path(const float *xs, int n, float *out, int cap);

/* Runs roadmap build, online checks, exploration, solution search and
 * smoothing exactly as the reference's main() and PUMP() do. */
int orc_plan(const orc_problem *pb, orc_result *res);

/* ---------------- path refinement objective and its adjoint (binary64) ----------------
 * Not a function of the reference: the objective the refinement after the
 * search minimises, defined here in binary64 as the checker of the device
 * adjoint.  For a path of n node states x_0..x_{n-1} (6 each):
 *   J = sum_i c(tau_i; x_i, x_{i+1}) + lambda * B
 * c is the reference's 2pBVP cost (2pBVP.cu:97-107) and tau_i its global
 * minimiser on (0, tmax].  B sums, over the waypoints p(s), v(s) at
 * s = k/W (k < W) of every segment (the cubic of pathPoint, 2pBVP.cu:117-131)
 * and over every box, Phi(-d / (offsetMult * sigma(T))): d = |a| with a the
 * offset from the waypoint to the box's closest point minus its component
 * along the velocity (the half-space of cacheHalfspaces, hsmc.cu:70-96,
 * without its distance gate or slot limit), sigma^2(T) = the closed-loop
 * position variance at the waypoint's time T = tau_0 + .. + tau_{i-1} + s tau_i
 * (linear between steps of dt, last row beyond the table) + sigmaFloor^2. */
typedef struct orc_refine_args {
  int W;
  double tmax;
  int numObs;
  const float *obstacles;  /* numObs x 12: lo[6], hi[6] */
  double offsetMult;
  const double *posVar;    /* per-axis position variance per step, T_rows */
  int T_rows;
  double dt;
  double sigmaFloor;
} orc_refine_args;

/* Global minimiser of the cost on (0, tmax] in binary64; *clamped = 1 when it
 * is tmax with the cost still decreasing there. */
double orc_tau_exact(const double *x0, const double *x1, double tmax, int *clamped);
/* Per-axis position variance of the particle model per step (orc_particle_cov's first entry). */
void orc_position_variance(int T, double *var);
double orc_refine_objective(const orc_refine_args *a, const double *nodes, int n, double lambda,
                            double *cost, double *bound);
/* dJ/dx for every node (rows 0 and n-1 are zero); returns J. */
double orc_refine_grad(const orc_refine_args *a, const double *nodes, int n, double lambda,
                       double *grad);

#ifdef __cplusplus
}
#endif
#endif
