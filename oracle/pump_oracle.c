/*
 * pump_oracle.c -- CPU restatement of the PUMP hot path (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY (see pump_oracle.h).  Build with
 * -ffp-contract=off so that no multiply-add is fused: every expression below
 * is written with the evaluation types of the reference's C++ source, one
 * rounding per operation.
 */
#include "pump_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================
 * Integer powers, correctly rounded for float-valued x (x*x is exact).
 * The reference writes pow(float, int); C++ promotes it to
 * pow(double, double) (2pBVP.cu:99-105).
 * ==================================================================== */
static inline double p2f(float x) { double d = x; return d * d; }
static inline double p3f(float x) { double d = x; return (d * d) * d; }
static inline double p4f(float x) { double d = x; double s = d * d; return s * s; }

/* ======================================================================
 * Particle stream
 * ==================================================================== */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ln(x) = e ln2 + 2 atanh(s), s = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)).
 * |s| <= 0.1716, s^2 <= 0.0295: 13 odd terms reach 1e-19 relative. */
double orc_det_log(double x) {
  int e;
  double m = frexp(x, &e);                 /* exact: x = m 2^e, m in [0.5,1) */
  if (m < 0.70710678118654752440) { m = m * 2.0; e = e - 1; }
  double s = (m - 1.0) / (m + 1.0);
  double z = s * s;
  double t = 1.0 / 25.0;
  t = t * z + 1.0 / 23.0;
  t = t * z + 1.0 / 21.0;
  t = t * z + 1.0 / 19.0;
  t = t * z + 1.0 / 17.0;
  t = t * z + 1.0 / 15.0;
  t = t * z + 1.0 / 13.0;
  t = t * z + 1.0 / 11.0;
  t = t * z + 1.0 / 9.0;
  t = t * z + 1.0 / 7.0;
  t = t * z + 1.0 / 5.0;
  t = t * z + 1.0 / 3.0;
  t = t * z + 1.0;
  double lm = 2.0 * s * t;
  return (double)e * 0.69314718055994530942 + lm;
}

/* sin/cos of 2 pi u: quadrant k = floor(4u) (exact), theta = frac(4u) pi/2,
 * Taylor series in theta^2 to degree 25 (error < 1e-19 for theta <= pi/2). */
void orc_det_sincos_2pi(double u, double *s, double *c) {
  double q = u * 4.0;
  int k = (int)q;
  double f = q - (double)k;
  double th = f * 1.57079632679489661923;
  double z = th * th;
  double sn = -1.0 / 15511210043330985984000000.0; /* -1/25! */
  sn = sn * z + 1.0 / 25852016738884976640000.0;    /*  1/23! */
  sn = sn * z - 1.0 / 51090942171709440000.0;       /* -1/21! */
  sn = sn * z + 1.0 / 121645100408832000.0;         /*  1/19! */
  sn = sn * z - 1.0 / 355687428096000.0;            /* -1/17! */
  sn = sn * z + 1.0 / 1307674368000.0;              /*  1/15! */
  sn = sn * z - 1.0 / 6227020800.0;                 /* -1/13! */
  sn = sn * z + 1.0 / 39916800.0;                   /*  1/11! */
  sn = sn * z - 1.0 / 362880.0;                     /* -1/9! */
  sn = sn * z + 1.0 / 5040.0;                       /*  1/7! */
  sn = sn * z - 1.0 / 120.0;                        /* -1/5! */
  sn = sn * z + 1.0 / 6.0;                          /*  1/3! */
  sn = sn * z - 1.0;
  sn = -(sn * th);
  double cs = 1.0 / 620448401733239439360000.0;     /*  1/24! */
  cs = cs * z - 1.0 / 1124000727777607680000.0;     /* -1/22! */
  cs = cs * z + 1.0 / 2432902008176640000.0;        /*  1/20! */
  cs = cs * z - 1.0 / 6402373705728000.0;           /* -1/18! */
  cs = cs * z + 1.0 / 20922789888000.0;             /*  1/16! */
  cs = cs * z - 1.0 / 87178291200.0;                /* -1/14! */
  cs = cs * z + 1.0 / 479001600.0;                  /*  1/12! */
  cs = cs * z - 1.0 / 3628800.0;                    /* -1/10! */
  cs = cs * z + 1.0 / 40320.0;                      /*  1/8! */
  cs = cs * z - 1.0 / 720.0;                        /* -1/6! */
  cs = cs * z + 1.0 / 24.0;                         /*  1/4! */
  cs = cs * z - 0.5;                                /* -1/2! */
  cs = cs * z + 1.0;
  switch (k & 3) {
    case 0: *s = sn; *c = cs; break;
    case 1: *s = cs; *c = -sn; break;
    case 2: *s = -sn; *c = -cs; break;
    default: *s = -cs; *c = sn; break;
  }
}

/* Closed-loop tracking error of the double integrator at the reference's
 * offset step dt = 0.05 s (mainPUMP.cu:60), one axis at a time:
 *   a_t   = w_t - (KP p_t + KD v_t),   w_t ~ N(0, SIGMA_W^2)
 *   p_t+1 = (p_t + DT v_t) + H2 a_t,    v_t+1 = v_t + DT a_t,   p_0 = v_0 = 0
 * with DT = 0.05, H2 = DT^2/2 = 0.00125, KP = 16, KD = 5.6 (a PD tracking
 * law, closed-loop spectral radius 0.860) and SIGMA_W = 4, giving a
 * stationary position standard deviation of 0.069 before the noise
 * multiplier.  Noise for particle p at step t uses Philox counter
 * (p, t, 0, 0) and key (seed lo, seed hi); its four 32-bit words give
 * u = (word + 0.5) 2^-32 and Box-Muller pairs (u0,u1) -> axes x,y and
 * (u2,u3) -> axis z. */
#define ORC_DT 0.05
#define ORC_H2 0.00125
#define ORC_KP 16.0
#define ORC_KD 5.6
#define ORC_SIGMA_W 4.0

static void orc_gauss3(uint64_t seed, uint32_t p, uint32_t t, double z[3]) {
  uint32_t ctr[4] = {p, t, 0u, 0u};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  orc_philox4x32_10(ctr, key, o);
  const double sc = 2.3283064365386962890625e-10; /* 2^-32 */
  double u0 = ((double)o[0] + 0.5) * sc, u1 = ((double)o[1] + 0.5) * sc;
  double u2 = ((double)o[2] + 0.5) * sc, u3 = ((double)o[3] + 0.5) * sc;
  double r0 = sqrt(-2.0 * orc_det_log(u0));
  double r1 = sqrt(-2.0 * orc_det_log(u2));
  double s0, c0, s1, c1;
  orc_det_sincos_2pi(u1, &s0, &c0);
  orc_det_sincos_2pi(u3, &s1, &c1);
  z[0] = r0 * c0;
  z[1] = r0 * s0;
  z[2] = r1 * c1;
}

void orc_particle_tables(uint64_t seed, int P, int T, float *tmajor, float *pmajor) {
  for (int p = 0; p < P; ++p) {
    double pos[3] = {0, 0, 0}, vel[3] = {0, 0, 0};
    for (int t = 0; t < T; ++t) {
      for (int d = 0; d < 3; ++d) {
        float v = (float)pos[d];
        if (tmajor) tmajor[((long long)t * P + p) * 3 + d] = v;
        if (pmajor) pmajor[((long long)p * T + t) * 3 + d] = v;
      }
      double z[3];
      orc_gauss3(seed, (uint32_t)p, (uint32_t)t, z);
      for (int d = 0; d < 3; ++d) {
        double a = ORC_SIGMA_W * z[d] - (ORC_KP * pos[d] + ORC_KD * vel[d]);
        double pn = (pos[d] + ORC_DT * vel[d]) + ORC_H2 * a;
        double vn = vel[d] + ORC_DT * a;
        pos[d] = pn;
        vel[d] = vn;
      }
    }
  }
}

void orc_particle_cov(int T, double *cov) {
  /* A_cl = [[1 - H2 KP, DT - H2 KD], [-DT KP, 1 - DT KD]], G = [H2, DT] SIGMA_W */
  const double a00 = 1.0 - ORC_H2 * ORC_KP, a01 = ORC_DT - ORC_H2 * ORC_KD;
  const double a10 = -(ORC_DT * ORC_KP), a11 = 1.0 - ORC_DT * ORC_KD;
  const double g0 = ORC_H2 * ORC_SIGMA_W, g1 = ORC_DT * ORC_SIGMA_W;
  double spp = 0, spv = 0, svv = 0;
  for (int t = 0; t < T; ++t) {
    cov[t * 3 + 0] = spp; cov[t * 3 + 1] = spv; cov[t * 3 + 2] = svv;
    /* S' = A S A^T + G G^T */
    double m00 = a00 * spp + a01 * spv, m01 = a00 * spv + a01 * svv;
    double m10 = a10 * spp + a11 * spv, m11 = a10 * spv + a11 * svv;
    double npp = m00 * a00 + m01 * a01 + g0 * g0;
    double npv = m00 * a10 + m01 * a11 + g0 * g1;
    double nvv = m10 * a10 + m11 * a11 + g1 * g1;
    spp = npp; spv = npv; svv = nvv;
  }
}

/* ======================================================================
 * 2pBVP (2pBVP.cu)
 * ==================================================================== */
/* 2pBVP.cu:3, `const float g = -9.81;` */
#define ORC_G ((float)-9.81)

float orc_cost(float tau, const float *x0, const float *x1) {
  const float g = ORC_G;
  double s;
  s = 12 * p2f(x0[0]);
  s = s + 12 * p2f(x0[2]);
  s = s + 12 * p2f(x0[1]);
  s = s + 12 * p2f(x1[0]);
  s = s + 12 * p2f(x1[2]);
  s = s - (double)(24 * x0[1] * x1[1]);
  s = s + 12 * p2f(x1[1]);
  s = s + (double)(12 * x0[4] * x0[1] * tau);
  s = s + (double)(12 * x0[1] * x1[4] * tau);
  s = s - (double)(12 * x0[3] * x1[0] * tau);
  s = s - (double)(12 * x1[3] * x1[0] * tau);
  s = s - (double)(12 * x0[5] * x1[2] * tau);
  s = s - (double)(12 * x1[5] * x1[2] * tau);
  s = s - (double)(12 * x0[4] * x1[1] * tau);
  s = s - (double)(12 * x1[4] * x1[1] * tau);
  const double t2 = p2f(tau), t3 = p3f(tau), t4 = p4f(tau);
  s = s + (4 * p2f(x0[4])) * t2;
  s = s + (4 * p2f(x0[3])) * t2;
  s = s + (4 * p2f(x0[5])) * t2;
  s = s + (double)(4 * x0[4] * x1[4]) * t2;
  s = s + (4 * p2f(x1[4])) * t2;
  s = s + (double)(4 * x0[3] * x1[3]) * t2;
  s = s + (4 * p2f(x1[3])) * t2;
  s = s + (double)(4 * x0[5] * x1[5]) * t2;
  s = s + (4 * p2f(x1[5])) * t2;
  s = s + (double)(2 * g * x0[5]) * t3;
  s = s - (double)(2 * g * x1[5]) * t3;
  s = s + t4;
  s = s + p2f(g) * t4;
  s = s + (double)(12 * x0[0] * (-2 * x1[0] + (x0[3] + x1[3]) * tau));
  s = s + (double)(12 * x0[2] * (-2 * x1[2] + (x0[5] + x1[5]) * tau));
  return (float)((1 / t3) * s);
}

float orc_dcost(float tau, const float *x0, const float *x1) {
  const float dtau = (float)0.000001;
  return (orc_cost(tau + dtau / 2, x0, x1) - orc_cost(tau - dtau / 2, x0, x1)) / dtau;
}

/* The halving loop of 2pBVP.cu:78-80 has no bound in the reference; it ends
 * for every state pair with distinct positions.  It is bounded here at 160
 * halvings (tl below 1e-50 underflows to 0 long before). */
float orc_topt_bisection(const float *x0, const float *x1, float tmax, int *evals) {
  int ev = 2;
  float tu = tmax;
  if (orc_dcost(tmax, x0, x1) < 0) {
    if (evals) *evals = ev;
    return tmax;
  }
  float tl = (float)0.01;
  int halvings = 0;
  while (ev += 2, orc_dcost(tl, x0, x1) > 0 && halvings < 160) {
    tl = tl / 2;
    ++halvings;
  }
  float topt = 0;
  float dcval = 1;
  int maxItrs = 50;
  int itr = 0;
  while ((double)fabsf(dcval) > 0.0001 && itr < maxItrs && ++itr) {
    topt = (tu + tl) / 2;
    dcval = orc_dcost(topt, x0, x1);
    ev += 2;
    if (dcval > 0)
      tu = topt;
    else
      tl = topt;
  }
  if (evals) *evals = ev;
  return topt;
}

void orc_path_point(float t, float tau, const float *x0, const float *x1, float *x) {
  const double t2 = p2f(t), t3 = p3f(t), u2 = p2f(tau), u3 = p3f(tau);
  /* x[0], x[1]: 2pBVP.cu:119-122 */
  for (int k = 0; k < 2; ++k) {
    const int a = k, b = k + 3;
    double r = (double)(t * x0[b] + x0[a]);
    r = r + (t3 * (double)(2 * x0[a] - 2 * x1[a] + (x0[b] + x1[b]) * tau)) / u3;
    r = r - (t2 * (double)(3 * x0[a] - 3 * x1[a] + (2 * x0[b] + x1[b]) * tau)) / u2;
    x[k] = (float)r;
  }
  /* x[2]: 2pBVP.cu:123-124 */
  {
    double r = (double)(t * x0[5]) * u3 + (double)x0[2] * u3;
    double q1 = -3. * x0[2] + 3. * x1[2] - 2. * x0[5] * tau - 1. * x1[5] * tau;
    r = r + (t2 * (double)tau) * q1;
    double q2 = 2. * x0[2] - 2. * x1[2] + (double)((x0[5] + x1[5]) * tau);
    r = r + t3 * q2;
    x[2] = (float)(r / u3);
  }
  /* x[3], x[4]: 2pBVP.cu:125-129 */
  for (int k = 0; k < 2; ++k) {
    const int a = k, b = k + 3;
    float f1 = -(2 * t * (3 * x0[a] - 3 * x1[a] + x1[b] * tau));
    double r = (double)f1 / u2;
    r = r + (3 * t2 * (double)(2 * x0[a] - 2 * x1[a] + x1[b] * tau)) / u3;
    double inner = 3 * t2 - (double)(4 * t * tau) + u2;
    r = r + ((double)x0[b] * inner) / u2;
    x[3 + k] = (float)r;
  }
  /* x[5]: 2pBVP.cu:130-131 */
  {
    double r = (double)x0[5] * u3;
    double q1 = -6. * x0[2] + 6. * x1[2] - 4. * x0[5] * tau - 2. * x1[5] * tau;
    r = r + (double)(t * tau) * q1;
    double q2 = 6. * x0[2] - 6. * x1[2] + 3. * x0[5] * tau + 3. * x1[5] * tau;
    r = r + t2 * q2;
    x[5] = (float)(r / u3);
  }
}

float orc_find_discretized_path(float *split, const float *x0, const float *x1, int numDisc) {
  float topt = orc_topt_bisection(x0, x1, 5, NULL);
  float dt = topt / numDisc;
  for (int d = 0; d < ORC_DIM; ++d) {
    split[d] = x0[d];
    split[d + numDisc * ORC_DIM] = x1[d];
  }
  for (int i = 1; i < numDisc; ++i) orc_path_point(dt * i, topt, x0, x1, &split[i * ORC_DIM]);
  return topt;
}

float orc_find_optimal_path(float dt, float *split, int cap, const float *xs, int n, int *len) {
  float tmax = 5;
  float toff = 0, topt = 0, t = 0, ttotal = 0;
  int Tprev = 0;
  for (int i = 0; i < n - 1; ++i) {
    const float *x0 = &xs[i * ORC_DIM], *x1 = &xs[(i + 1) * ORC_DIM];
    topt = orc_topt_bisection(x0, x1, tmax, NULL);
    int T = (int)((topt - toff) / dt + 1);
    if (T > 0 && Tprev + T > cap) {
      *len = -1;
      return ttotal;
    }
    for (int tidx = 0; tidx < T; ++tidx) {
      t = dt * tidx + toff;
      orc_path_point(t, topt, x0, x1, &split[(Tprev + tidx) * ORC_DIM]);
    }
    Tprev += T;
    toff = (t - topt) + dt;
    ttotal += topt;
  }
  *len = Tprev;
  return ttotal;
}

void orc_bvp_pairs(int N, const float *samples, float tmax, float *copts, float *topts) {
#pragma omp parallel for schedule(dynamic, 64)
  for (long long tid = 0; tid < (long long)N * N; ++tid) {
    int i = (int)(tid / N), j = (int)(tid % N);
    if (i == j) continue;
    long long idx = (long long)i * (N - 1) + j;
    if (i < j) idx--;
    float tp = orc_topt_bisection(&samples[i * ORC_DIM], &samples[j * ORC_DIM], tmax, NULL);
    topts[idx] = tp;
    copts[idx] = orc_cost(tp, &samples[i * ORC_DIM], &samples[j * ORC_DIM]);
  }
}

/* ---------------- precision-mode reference (long double) ---------------- */
typedef struct { long double A0, A1, A2, A3, A4; } orc_quartic;

static orc_quartic orc_make_quartic(const float *x0, const float *x1) {
  const long double g = (long double)ORC_G;
  long double dx = (long double)x1[0] - x0[0], dy = (long double)x1[1] - x0[1],
              dz = (long double)x1[2] - x0[2];
  long double sx = (long double)x0[3] + x1[3], sy = (long double)x0[4] + x1[4],
              sz = (long double)x0[5] + x1[5];
  orc_quartic q;
  q.A0 = 12.0L * (dx * dx + dy * dy + dz * dz);
  q.A1 = -12.0L * (dx * sx + dy * sy + dz * sz);
  q.A2 = 4.0L * ((long double)x0[3] * x0[3] + (long double)x0[4] * x0[4] + (long double)x0[5] * x0[5] +
                 (long double)x0[3] * x1[3] + (long double)x0[4] * x1[4] + (long double)x0[5] * x1[5] +
                 (long double)x1[3] * x1[3] + (long double)x1[4] * x1[4] + (long double)x1[5] * x1[5]);
  q.A3 = 2.0L * g * ((long double)x0[5] - x1[5]);
  q.A4 = 1.0L + g * g;
  return q;
}
static long double orc_qc(const orc_quartic *q, long double t) {
  return q->A0 / (t * t * t) + q->A1 / (t * t) + q->A2 / t + q->A3 + q->A4 * t;
}
static long double orc_qdc(const orc_quartic *q, long double t) {
  return -3.0L * q->A0 / (t * t * t * t) - 2.0L * q->A1 / (t * t * t) - q->A2 / (t * t) + q->A4;
}

double orc_cost_exact(double t, const float *x0, const float *x1) {
  orc_quartic q = orc_make_quartic(x0, x1);
  return (double)orc_qc(&q, (long double)t);
}

void orc_bvp_precise(const float *x0, const float *x1, float tmax, double *topt, double *cost) {
  orc_quartic q = orc_make_quartic(x0, x1);
  const int K = 4000;
  const long double tm = tmax, lo = 1e-4L * tm;
  long double best_t = tm, best_c = orc_qc(&q, tm);
  long double tp = lo, dp = orc_qdc(&q, lo);
  for (int k = 1; k < K; ++k) {
    long double t = lo * powl(tm / lo, (long double)k / (K - 1));
    if (k == K - 1) t = tm;
    long double d = orc_qdc(&q, t);
    if (dp < 0 && d > 0) {
      long double a = tp, b = t;
      for (int it = 0; it < 200; ++it) {
        long double m = 0.5L * (a + b);
        if (orc_qdc(&q, m) < 0) a = m; else b = m;
      }
      long double r = 0.5L * (a + b), c = orc_qc(&q, r);
      if (c < best_c) { best_c = c; best_t = r; }
    }
    tp = t;
    dp = d;
  }
  *topt = (double)best_t;
  *cost = (double)best_c;
}

/* ======================================================================
 * Sampler (sampler.cu)
 * ==================================================================== */
float orc_halton(int n, int b) {
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

void orc_halton_samples(int N, float *samples, const float *init, const float *goal,
                        const float *lo, const float *hi) {
  static const int bases[] = {2, 3, 5, 7, 11, 13};
  for (int d = 0; d < ORC_DIM; ++d)
    for (int n = 0; n < N; ++n)
      samples[n * ORC_DIM + d] = orc_halton(n, bases[d]) * (hi[d] - lo[d]) + lo[d];
  for (int d = 0; d < ORC_DIM; ++d) {
    samples[d] = init[d];
    samples[(N - 1) * ORC_DIM + d] = goal[d];
  }
}

void orc_sample_free(int N, const float *samples, int nobs, const float *obs, uint8_t *isFree) {
  for (int node = 0; node < N; ++node) {
    const float *p = &samples[node * ORC_DIM];
    uint8_t fr = 1;
    for (int o = 0; o < nobs && fr; ++o) {
      int notFree = 1;
      for (int d = 0; d < 3; ++d) {
        notFree = notFree && p[d] > obs[o * 12 + d] && p[d] < obs[o * 12 + 6 + d];
        if (!notFree) break;
      }
      if (notFree) fr = 0;
    }
    isFree[node] = fr;
  }
}

/* ======================================================================
 * Roadmap (mainPUMP.cu)
 * ==================================================================== */
static int cmp_float(const void *a, const void *b) {
  float x = *(const float *)a, y = *(const float *)b;
  return (x > y) - (x < y);
}

float orc_select_kth(long long count, const float *v, long long k) {
  float *c = (float *)malloc(sizeof(float) * (size_t)count);
  memcpy(c, v, sizeof(float) * (size_t)count);
  qsort(c, (size_t)count, sizeof(float), cmp_float);
  float r = c[k];
  free(c);
  return r;
}

long long orc_build_edges(int N, const float *copts, const float *topts, float rn, int *src,
                          int *dst, float *coptE, float *toptE) {
  long long e = 0, idx = 0;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      if (j == i) continue;
      if (copts[idx] < rn) {
        if (src) src[e] = i;
        if (dst) dst[e] = j;
        if (coptE) coptE[e] = copts[idx];
        if (toptE) toptE[e] = topts[idx];
        ++e;
      }
      ++idx;
    }
  return e;
}

/* Per-edge waypoint counts by edge length (no counterpart in the reference,
 * whose numDisc is one value per problem, mainPUMP.cu:57): with discLen > 0,
 * numDisc_e = ceil(L_e / discLen) clamped to [minDisc, maxDisc], L_e the
 * binary32 distance between the edge's end positions, sqrtf((dx*dx + dy*dy)
 * + dz*dz) with d = p1 - p0; otherwise every edge has maxDisc.  Writes
 * off[e] = sum over e' < e of (numDisc_e' + 1), off[E] included; returns
 * off[E]. */
static int disc_count(const float *x0, const float *x1, float discLen, int minDisc, int maxDisc) {
  if (!(discLen > 0)) return maxDisc;
  const float dx = x1[0] - x0[0], dy = x1[1] - x0[1], dz = x1[2] - x0[2];
  const float L = sqrtf(dx * dx + dy * dy + dz * dz);
  const float q = ceilf(L / discLen);
  if (!(q >= (float)minDisc)) return minDisc; /* also NaN */
  if (q > (float)maxDisc) return maxDisc;
  return (int)q;
}

long long orc_disc_offsets(long long E, const int *src, const int *dst, const float *samples,
                           float discLen, int minDisc, int maxDisc, long long *off) {
  long long t = 0;
  for (long long e = 0; e < E; ++e) {
    off[e] = t;
    t += disc_count(&samples[src[e] * ORC_DIM], &samples[dst[e] * ORC_DIM], discLen, minDisc,
                    maxDisc) + 1;
  }
  off[E] = t;
  return t;
}

static long long *uniform_offsets(long long E, int W) {
  long long *off = (long long *)malloc(sizeof(long long) * (E + 1));
  for (long long e = 0; e <= E; ++e) off[e] = e * W;
  return off;
}

void orc_discretize_edges_off(long long E, const int *src, const int *dst, const float *samples,
                              const long long *off, float *disc) {
#pragma omp parallel for schedule(dynamic, 256)
  for (long long e = 0; e < E; ++e)
    orc_find_discretized_path(&disc[off[e] * ORC_DIM], &samples[src[e] * ORC_DIM],
                              &samples[dst[e] * ORC_DIM], (int)(off[e + 1] - off[e] - 1));
}

void orc_discretize_edges(long long E, const int *src, const int *dst, const float *samples,
                          int numDisc, float *disc) {
  long long *off = uniform_offsets(E, numDisc + 1);
  orc_discretize_edges_off(E, src, dst, samples, off, disc);
  free(off);
}

void orc_heuristic(int N, const float *samples, const float *goal, float *h) {
  for (int i = 0; i < N - 1; ++i) {
    float topt = orc_topt_bisection(&samples[i * ORC_DIM], goal, 5, NULL);
    h[i] = orc_cost(topt, &samples[i * ORC_DIM], goal);
  }
  h[N - 1] = 0;
}

/* ======================================================================
 * Collision check (collisionCheck.cu)
 * ==================================================================== */
static int broadphase_valid(const float *bbMin, const float *bbMax, const float *o) {
  for (int d = 0; d < 3; ++d)
    if (bbMax[d] <= o[d] || o[6 + d] <= bbMin[d]) return 1;
  return 0;
}

static int face_contains_projection(const float *v, const float *w, float lambda, int j,
                                    const float *o) {
  for (int d = 0; d < 3; ++d) {
    float projection = v[d] + (w[d] - v[d]) * lambda;
    if (d != j && !(o[d] <= projection && projection <= o[6 + d])) return 0;
  }
  return 1;
}

static int motion_valid_q(const float *v, const float *w, const float *o) {
  for (int d = 0; d < 3; ++d) {
    float lambda;
    float v_to_w = w[d] - v[d];
    if (v[d] < o[d])
      lambda = (o[d] - v[d]) / v_to_w;
    else
      lambda = (o[6 + d] - v[d]) / v_to_w;
    if (face_contains_projection(v, w, lambda, d, o)) return 0;
  }
  return 1;
}

int orc_is_motion_valid(const float *v, const float *w, int nobs, const float *obs) {
  float bbMin[3], bbMax[3];
  for (int d = 0; d < 3; ++d) {
    if (v[d] > w[d]) { bbMin[d] = w[d]; bbMax[d] = v[d]; }
    else { bbMin[d] = v[d]; bbMax[d] = w[d]; }
  }
  for (int o = 0; o < nobs; ++o) {
    const float *ob = &obs[o * 12];
    if (!broadphase_valid(bbMin, bbMax, ob))
      if (!motion_valid_q(v, w, ob)) return 0;
  }
  return 1;
}

void orc_free_edges_off(long long E, const long long *off, const float *disc, int nobs,
                        const float *obs, uint8_t *isFreeEdge) {
#pragma omp parallel for schedule(dynamic, 256)
  for (long long e = 0; e < E; ++e) {
    int ok = 1;
    const int numDisc = (int)(off[e + 1] - off[e] - 1);
    for (int i = 0; i < numDisc && ok; ++i) {
      const float *v = &disc[(off[e] + i) * ORC_DIM];
      ok = orc_is_motion_valid(v, v + ORC_DIM, nobs, obs);
    }
    isFreeEdge[e] = (uint8_t)ok;
  }
}

void orc_free_edges(long long E, int numDisc, const float *disc, int nobs, const float *obs,
                    uint8_t *isFreeEdge) {
  long long *off = uniform_offsets(E, numDisc + 1);
  orc_free_edges_off(E, off, disc, nobs, obs, isFreeEdge);
  free(off);
}

/* ======================================================================
 * Half-spaces (hsmc.cu, bvls.cu:259-273)
 * ==================================================================== */
static void halfspaces_of_waypoint(long long wp, const float *disc, int nobs, const float *obs,
                                   int maxHS, float maxd2, float *as, float *bs, int *count);

void orc_cache_halfspaces_off(long long E, const long long *off, const float *disc,
                              const uint8_t *isFreeEdge, int nobs, const float *obs, int maxHS,
                              float maxd2, float *as, float *bs, int *count) {
  const long long nhs = off[E] * maxHS;
  for (long long i = 0; i < nhs; ++i) {
    as[i * 3 + 0] = -1; as[i * 3 + 1] = -1; as[i * 3 + 2] = -1;
    bs[i] = 1111;
  }
#pragma omp parallel for schedule(dynamic, 256)
  for (long long e = 0; e < E; ++e) {
    if (!isFreeEdge[e]) continue;
    for (long long wp = off[e]; wp < off[e + 1]; ++wp)
      halfspaces_of_waypoint(wp, disc, nobs, obs, maxHS, maxd2, as, bs, count);
  }
}

void orc_cache_halfspaces(long long E, int W, const float *disc, const uint8_t *isFreeEdge,
                          int nobs, const float *obs, int maxHS, float maxd2, float *as,
                          float *bs, int *count) {
  long long *off = uniform_offsets(E, W);
  orc_cache_halfspaces_off(E, off, disc, isFreeEdge, nobs, obs, maxHS, maxd2, as, bs, count);
  free(off);
}

/* cacheHalfspaces (hsmc.cu:10-99) for one waypoint of a free edge */
static void halfspaces_of_waypoint(long long wp, const float *disc, int nobs, const float *obs,
                                   int maxHS, float maxd2, float *as, float *bs, int *count) {
  {
    const float *pos = &disc[wp * ORC_DIM], *vel = pos + 3;
    long long hsIdx = wp * maxHS;
    int stored = 0;
    for (int o = 0; o < nobs; ++o) {
      const float *l = &obs[o * 12], *u = &obs[o * 12 + 6];
      float x[3];
      for (int d = 0; d < 3; ++d) {
        if (pos[d] <= l[d]) x[d] = l[d];
        else if (pos[d] >= u[d]) x[d] = u[d];
        else x[d] = pos[d];
      }
      for (int d = 0; d < 3; ++d) x[d] = x[d] - pos[d];
      float d2 = 0;
      for (int d = 0; d < 3; ++d) d2 += x[d] * x[d];
      if (d2 > maxd2) continue;
      float xdotv = 0, vdotv = 0;
      for (int d = 0; d < 3; ++d) {
        xdotv += x[d] * vel[d];
        vdotv += vel[d] * vel[d];
      }
      if (vdotv == 0) vdotv = (float)1e-5;
      float dotratio = xdotv / vdotv;
      for (int d = 0; d < 3; ++d) x[d] = x[d] - dotratio * vel[d];
      float xdotx = 0;
      for (int d = 0; d < 3; ++d) {
        as[hsIdx * 3 + d] = x[d];
        xdotx += x[d] * x[d];
      }
      bs[hsIdx] = xdotx;
      stored++;
      hsIdx++;
      if (stored == maxHS) break;
    }
    count[wp] = stored;
  }
}

/* ======================================================================
 * HSMC propagation and CP (PUMP.cu:613-655, 745-758)
 * ==================================================================== */
void orc_hsmc_propagate_off(int numNew, const long long *off, const int *wfEdge, const int *wfPrev,
                            int base, const float *as, const float *bs, const float *times,
                            const float *topts, float dt, int maxHS, const float *offsetsT,
                            float offsetMult, int Pmc, uint8_t *valid, int P, float *pathCP) {
#pragma omp parallel for schedule(dynamic, 16)
  for (int w = 0; w < numNew; ++w) {
    const int edge = wfEdge[w], prev = wfPrev[w];
    const long long pathIdx = (long long)base + w;
    const int W = (int)(off[edge + 1] - off[edge]);
    int collisions = 0;
    for (int p = 0; p < P; ++p) {
      int vp = valid[(long long)prev * P + p];
      float dtLocal = topts[edge] / (W - 1);
      long long hsHead = off[edge] * maxHS;
      for (int i = 0; i < W; ++i) {
        float time = times[prev] + i * dtLocal;
        int dtIdx = (int)(time / dt);
        for (int o = 0; o < maxHS; ++o) {
          const long long h = hsHead + (long long)i * maxHS + o;
          if (bs[h] >= 1000) continue;
          float LHS = 0;
          for (int d = 0; d < 3; ++d)
            LHS += offsetsT[((long long)dtIdx * Pmc + p) * 3 + d] * as[h * 3 + d];
          vp &= (LHS * offsetMult < bs[h]);
        }
      }
      valid[pathIdx * P + p] = (uint8_t)vp;
      if (!vp) collisions++;
    }
    if (pathCP) pathCP[pathIdx] = ((float)collisions) / P;
  }
}

void orc_hsmc_propagate(int numNew, int W, const int *wfEdge, const int *wfPrev, int base,
                        const float *as, const float *bs, const float *times, const float *topts,
                        float dt, int maxHS, const float *offsetsT, float offsetMult, int Pmc,
                        uint8_t *valid, int P, float *pathCP) {
  long long E = 0;
  for (int w = 0; w < numNew; ++w)
    if (wfEdge[w] + 1 > E) E = wfEdge[w] + 1;
  long long *off = uniform_offsets(E, W);
  orc_hsmc_propagate_off(numNew, off, wfEdge, wfPrev, base, as, bs, times, topts, dt, maxHS,
                         offsetsT, offsetMult, Pmc, valid, P, pathCP);
  free(off);
}

/* ======================================================================
 * Monte Carlo CP (collisionProbability.cu:39-92)
 * ==================================================================== */
int orc_mccp(const float *path, int T, const float *pmajor, int T_stride, float offsetMult,
             int nobs, const float *obs, int Pmc, float *cp) {
  int hits = 0;
#pragma omp parallel for reduction(+ : hits) schedule(dynamic, 64)
  for (int p = 0; p < Pmc; ++p) {
    float v[3], w[3];
    int coll = 0;
    for (int t = 0; t < T - 2 && !coll; ++t) {
      for (int d = 0; d < 3; ++d) {
        v[d] = path[t * ORC_DIM + d] + pmajor[((long long)p * T_stride + t) * 3 + d] * offsetMult;
        w[d] = path[(t + 1) * ORC_DIM + d] +
               pmajor[((long long)p * T_stride + t + 1) * 3 + d] * offsetMult;
      }
      if (!orc_is_motion_valid(v, w, nobs, obs)) coll = 1;
    }
    hits += coll;
  }
  if (cp) *cp = ((float)hits) / ((float)Pmc);
  return hits;
}

/* The same Monte Carlo CP with every collision-test operation in binary64
 * (positions path + offset * offsetMult formed in binary64): the binary64
 * reference the binary32 estimate of the precision mode is stated against. */
static int motion_valid64(const double *v, const double *w, const float *o) {
  double bbMin[3], bbMax[3];
  for (int d = 0; d < 3; ++d) {
    if (v[d] > w[d]) { bbMin[d] = w[d]; bbMax[d] = v[d]; }
    else { bbMin[d] = v[d]; bbMax[d] = w[d]; }
  }
  for (int d = 0; d < 3; ++d)
    if (bbMax[d] <= o[d] || o[6 + d] <= bbMin[d]) return 1;
  for (int j = 0; j < 3; ++j) {
    const double v_to_w = w[j] - v[j];
    const double lambda = v[j] < o[j] ? (o[j] - v[j]) / v_to_w : (o[6 + j] - v[j]) / v_to_w;
    int inside = 1;
    for (int d = 0; d < 3 && inside; ++d) {
      const double pr = v[d] + (w[d] - v[d]) * lambda;
      if (d != j && !(o[d] <= pr && pr <= o[6 + d])) inside = 0;
    }
    if (inside) return 0;
  }
  return 1;
}

int orc_mccp64(const float *path, int T, const float *pmajor, int T_stride, float offsetMult,
               int nobs, const float *obs, int Pmc) {
  int hits = 0;
#pragma omp parallel for reduction(+ : hits) schedule(dynamic, 64)
  for (int p = 0; p < Pmc; ++p) {
    int coll = 0;
    for (int t = 0; t < T - 2 && !coll; ++t) {
      double v[3], w[3];
      for (int d = 0; d < 3; ++d) {
        v[d] = (double)path[t * ORC_DIM + d] +
               (double)pmajor[((long long)p * T_stride + t) * 3 + d] * (double)offsetMult;
        w[d] = (double)path[(t + 1) * ORC_DIM + d] +
               (double)pmajor[((long long)p * T_stride + t + 1) * 3 + d] * (double)offsetMult;
      }
      for (int o = 0; o < nobs && !coll; ++o)
        if (!motion_valid64(v, w, &obs[o * 12])) coll = 1;
    }
    hits += coll;
  }
  return hits;
}

/* ======================================================================
 * Frontier compaction (GMT.cu:48-76, 166-176)
 * ==================================================================== */
int orc_frontier_compact(int N, const uint8_t *flags, int *active) {
  int n = 0;
  for (int i = 0; i < N; ++i)
    if (flags[i]) active[n++] = i;
  return n;
}

/* ======================================================================
 * Whole query (mainPUMP.cu:248-687, PUMP.cu:3-607)
 * ==================================================================== */
static int build_xs(int pathIdx, const int *pathPrev, const int *pathNode, const float *samples,
                    float *xs, int *nodes, int cap) {
  /* PUMP.cu:377-386: nodes from the goal back to init, stored init first */
  int n = 0, p = pathIdx;
  while (p != -2) { ++n; p = pathPrev[p]; }
  if (n > cap) return -1;
  p = pathIdx;
  for (int k = n - 1; k >= 0; --k) {
    int node = pathNode[p];
    if (nodes) nodes[k] = node;
    for (int d = 0; d < ORC_DIM; ++d) xs[k * ORC_DIM + d] = samples[node * ORC_DIM + d];
    p = pathPrev[p];
  }
  return n;
}

typedef struct { float cost; int idx; } cost_idx;
static int cmp_cost_idx(const void *a, const void *b) {
  const cost_idx *x = (const cost_idx *)a, *y = (const cost_idx *)b;
  if (x->cost < y->cost) return -1;
  if (x->cost > y->cost) return 1;
  return (x->idx > y->idx) - (x->idx < y->idx);
}

int orc_control_path(const float *xs, int n, float *out, int cap) {
  const float controlDt = 0.05f;
  int rows = 1;
  for (int i = 0; i < n - 1; ++i) {
    float tau = orc_topt_bisection(&xs[i * ORC_DIM], &xs[(i + 1) * ORC_DIM], 2, NULL);
    rows = (int)((float)rows + (tau / controlDt + 1));  /* PUMP.cu:556-560: int += float */
  }
  if (out && cap > 0) memset(out, 0, sizeof(float) * ORC_DIM * (size_t)cap);
  float *seg = NULL;
  int segCap = 0, cur = 0;
  for (int i = 0; i < n - 1; ++i) {
    float tau = orc_topt_bisection(&xs[i * ORC_DIM], &xs[(i + 1) * ORC_DIM], 2, NULL);
    int nw = (int)(tau / controlDt + 1);
    if (nw + 1 > segCap) {
      segCap = nw + 1;
      seg = (float *)realloc(seg, sizeof(float) * ORC_DIM * (size_t)segCap);
    }
    orc_find_discretized_path(seg, &xs[i * ORC_DIM], &xs[(i + 1) * ORC_DIM], nw);
    for (int r = 0; r <= nw; ++r)
      if (cur + r < cap && out)
        memcpy(&out[(size_t)(cur + r) * ORC_DIM], &seg[(size_t)r * ORC_DIM], sizeof(float) * ORC_DIM);
    cur += nw;
  }
  free(seg);
  return rows;
}

int orc_plan(const orc_problem *pb, orc_result *res) {
  const int N = pb->N, numDisc = pb->numDisc, P = pb->P, Pmc = pb->Pmc;
  const int nobs = pb->numObs;
  const float *obs = pb->obstacles;
  const float dt = (float)0.05, lambda = (float)0.5, epsCost = (float)0.0002,
              epsCP = (float)0.0002;
  const int numBuckets = 2;
  const float maxd2 = (float)(0.1 * pb->offsetMult * pb->offsetMult); /* mainPUMP.cu:201 */
  const int maxHS = nobs > 5 ? 5 : nobs;                              /* mainPUMP.cu:241 */
  memset(res->wavefront_sizes ? (void *)res->wavefront_sizes : (void *)&res->status, 0,
         res->wavefront_sizes ? sizeof(int) * 32 : sizeof(int));
  res->status = 0;
  res->wf_trace_len = 0;

  /* samples (mainPUMP.cu:249-250) */
  float *samples = (float *)malloc(sizeof(float) * N * ORC_DIM);
  if (pb->samples) memcpy(samples, pb->samples, sizeof(float) * N * ORC_DIM);
  else orc_halton_samples(N, samples, pb->init, pb->goal, pb->lo, pb->hi);

  /* pair BVPs and rn (mainPUMP.cu:261-304) */
  const long long npairs = (long long)N * (N - 1);
  float *copts = (float *)malloc(sizeof(float) * npairs);
  float *topts = (float *)malloc(sizeof(float) * npairs);
  orc_bvp_pairs(N, samples, 5, copts, topts);
  const long long rnIdx = (long long)((N - 1) * (N) * (float)0.05);
  const float rn = orc_select_kth(npairs, copts, rnIdx);
  res->rn = rn;

  /* edges (mainPUMP.cu:313-346) */
  const long long E = orc_build_edges(N, copts, topts, rn, NULL, NULL, NULL, NULL);
  res->numEdges = E;
  int *src = (int *)malloc(sizeof(int) * (E + 1)), *dst = (int *)malloc(sizeof(int) * (E + 1));
  float *coptE = (float *)malloc(sizeof(float) * (E + 1));
  float *toptE = (float *)malloc(sizeof(float) * (E + 1));
  orc_build_edges(N, copts, topts, rn, src, dst, coptE, toptE);
  free(copts);
  free(topts);
  /* waypoints (mainPUMP.cu:327-346): numDisc per edge, or by edge length */
  long long *off = (long long *)malloc(sizeof(long long) * (E + 1));
  const long long nwp = orc_disc_offsets(E, src, dst, samples, pb->discLen, pb->discMin, numDisc, off);
  float *disc = (float *)malloc(sizeof(float) * (nwp + 1) * ORC_DIM);
  orc_discretize_edges_off(E, src, dst, samples, off, disc);
  float *h = (float *)malloc(sizeof(float) * N);
  orc_heuristic(N, samples, pb->goal, h);

  /* go-adjacency in (i, j asc) order and edge lookup (mainPUMP.cu:338, 379-392) */
  int *goStart = (int *)calloc(N + 1, sizeof(int));
  for (long long e = 0; e < E; ++e) goStart[src[e] + 1]++;
  for (int i = 0; i < N; ++i) goStart[i + 1] += goStart[i];
  /* edges are already sorted by (src, dst): edge e is the k-th go edge of src[e] */

  /* online (mainPUMP.cu:428-497) */
  uint8_t *isFreeS = (uint8_t *)malloc(N);
  orc_sample_free(N, samples, nobs, obs, isFreeS);
  uint8_t *isFreeE = (uint8_t *)malloc(E + 1);
  orc_free_edges_off(E, off, disc, nobs, obs, isFreeE);
  float *as = (float *)malloc(sizeof(float) * ((nwp * maxHS) * 3 + 1));
  float *bs = (float *)malloc(sizeof(float) * (nwp * maxHS + 1));
  int *cnt = (int *)calloc(nwp + 1, sizeof(int));
  orc_cache_halfspaces_off(E, off, disc, isFreeE, nobs, obs, maxHS, maxd2, as, bs, cnt);
  free(cnt);

  /* exploration state (mainPUMP.cu:623-681) */
  const int maxPathCount = (int)(2 * N * sqrt((double)N));
  int *Ptab = (int *)malloc(sizeof(int) * (size_t)N * N);
  int *Pcounts = (int *)calloc(N, sizeof(int));
  int *pathPrev = (int *)calloc(maxPathCount + 1, sizeof(int));
  int *pathNode = (int *)calloc(maxPathCount + 1, sizeof(int));
  float *pathCost = (float *)calloc(maxPathCount + 1, sizeof(float));
  float *pathTime = (float *)calloc(maxPathCount + 1, sizeof(float));
  float *pathCP = (float *)calloc(maxPathCount + 1, sizeof(float));
  float *d_pathTime = (float *)calloc(maxPathCount + 1, sizeof(float));
  float *d_pathCP = (float *)malloc(sizeof(float) * (maxPathCount + 1));
  int *G = (int *)malloc(sizeof(int) * numBuckets * (size_t)maxPathCount);
  int sizeG[2] = {0, 0};
  uint8_t *valid = (uint8_t *)malloc((size_t)P * (maxPathCount + 1));
  int *wfPrev = (int *)malloc(sizeof(int) * (maxPathCount + 2));
  int *wfNode = (int *)malloc(sizeof(int) * (maxPathCount + 2));
  int *wfEdge = (int *)malloc(sizeof(int) * (maxPathCount + 2));
  int *PnewCount = (int *)malloc(sizeof(int) * N);
  for (size_t i = 0; i < (size_t)N * N; ++i) Ptab[i] = -1;
  for (int i = 0; i < numBuckets * maxPathCount; ++i) G[i] = -1;
  memset(valid, 1, (size_t)P * (maxPathCount + 1));
  for (int i = 0; i <= maxPathCount; ++i) d_pathCP[i] = 1;

  /* PUMP.cu:10-35 */
  const float cpTarget = pb->cpTarget;
  const float dr = lambda * rn;
  const float cpMinSoln = cpTarget / pb->cpFactor;
  const float cpCutoff = cpTarget * pb->cpFactor;
  const int initIdx = 0, goalIdx = N - 1;
  int numPaths = 1, Gidx = 0;
  int goalCondition = 0, goalConditionNext = 0, emptyOpenSet = 0;
  Ptab[initIdx * N + 0] = 0;
  Pcounts[initIdx]++;
  pathPrev[0] = -2; pathNode[0] = initIdx; pathCost[0] = 0; pathCP[0] = 0; pathTime[0] = 0;
  sizeG[Gidx]++;
  G[0] = 0;
  float costThreshold = h[initIdx];
  const int maxItrs = 20;
  int itrs = 0, numConsidered = 0;
  int status = 0;

  while (itrs < maxItrs && !goalCondition && !emptyOpenSet) {
    ++itrs;
    if (goalConditionNext) goalCondition = 1;
    int numNew = 0;
    int overflow = 0;
    /* PUMP.cu:47-66 */
    for (int g = 0; g < sizeG[Gidx] && !overflow; ++g) {
      int prev = G[Gidx * maxPathCount + g];
      G[Gidx * maxPathCount + g] = -1;
      int nodePrev = pathNode[prev];
      for (int e = goStart[nodePrev]; e < goStart[nodePrev + 1]; ++e) {
        int nodeNext = dst[e];
        if (!isFreeE[e] || !isFreeS[nodeNext]) continue;
        wfPrev[numNew] = prev; wfNode[numNew] = nodeNext; wfEdge[numNew] = e;
        numNew++;
        if (numNew > maxPathCount) { overflow = 1; break; }
      }
    }
    if (overflow) { status = 1; break; }
    if (res->wavefront_sizes && itrs <= 32) res->wavefront_sizes[itrs - 1] = numNew;
    if (numNew == 0) break;
    if (numPaths + numNew >= maxPathCount) { status = 1; break; }
    if (res->wf_trace) {
      for (int i = 0; i < numNew && res->wf_trace_len + 2 <= res->wf_trace_cap; ++i) {
        res->wf_trace[res->wf_trace_len++] = wfPrev[i];
        res->wf_trace[res->wf_trace_len++] = wfEdge[i];
      }
    }
    sizeG[Gidx] = 0;
    numConsidered += numNew;

    /* PUMP.cu:94-160: device propagation reads the device copy of path times */
    orc_hsmc_propagate_off(numNew, off, wfEdge, wfPrev, numPaths, as, bs, d_pathTime, toptE, dt, maxHS,
                       pb->tmajor, pb->offsetMult, Pmc, valid, P, d_pathCP);
    for (int i = 0; i < numNew; ++i) pathCP[numPaths + i] = d_pathCP[numPaths + i];

    /* PUMP.cu:164-167 */
    for (int i = 0; i < numNew; ++i) {
      pathTime[numPaths + i] = pathTime[wfPrev[i]] + toptE[wfEdge[i]];
      pathCost[numPaths + i] = pathCost[wfPrev[i]] + coptE[wfEdge[i]];
    }
    /* PUMP.cu:171-185 */
    for (int i = 0; i < N; ++i) PnewCount[i] = 0;
    for (int i = 0; i < numNew; ++i) {
      int node = wfNode[i], pathIdx = numPaths + i;
      if (pathCP[pathIdx] > cpCutoff) { wfNode[i] = -1; continue; }
      Ptab[node * N + Pcounts[node] + PnewCount[node]] = pathIdx;
      PnewCount[node]++;
    }
    /* PUMP.cu:188-218 */
    for (int i = 0; i < numNew; ++i) {
      int node = wfNode[i];
      if (wfNode[i] == -1 || node == goalIdx) continue;
      int pathIdx = numPaths + i;
      for (int j = 0; j < Pcounts[node] + PnewCount[node]; ++j) {
        int cmp = Ptab[node * N + j];
        if (cmp == pathIdx) continue;
        if (pathCP[cmp] < epsCP + pathCP[pathIdx] && pathCost[cmp] < epsCost + pathCost[pathIdx]) {
          if (pathCP[cmp] + epsCP >= pathCP[pathIdx] &&
              pathCost[cmp] + epsCost >= pathCost[pathIdx] && pathIdx < cmp)
            continue;
          wfNode[i] = -1;
          break;
        }
      }
    }
    /* PUMP.cu:221-256 */
    int numValid = 0;
    for (int i = 0; i < numNew; ++i) {
      int node = wfNode[i], pathIdx = numPaths + i;
      if (wfNode[i] == -1 || wfNode[i] == 0) { wfNode[i] = -1; continue; }
      int st = numPaths + numValid;
      pathCP[st] = pathCP[pathIdx];
      pathTime[st] = pathTime[pathIdx];
      pathCost[st] = pathCost[pathIdx];
      memmove(&valid[(size_t)P * st], &valid[(size_t)P * pathIdx], (size_t)P);
      float dCost = (pathCost[st] + h[node] - costThreshold);
      dCost = dCost > (float)0 ? dCost : (float)0;
      int bucket = (((int)(dCost / dr)) + Gidx + 1) % numBuckets;
      G[bucket * maxPathCount + sizeG[bucket]] = st;
      sizeG[bucket]++;
      pathPrev[st] = wfPrev[i];
      pathNode[st] = wfNode[i];
      Ptab[node * N + Pcounts[node]] = st;
      Pcounts[node]++;
      wfNode[i] = -1;
      numValid++;
    }
    for (int i = 0; i < numValid; ++i) {
      d_pathCP[numPaths + i] = pathCP[numPaths + i];
      d_pathTime[numPaths + i] = pathTime[numPaths + i];
    }
    numPaths += numValid;
    /* PUMP.cu:259-282 */
    for (int i = 0; i < Pcounts[goalIdx]; ++i) {
      int pi = Ptab[goalIdx * N + i];
      if (pathCP[pi] <= cpMinSoln) { goalConditionNext = 1; goalCondition = 1; }
    }
    if (goalCondition) break;
    emptyOpenSet = 1;
    for (int b = 0; b < numBuckets; ++b) emptyOpenSet = emptyOpenSet && (sizeG[b] == 0);
    if (emptyOpenSet) break;
    Gidx = (Gidx + 1) % numBuckets;
    costThreshold += dr;
    if (numPaths >= maxPathCount) { status = 1; break; }
  }
  res->itrs = itrs;
  res->numPaths = numPaths;
  res->numConsidered = numConsidered;
  res->goalPathCount = Pcounts[goalIdx];
  res->success = 0;
  res->solnPathIdx = -1;
  res->numNodes = 0;
  res->pathLen = 0;

  /* solution search (PUMP.cu:349-405); the reference returns from PUMP()
   * without a solution when maxPathCount is hit. */
  const int Tcap = pb->T_table;
  float *splitPath = (float *)malloc(sizeof(float) * ORC_DIM * (Tcap + 2));
  float *xs = (float *)malloc(sizeof(float) * ORC_DIM * (maxItrs + 2));
  int *nodes = (int *)malloc(sizeof(int) * (maxItrs + 2));
  int pathNumSamples = 0, pathLength = 0;
  float solnPathCP = 0, solnPathCost = 0;
  int success = 0, solnPathIdx = -1;
  if (status == 0) {
    int gcount = Pcounts[goalIdx];
    cost_idx *gp = (cost_idx *)malloc(sizeof(cost_idx) * (gcount + 1));
    for (int i = 0; i < gcount; ++i) {
      int pi = Ptab[goalIdx * N + i];
      gp[i].cost = pathCost[pi];
      gp[i].idx = pi;
    }
    qsort(gp, gcount, sizeof(cost_idx), cmp_cost_idx);
    for (int k = 0; k < gcount; ++k) {
      solnPathIdx = gp[k].idx;
      pathNumSamples = build_xs(solnPathIdx, pathPrev, pathNode, samples, xs, nodes, maxItrs + 2);
      orc_find_optimal_path(dt, splitPath, Tcap, xs, pathNumSamples, &pathLength);
      if (pathLength < 0) { status = 2; break; }
      orc_mccp(splitPath, pathLength, pb->pmajor, pb->T_table, pb->offsetMult, nobs, obs, Pmc,
               &solnPathCP);
      solnPathCost = pathCost[solnPathIdx];
      if (solnPathCP < cpTarget) { success = 1; break; }
    }
    free(gp);
  }

  /* smoothing (PUMP.cu:406-545) */
  float lastCP = solnPathCP, lastCost = solnPathCost;
  int lastLen = pathLength;
  /* xsSmooth of PUMP.cu:411: zeros unless a smoothing iterate was computed */
  float *xsFinal = (float *)calloc((size_t)ORC_DIM * (pathNumSamples > 0 ? pathNumSamples : 1), sizeof(float));
  float *lastPath = (float *)malloc(sizeof(float) * ORC_DIM * (Tcap + 2));
  if (pathLength > 0) memcpy(lastPath, splitPath, sizeof(float) * ORC_DIM * pathLength);
  if (success && status == 0) {
    const int dtMult = 10;
    const int optCap = Tcap * dtMult;
    float *optPath = (float *)malloc(sizeof(float) * ORC_DIM * (optCap + 2));
    float xsOpt2[12];
    for (int d = 0; d < ORC_DIM; ++d) {
      xsOpt2[d] = xs[d];
      xsOpt2[ORC_DIM + d] = xs[(pathNumSamples - 1) * ORC_DIM + d];
    }
    int optLen = 0;
    orc_find_optimal_path(dt / dtMult, optPath, optCap, xsOpt2, 2, &optLen);
    if (optLen < 0) status = 2;
    float *splitT = (float *)calloc(pathNumSamples, sizeof(float));
    int *splitI = (int *)calloc(pathNumSamples, sizeof(int));
    float *xsOpt = (float *)malloc(sizeof(float) * ORC_DIM * pathNumSamples);
    float *xsSmooth = (float *)malloc(sizeof(float) * ORC_DIM * pathNumSamples);
    float *smoothPath = (float *)malloc(sizeof(float) * ORC_DIM * (Tcap + 2));
    if (status == 0) {
      for (int i = 0; i < pathNumSamples - 1; ++i)
        splitT[i + 1] = splitT[i] + orc_topt_bisection(&xs[i * ORC_DIM], &xs[(i + 1) * ORC_DIM], 2, NULL);
      for (int i = 0; i < pathNumSamples; ++i)
        splitI[i] = (int)((optLen - 1) * splitT[i] / splitT[pathNumSamples - 1]);
      for (int i = 0; i < pathNumSamples; ++i)
        for (int d = 0; d < ORC_DIM; ++d) xsOpt[i * ORC_DIM + d] = optPath[splitI[i] * ORC_DIM + d];
      const int maxSmoothItrs = 30;
      const float epsSmoothCP = (float)0.0002;
      float alpha = 1.0f, alphaU = 1.0f, alphaL = 0.0f;
      for (int it = 0; it < maxSmoothItrs; ++it) {
        for (int i = 0; i < pathNumSamples * ORC_DIM; ++i)
          xsSmooth[i] = (1 - alpha) * xs[i] + alpha * xsOpt[i];
        memcpy(xsFinal, xsSmooth, sizeof(float) * ORC_DIM * pathNumSamples);
        int sLen = 0;
        float sCost = 0;
        orc_find_optimal_path(dt, smoothPath, Tcap, xsSmooth, pathNumSamples, &sLen);
        if (sLen < 0) { status = 2; break; }
        for (int i = 0; i < pathNumSamples - 1; ++i) {
          float tau = orc_topt_bisection(&xsSmooth[i * ORC_DIM], &xsSmooth[(i + 1) * ORC_DIM], 2, NULL);
          sCost += orc_cost(tau, &xsSmooth[i * ORC_DIM], &xsSmooth[(i + 1) * ORC_DIM]);
        }
        float cp = 0;
        orc_mccp(smoothPath, sLen, pb->pmajor, pb->T_table, pb->offsetMult, nobs, obs, Pmc, &cp);
        if (cp < cpTarget) alphaL = alpha;
        if (cp >= cpTarget) alphaU = alpha;
        alpha = (alphaL + alphaU) / 2;
        int satisfies = cp < cpTarget;
        int closer = cp > lastCP;
        int eqLower = (cp == lastCP && sCost < lastCost);
        if (satisfies && (closer || eqLower)) {
          memcpy(lastPath, smoothPath, sizeof(float) * ORC_DIM * sLen);
          lastLen = sLen;
          lastCost = sCost;
          lastCP = cp;
        }
        if (fabsf(cpTarget - cp) < epsSmoothCP && cpTarget - cp > 0) break;
      }
    }
    free(optPath); free(splitT); free(splitI); free(xsOpt); free(xsSmooth); free(smoothPath);
  }
  res->success = success;
  res->solnPathIdx = solnPathIdx;
  res->solnCP = lastCP;
  res->solnCost = lastCost;
  res->pathLen = success ? lastLen : 0;
  if (success && res->path)
    memcpy(res->path, lastPath, sizeof(float) * ORC_DIM * (lastLen < res->path_cap ? lastLen : res->path_cap));
  if (solnPathIdx >= 0) {
    int n = build_xs(solnPathIdx, pathPrev, pathNode, samples, xs, nodes, maxItrs + 2);
    res->numNodes = n;
    if (res->nodes)
      for (int k = 0; k < n && k < res->nodes_cap; ++k) res->nodes[k] = nodes[k];
  }
  res->status = status;
  res->ctrlLen = 0;
  if (status != 1) /* with maxPathCount hit the reference returns before this */
    res->ctrlLen = orc_control_path(xsFinal, pathNumSamples, res->ctrl_path, res->ctrl_path ? res->ctrl_cap : 0);
  free(xsFinal);

  free(samples); free(src); free(dst); free(coptE); free(toptE); free(disc); free(h); free(off);
  free(goStart); free(isFreeS); free(isFreeE); free(as); free(bs);
  free(Ptab); free(Pcounts); free(pathPrev); free(pathNode); free(pathCost); free(pathTime);
  free(pathCP); free(d_pathTime); free(d_pathCP); free(G); free(valid); free(wfPrev);
  free(wfNode); free(wfEdge); free(PnewCount); free(splitPath); free(xs); free(nodes);
  free(lastPath);
  return status;
}

/* ======================================================================
 * Path refinement objective and adjoint (binary64 checker)
 * ==================================================================== */
typedef struct { double A0, A1, A2, A3, A4; } quartic64;

static quartic64 quartic_of(const double *x0, const double *x1) {
  const double g = (double)ORC_G;
  quartic64 q;
  double dd = 0, ds = 0;
  for (int d = 0; d < 3; ++d) {
    const double D = x1[d] - x0[d], S = x0[3 + d] + x1[3 + d];
    dd += D * D;
    ds += D * S;
  }
  double v00 = 0, v01 = 0, v11 = 0;
  for (int d = 3; d < 6; ++d) {
    v00 += x0[d] * x0[d];
    v01 += x0[d] * x1[d];
    v11 += x1[d] * x1[d];
  }
  q.A0 = 12 * dd;
  q.A1 = -12 * ds;
  q.A2 = 4 * (v00 + v01 + v11);
  q.A3 = 2 * g * (x0[5] - x1[5]);
  q.A4 = 1 + g * g;
  return q;
}
static double q_cost(const quartic64 *q, double t) {
  return q->A0 / (t * t * t) + q->A1 / (t * t) + q->A2 / t + q->A3 + q->A4 * t;
}
static double q_Q(const quartic64 *q, double t) {
  return q->A4 * t * t * t * t - q->A2 * t * t - 2 * q->A1 * t - 3 * q->A0;
}

double orc_tau_exact(const double *x0, const double *x1, double tmax, int *clamped) {
  /* minima of c are the upward zero crossings of Q = t^4 c'(t); bracket them
   * on a fine grid from Q(0) = -3 A0, bisect to the last bit, compare costs
   * (and tmax when Q(tmax) < 0) */
  const quartic64 q = quartic_of(x0, x1);
  const int G = 4096;
  double best_t = tmax, best_c = INFINITY;
  int have = 0;
  double ta = 0, qa = q_Q(&q, 0);
  for (int k = 1; k <= G; ++k) {
    const double tb = tmax * k / G, qb = q_Q(&q, tb);
    if (qa < 0 && qb >= 0) {
      double lo = ta, hi = tb;
      for (int it = 0; it < 200 && hi - lo > 0; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (q_Q(&q, mid) < 0) lo = mid; else hi = mid;
      }
      const double t = fabs(q_Q(&q, lo)) < fabs(q_Q(&q, hi)) ? lo : hi;
      if (t > 0) {
        const double c = q_cost(&q, t);
        if (!have || c < best_c) { best_c = c; best_t = t; have = 1; }
      }
    }
    ta = tb;
    qa = qb;
  }
  int cl = 0;
  if (qa < 0) {
    const double c = q_cost(&q, tmax);
    if (!have || c < best_c) { best_c = c; best_t = tmax; cl = 1; have = 1; }
  }
  if (clamped) *clamped = cl;
  return best_t;
}

void orc_position_variance(int T, double *var) {
  double *cov = (double *)malloc(sizeof(double) * 3 * (size_t)T);
  orc_particle_cov(T, cov);
  for (int t = 0; t < T; ++t) var[t] = cov[3 * t];
  free(cov);
}

/* dA/dx for the 12 inputs (x0 then x1) */
static void quartic_grad(const double *x0, const double *x1, double dA[4][12]) {
  const double g = (double)ORC_G;
  memset(dA, 0, sizeof(double) * 48);
  for (int d = 0; d < 3; ++d) {
    const double D = x1[d] - x0[d], S = x0[3 + d] + x1[3 + d];
    dA[0][d] = -24 * D;
    dA[0][6 + d] = 24 * D;
    dA[1][d] = 12 * S;
    dA[1][6 + d] = -12 * S;
    dA[1][3 + d] = -12 * D;
    dA[1][9 + d] = -12 * D;
    dA[2][3 + d] = 4 * (2 * x0[3 + d] + x1[3 + d]);
    dA[2][9 + d] = 4 * (2 * x1[3 + d] + x0[3 + d]);
  }
  dA[3][5] = 2 * g;
  dA[3][11] = -2 * g;
}

static void hermite(double s, double h[4], double gd[3]) {
  const double s2 = s * s, s3 = s2 * s;
  h[0] = 2 * s3 - 3 * s2 + 1;  /* h00: p0 */
  h[1] = -2 * s3 + 3 * s2;     /* h01: p1 */
  h[2] = s3 - 2 * s2 + s;      /* h10: tau v0 */
  h[3] = s3 - s2;              /* h11: tau v1 */
  gd[0] = 6 * s2 - 6 * s;      /* (p0 - p1) / tau */
  gd[1] = 3 * s2 - 4 * s + 1;  /* v0 */
  gd[2] = 3 * s2 - 2 * s;      /* v1 */
}

static void variance_at(const orc_refine_args *a, double T, double *V, double *dVdT) {
  const double u = T / a->dt;
  if (!(u < (double)(a->T_rows - 1))) {
    *V = a->posVar[a->T_rows - 1];
    *dVdT = 0;
    return;
  }
  const int j = (int)floor(u);
  const double f = u - j;
  *V = a->posVar[j] + f * (a->posVar[j + 1] - a->posVar[j]);
  *dVdT = (a->posVar[j + 1] - a->posVar[j]) / a->dt;
}

#define REFINE_EPS_V 1e-12  /* added to v.v */
#define REFINE_EPS_D 1e-12  /* added to a.a under the square root */

/* One waypoint's bound terms over all boxes; with grads, adds dB/dp, dB/dv, dB/dS. */
static double waypoint_terms(const orc_refine_args *a, const double *p, const double *v, double S,
                             double *gp, double *gv, double *gS) {
  double B = 0;
  const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + REFINE_EPS_V;
  for (int o = 0; o < a->numObs; ++o) {
    const float *box = &a->obstacles[o * 12];
    double r[3];
    int inside[3];
    for (int d = 0; d < 3; ++d) {
      const double lo = box[d], hi = box[6 + d];
      const double q = p[d] < lo ? lo : (p[d] > hi ? hi : p[d]);
      inside[d] = (p[d] >= lo && p[d] <= hi);
      r[d] = q - p[d];
    }
    const double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    const double beta = rv / vv;
    double av[3], aa = 0;
    for (int d = 0; d < 3; ++d) { av[d] = r[d] - beta * v[d]; aa += av[d] * av[d]; }
    const double dist = sqrt(aa + REFINE_EPS_D);
    const double z = dist / S;
    B += 0.5 * erfc(z / sqrt(2.0));
    if (gp) {
      const double zb = -exp(-0.5 * z * z) * 0.39894228040143267794;  /* dPhi(-z)/dz = -phi(z) */
      const double db = zb / S;
      *gS += -zb * z / S;
      double abar[3], rbar[3], vbar[3];
      for (int d = 0; d < 3; ++d) abar[d] = db * av[d] / dist;
      const double betabar = -(abar[0] * v[0] + abar[1] * v[1] + abar[2] * v[2]);
      for (int d = 0; d < 3; ++d) {
        rbar[d] = abar[d] + betabar * v[d] / vv;
        vbar[d] = -beta * abar[d] + betabar * r[d] / vv;
      }
      const double vvbar = -betabar * beta / vv;
      for (int d = 0; d < 3; ++d) {
        vbar[d] += 2 * vvbar * v[d];
        gv[d] += vbar[d];
        if (!inside[d]) gp[d] += -rbar[d];
      }
    }
  }
  return B;
}

static double refine_eval(const orc_refine_args *a, const double *X, int n, double lambda,
                          double *cost_out, double *bound_out, double *grad) {
  const int nseg = n - 1;
  double *tau = (double *)malloc(sizeof(double) * (nseg > 0 ? nseg : 1));
  int *clamped = (int *)malloc(sizeof(int) * (nseg > 0 ? nseg : 1));
  double *taubar = (double *)calloc(nseg > 0 ? nseg : 1, sizeof(double));
  double *Tbar = (double *)calloc(nseg > 0 ? nseg : 1, sizeof(double));
  double C = 0, B = 0;
  if (grad) memset(grad, 0, sizeof(double) * 6 * (size_t)n);
  for (int i = 0; i < nseg; ++i) {
    const double *x0 = &X[6 * i], *x1 = &X[6 * (i + 1)];
    tau[i] = orc_tau_exact(x0, x1, a->tmax, &clamped[i]);
    const quartic64 q = quartic_of(x0, x1);
    C += q_cost(&q, tau[i]);
    if (grad) {
      double dA[4][12];
      quartic_grad(x0, x1, dA);
      const double t = tau[i];
      for (int m = 0; m < 12; ++m) {
        const double dc = dA[0][m] / (t * t * t) + dA[1][m] / (t * t) + dA[2][m] / t + dA[3][m];
        grad[6 * i + m] += dc;
      }
    }
  }
  double Tstart = 0;
  for (int i = 0; i < nseg; ++i) {
    const double *x0 = &X[6 * i], *x1 = &X[6 * (i + 1)];
    const double t = tau[i];
    for (int k = 0; k < a->W; ++k) {
      const double s = (double)k / a->W;
      double h[4], gd[3], p[3], v[3];
      hermite(s, h, gd);
      for (int d = 0; d < 3; ++d) {
        p[d] = h[0] * x0[d] + h[1] * x1[d] + t * (h[2] * x0[3 + d] + h[3] * x1[3 + d]);
        v[d] = gd[0] * (x0[d] - x1[d]) / t + gd[1] * x0[3 + d] + gd[2] * x1[3 + d];
      }
      const double T = Tstart + s * t;
      double V, dVdT;
      variance_at(a, T, &V, &dVdT);
      const double S = a->offsetMult * sqrt(V + a->sigmaFloor * a->sigmaFloor);
      double gp[3] = {0, 0, 0}, gv[3] = {0, 0, 0}, gS = 0;
      B += waypoint_terms(a, p, v, S, grad ? gp : NULL, gv, &gS);
      if (grad) {
        for (int d = 0; d < 3; ++d) {
          gp[d] *= lambda;
          gv[d] *= lambda;
        }
        gS *= lambda;
        const double Vbar = gS * a->offsetMult * a->offsetMult / (2 * S);
        const double Tb = Vbar * dVdT;
        double tb = s * Tb;
        Tbar[i] += Tb;
        for (int d = 0; d < 3; ++d) {
          grad[6 * i + d] += h[0] * gp[d] + gd[0] / t * gv[d];
          grad[6 * (i + 1) + d] += h[1] * gp[d] - gd[0] / t * gv[d];
          grad[6 * i + 3 + d] += t * h[2] * gp[d] + gd[1] * gv[d];
          grad[6 * (i + 1) + 3 + d] += t * h[3] * gp[d] + gd[2] * gv[d];
          tb += (h[2] * x0[3 + d] + h[3] * x1[3 + d]) * gp[d];
          tb += -gd[0] * (x0[d] - x1[d]) / (t * t) * gv[d];
        }
        taubar[i] += tb;
      }
    }
    Tstart += t;
  }
  if (grad) {
    /* T_i = tau_0 + .. + tau_{i-1}: each tau_j collects Tbar of later segments */
    double suffix = 0;
    for (int i = nseg - 1; i >= 0; --i) {
      taubar[i] += suffix;
      suffix += Tbar[i];
    }
    for (int i = 0; i < nseg; ++i) {
      if (clamped[i]) continue;  /* tau = tmax does not move */
      const double *x0 = &X[6 * i], *x1 = &X[6 * (i + 1)];
      const quartic64 q = quartic_of(x0, x1);
      double dA[4][12];
      quartic_grad(x0, x1, dA);
      const double t = tau[i], t2 = t * t, t3 = t2 * t, t4 = t3 * t, t5 = t4 * t;
      /* F = c'(t) = -3 A0/t^4 - 2 A1/t^3 - A2/t^2 + A4 = 0, dtau/dx = -F_x / F_t */
      const double Ft = 12 * q.A0 / t5 + 6 * q.A1 / t4 + 2 * q.A2 / t3;
      for (int m = 0; m < 12; ++m) {
        const double Fx = -3 * dA[0][m] / t4 - 2 * dA[1][m] / t3 - dA[2][m] / t2;
        grad[6 * i + m] += taubar[i] * (-Fx / Ft);
      }
    }
    for (int d = 0; d < 6; ++d) {
      grad[d] = 0;
      grad[6 * (n - 1) + d] = 0;
    }
  }
  if (cost_out) *cost_out = C;
  if (bound_out) *bound_out = B;
  free(tau); free(clamped); free(taubar); free(Tbar);
  return C + lambda * B;
}

double orc_refine_objective(const orc_refine_args *a, const double *nodes, int n, double lambda,
                            double *cost, double *bound) {
  return refine_eval(a, nodes, n, lambda, cost, bound, NULL);
}

double orc_refine_grad(const orc_refine_args *a, const double *nodes, int n, double lambda,
                       double *grad) {
  return refine_eval(a, nodes, n, lambda, NULL, NULL, grad);
}
