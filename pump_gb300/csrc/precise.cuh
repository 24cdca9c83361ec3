// Closed-form optimal time of the 2pBVP (precision mode), shared by the
// pair kernels and the path-refinement adjoint.  Include only from
// translation units compiled with multiply-add contraction.
//
// The global minimiser of the reference's cost (2pBVP.cu:97-107) in closed
// form.  Written out, the cost is
//   c(t) = A0/t^3 + A1/t^2 + A2/t + A3 + A4 t with
//   A0 = 12|p1-p0|^2, A1 = -12 (p1-p0).(v0+v1), A2 = 4(|v0|^2+v0.v1+|v1|^2),
//   A3 = 2g(v0z-v1z), A4 = 1+g^2,
// so c'(t) = 0 is the quartic Q(t) = A4 t^4 - A2 t^2 - 2 A1 t - 3 A0 = 0.
// The roots of Q are bracketed in binary32 (pieces split at the inflection
// point and the real roots of Q'), each candidate minimum is refined with one
// binary64 Newton step, and the candidates (and tmax) are compared by their
// binary64 cost.  Translation units including this header are compiled
// with multiply-add contraction (the mode is not bound to the reference's
// roundings): the binary64 Horner evaluations issue as DFMA, half the
// FP64-pipe instructions of separate multiply and add.
#pragma once
#include <math.h>

#include "common.cuh"

namespace pump {
namespace {

struct Quartic {
  double A0, A1, A2, A3, A4;
  __device__ double Q(double t) const { return ((A4 * t * t - A2) * t - 2.0 * A1) * t - 3.0 * A0; }
  __device__ double dQ(double t) const { return (4.0 * A4 * t * t - 2.0 * A2) * t - 2.0 * A1; }
  // 1/t from the hardware reciprocal estimate (rel. error < 2^-20) refined
  // by two binary64 Newton steps (~1e-16, below the float the cost becomes)
  __device__ double cost(double t) const {
    const double y0 = rcp_approx(t);
    const double y1 = fma(y0, fma(-t, y0, 1.0), y0);
    const double r = fma(y1, fma(-t, y1, 1.0), y1);
    return (((A0 * r + A1) * r + A2) * r + A3) + A4 * t;
  }
  __device__ static double rcp_approx(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return y;
  }
};

// The same polynomials in binary32 for the bracketing phase.
struct QuarticF {
  float A0, A1, A2, A4;  // binary32 copies for the bracketing phase
  __device__ float Q(float t) const { return ((A4 * t * t - A2) * t - 2.0f * A1) * t - 3.0f * A0; }
  __device__ float dQ(float t) const { return (4.0f * A4 * t * t - 2.0f * A2) * t - 2.0f * A1; }
  __device__ float d2Q(float t) const { return 12.0f * A4 * t * t - 2.0f * A2; }
};

__device__ __forceinline__ Quartic make_quartic(const float *x0, const float *x1) {
  const double g = (double)PUMP_G;
  const double dx = (double)x1[0] - x0[0], dy = (double)x1[1] - x0[1], dz = (double)x1[2] - x0[2];
  const double sx = (double)x0[3] + x1[3], sy = (double)x0[4] + x1[4], sz = (double)x0[5] + x1[5];
  Quartic q;
  q.A0 = 12.0 * (dx * dx + dy * dy + dz * dz);
  q.A1 = -12.0 * (dx * sx + dy * sy + dz * sz);
  const double v00 = (double)x0[3] * x0[3] + (double)x0[4] * x0[4] + (double)x0[5] * x0[5];
  const double v11 = (double)x1[3] * x1[3] + (double)x1[4] * x1[4] + (double)x1[5] * x1[5];
  const double v01 = (double)x0[3] * x1[3] + (double)x0[4] * x1[4] + (double)x0[5] * x1[5];
  q.A2 = 4.0 * (v00 + v01 + v11);
  q.A3 = 2.0 * g * ((double)x0[5] - x1[5]);
  q.A4 = 1.0 + g * g;
  return q;
}

// Root of a monotone function on [a, b] (sign change given) with fixed
// convexity: Newton started at the end where the function and its curvature
// have the same sign converges monotonically.  Binary32.
template <int Deriv>
__device__ float newton_f(const QuarticF &q, float a, float b, bool from_b) {
  float x = from_b ? b : a;
  for (int it = 0; it < 40; ++it) {
    const float f = Deriv ? q.dQ(x) : q.Q(x);
    const float df = Deriv ? q.d2Q(x) : q.dQ(x);
    if (f == 0.0f || df == 0.0f) break;
    float xn = x - __fdividef(f, df);  // approximate quotient: a Newton step needs no rounding guarantee
    if (!(xn >= a && xn <= b)) xn = 0.5f * (a + b);
    if (fabsf(xn - x) <= 2e-7f * fabsf(xn)) { x = xn; break; }
    x = xn;
  }
  return x;
}

// Binary32 analysis of the stationarity quartic: the local minima of the cost
// inside (0, tmax) (at most two) and whether the cost still decreases at
// tmax.  (0, tmax] is split at the inflection point tc of Q (Q'' = 0) and at
// the real roots of Q', so on every piece Q is monotone with fixed convexity
// and each upward sign change of Q is found by monotone Newton.
__device__ int minima_f32(const QuarticF &q, float tmax, float cand[2], bool *tmax_cand) {
  float bp[5];
  int nb = 0;
  bp[nb++] = 0.0f;
  const float tc = sqrtf(q.A2 / (6.0f * q.A4));
  const float d0 = -2.0f * q.A1;  // Q'(0)
  if (tc > 0.0f && tc < tmax) {
    const float dc = q.dQ(tc);
    if (d0 > 0.0f && dc < 0.0f) bp[nb++] = newton_f<1>(q, 0.0f, tc, false);
    bp[nb++] = tc;
    if (dc < 0.0f && q.dQ(tmax) > 0.0f) bp[nb++] = newton_f<1>(q, tc, tmax, true);
  } else if (tc <= 0.0f) {
    if (d0 < 0.0f && q.dQ(tmax) > 0.0f) bp[nb++] = newton_f<1>(q, 0.0f, tmax, true);
  } else if (d0 > 0.0f && q.dQ(tmax) < 0.0f) {
    bp[nb++] = newton_f<1>(q, 0.0f, tmax, false);
  }
  bp[nb++] = tmax;
  int nc = 0;
  float qa = -3.0f * q.A0;  // Q(0)
  for (int k = 0; k + 1 < nb; ++k) {
    const float a = bp[k], b = bp[k + 1];
    const float qb = q.Q(b);
    if (qa < 0.0f && qb > 0.0f && nc < 2) cand[nc++] = newton_f<0>(q, a, b, a >= tc);
    qa = qb;
  }
  *tmax_cand = qa < 0.0f;
  return nc;
}

// Global minimiser of the cost on (0, tmax]: candidates from the binary32
// analysis, each refined by one binary64 Newton step on Q (quadratic
// convergence takes a ~1e-6 relative root to ~1e-12) and compared by their
// binary64 cost.  In the common case of one candidate the binary64 work is the
// same straight-line sequence for every pair, so the FP64 pipe runs with full
// warps.
__device__ __forceinline__ QuarticF make_quartic_f32(const float *x0, const float *x1) {
  const float g = PUMP_G;
  const float dx = x1[0] - x0[0], dy = x1[1] - x0[1], dz = x1[2] - x0[2];
  const float sx = x0[3] + x1[3], sy = x0[4] + x1[4], sz = x0[5] + x1[5];
  QuarticF q;
  q.A0 = 12.0f * fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  q.A1 = -12.0f * fmaf(dx, sx, fmaf(dy, sy, dz * sz));
  q.A2 = 4.0f * (fmaf(x0[3], x0[3] + x1[3], fmaf(x0[4], x0[4] + x1[4], x0[5] * (x0[5] + x1[5]))) +
                 fmaf(x1[3], x1[3], fmaf(x1[4], x1[4], x1[5] * x1[5])));
  q.A4 = fmaf(g, g, 1.0f);
  return q;
}

// One binary64 Newton step on Q from a binary32 root estimate (the
// correction is ~1e-6 of x, so the 2^-20 reciprocal estimate of Q' leaves
// ~1e-12 relative error).
__device__ __forceinline__ double refine(const Quartic &q, double x) {
  const double f = q.Q(x), df = q.dQ(x);
  const double xn = fma(-f, Quartic::rcp_approx(df), x);
  return fabs(xn - x) <= 1e-3 * x ? xn : x;  // keep the estimate if Q' is tiny
}

// Global minimiser on (0, tmax] in binary64 (*t) and its binary64 cost (*c).
__device__ __forceinline__ void precise_tau(const float *x0, const float *x1, float tmax,
                                            double *t_out, double *c_out) {
  const QuarticF qf = make_quartic_f32(x0, x1);
  float cand[2];
  bool tmax_cand = false;
  const int nc = minima_f32(qf, tmax, cand, &tmax_cand);
  const Quartic q = make_quartic(x0, x1);
  // primary candidate, evaluated by every lane with the same instructions
  const bool primary_root = nc > 0;
  const double tm = (double)tmax;
  const double xr = refine(q, (double)(primary_root ? cand[0] : tmax));
  double best_t = primary_root ? xr : tm;
  double best_c = q.cost(best_t);
  // rare: a second interior minimum, or the cost still falling at tmax
  if (nc > 1) {
    const double t2 = refine(q, (double)cand[1]);
    const double c2 = q.cost(t2);
    if (c2 < best_c) { best_c = c2; best_t = t2; }
  }
  if (primary_root && tmax_cand) {
    const double c3 = q.cost((double)tmax);
    if (c3 < best_c) { best_c = c3; best_t = (double)tmax; }
  }
  *t_out = best_t;
  *c_out = best_c;
}

}  // namespace
}  // namespace pump
