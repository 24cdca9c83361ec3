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
// The coefficients are assembled exactly enough in float-float (pairs of
// binary32, ~46-bit significands) on the FP32 pipe; the roots of Q are
// bracketed in binary32 (pieces split at the inflection point and the real
// roots of Q'); each candidate minimum is refined with one Newton step whose
// residual Q(x) is evaluated in binary64 (the FP64 pipe, ~1/64 of the FP32
// rate on this GPU, does only Q(x) and the cost); the candidates (and tmax)
// are compared by their binary64 cost.  Translation units including this header are compiled
// with multiply-add contraction (the mode is not bound to the reference's
// roundings): the binary64 Horner evaluations issue as DFMA, half the
// FP64-pipe instructions of separate multiply and add.
#pragma once
#include <math.h>

#include "common.cuh"

namespace pump {
namespace {

// ---------------------------------------------------------------------------
// Float-float arithmetic (Dekker / Knuth error-free transformations): a value
// is h + l with |l| <= ulp(h) / 2.  No multiply-add is left to the compiler:
// products use explicit fmaf, sums have no products to contract.
struct FF {
  float h, l;
};
__device__ __forceinline__ FF two_sum(float a, float b) {
  const float s = a + b, bp = s - a;
  return {s, (a - (s - bp)) + (b - bp)};
}
__device__ __forceinline__ FF fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ FF two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ FF ff_add(FF x, FF y) {
  const FF s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, s.l + (x.l + y.l));
}
__device__ __forceinline__ FF ff_mul(FF x, FF y) {
  const FF p = two_prod(x.h, y.h);
  return fast_two_sum(p.h, p.l + fmaf(x.h, y.l, x.l * y.h));
}
__device__ __forceinline__ FF ff_mulf(FF x, float c) {
  const FF p = two_prod(x.h, c);
  return fast_two_sum(p.h, fmaf(x.l, c, p.l));
}

// Exact binary32 -> binary64 with integer operations (the FP64 pipe is the
// scarce resource): rebias the exponent, widen the significand.  Binary32
// subnormals become zero; infinities and NaNs stay what they are.
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned long long frac = (unsigned long long)(u & 0x7fffffu) << 29;
  const unsigned long long ex = e == 0xffu ? 0x7ffull : (unsigned long long)(e + 896u);
  const unsigned long long bits = e == 0 ? sign : (sign | (ex << 52) | frac);
  return __longlong_as_double((long long)bits);
}

// Binary64 -> binary32, round to nearest even, with integer operations for
// results in binary32's normal range; anything else takes the conversion
// instruction.
__device__ __forceinline__ float d2f_rn(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const int e = (int)((u >> 52) & 0x7ff) - 896;
  if (e <= 0 || e >= 255) return (float)d;
  unsigned mf = (unsigned)((u >> 29) & 0x7fffffu);
  const unsigned rem = (unsigned)(u & 0x1fffffffu);
  mf += (rem > 0x10000000u) | ((rem == 0x10000000u) & (mf & 1u));
  // a carry out of the significand moves into the exponent field (to
  // infinity only if the value rounds past the largest binary32)
  const unsigned bits = ((unsigned)(u >> 32) & 0x80000000u) + (((unsigned)e << 23) + mf);
  return __uint_as_float(bits);
}

// The cost's binary64 polynomials, with every expression written out in
// explicit fma() so that the all-pairs kernel and the explicit-pair kernel
// produce identical bits for the same pair.
struct Quartic {
  double A0, A1, A2, A3, A4;
  double A0x3, A1x2;  // 3 A0 and 2 A1 for Q
  __device__ double Q(double t) const {
    return fma(fma(fma(A4 * t, t, -A2), t, -A1x2), t, -A0x3);
  }
  // 1/t from the hardware reciprocal estimate refined by one binary64 Newton
  // step (relative error ~1e-14, far below the binary32 the cost becomes)
  __device__ double cost(double t) const {
    const double y0 = rcp_approx(t);
    const double r = fma(y0, fma(-t, y0, 1.0), y0);
    return fma(A4, t, fma(fma(fma(A0, r, A1), r, A2), r, A3));
  }
  __device__ static double rcp_approx(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return y;
  }
};

// A sample with |v|^2 in float-float: prepared once per launch for the
// all-pairs kernel, in registers for explicit pairs.
struct __align__(16) SampleF {
  float p[3], v[3];
  FF vv;
};

__device__ __forceinline__ SampleF to_sample_f(const float *x) {
  SampleF s;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    s.p[d] = x[d];
    s.v[d] = x[3 + d];
  }
  s.vv = ff_add(ff_add(two_prod(x[3], x[3]), two_prod(x[4], x[4])), two_prod(x[5], x[5]));
  return s;
}

__device__ __forceinline__ double ff2d(FF x) { return f2d_exact(x.h) + f2d_exact(x.l); }

// The same polynomials in binary32 for the bracketing phase.
struct QuarticF {
  float A0, A1, A2, A4;  // binary32 copies for the bracketing phase
  __device__ float Q(float t) const { return ((A4 * t * t - A2) * t - 2.0f * A1) * t - 3.0f * A0; }
  __device__ float dQ(float t) const { return (4.0f * A4 * t * t - 2.0f * A2) * t - 2.0f * A1; }
  __device__ float d2Q(float t) const { return 12.0f * A4 * t * t - 2.0f * A2; }
};


// Root of a monotone function on [a, b] (sign change given) with fixed
// convexity: Newton started at x0, on the side where the function and its
// curvature have the same sign, converges monotonically.  Binary32.
template <int Deriv>
__device__ float newton_f(const QuarticF &q, float a, float b, float x0) {
  float x = x0;
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
__device__ __forceinline__ int minima_f32(const QuarticF &q, float tmax, float *cand0,
                                          float *cand1, bool *tmax_cand) {
  int nc = 0;
  float a = 0.0f, qa = -3.0f * q.A0;  // left end of the current piece and Q there
  const float tc = sqrtf(q.A2 / (6.0f * q.A4));
  // Fujiwara's bound on the roots of the monic Q / A4 and Q' / (4 A4)
  // (2 max |a_k / a_n|^(1 / (n - k)), the constant term halved), with 1 %
  // margin: right-end Newton starts there instead of at tmax when that is
  // closer, on the same side of the root (checked), so it converges from the
  // same side in about half the steps.
  const float rA4 = 1.0f / q.A4;
  const float bq = 2.02f * fmaxf(sqrtf(fabsf(q.A2 * rA4)),
                                 fmaxf(cbrtf(fabsf(2.0f * q.A1 * rA4)),
                                       sqrtf(sqrtf(fabsf(1.5f * q.A0 * rA4)))));
  const float bd = 2.02f * fmaxf(sqrtf(fabsf(0.5f * q.A2 * rA4)), cbrtf(fabsf(0.25f * q.A1 * rA4)));
  auto start_q = [&](float b) {
    const float x = fminf(b, bq);
    return q.Q(x) >= 0.0f ? x : b;
  };
  auto start_d = [&](float b) {
    const float x = fminf(b, bd);
    return q.dQ(x) >= 0.0f ? x : b;
  };
  // close the piece [a, b]: an upward sign change of Q is a minimum of the cost
  auto piece = [&](float b) {
    const float qb = q.Q(b);
    if (qa < 0.0f && qb > 0.0f && nc < 2) {
      const float r = newton_f<0>(q, a, b, a >= tc ? start_q(b) : a);
      if (nc == 0) *cand0 = r; else *cand1 = r;
      ++nc;
    }
    qa = qb;
    a = b;
  };
  const float d0 = -2.0f * q.A1;  // Q'(0)
  if (tc > 0.0f && tc < tmax) {
    const float dc = q.dQ(tc);
    if (d0 > 0.0f && dc < 0.0f) piece(newton_f<1>(q, 0.0f, tc, 0.0f));
    piece(tc);
    if (dc < 0.0f && q.dQ(tmax) > 0.0f) piece(newton_f<1>(q, tc, tmax, start_d(tmax)));
  } else if (tc <= 0.0f) {
    if (d0 < 0.0f && q.dQ(tmax) > 0.0f) piece(newton_f<1>(q, 0.0f, tmax, start_d(tmax)));
  } else if (d0 > 0.0f && q.dQ(tmax) < 0.0f) {
    piece(newton_f<1>(q, 0.0f, tmax, 0.0f));
  }
  piece(tmax);
  *tmax_cand = qa < 0.0f;
  return nc;
}

// Coefficients of one pair: A0 = 12|D|^2, A1 = -12 D.S, A2 = 4(|v0|^2 +
// v0.v1 + |v1|^2), A3 = 2g(v0z - v1z) with D = p1 - p0, S = v0 + v1, in
// float-float (differences and products exact, sums to ~2^-46), then the
// binary32 copies (the high parts) for bracketing and binary64 values (hi +
// lo, one addition each) for the refinement and the cost.
struct PairQuartic {
  QuarticF f;
  Quartic q;
};

__device__ __forceinline__ PairQuartic make_pair_quartic(const SampleF &a, const SampleF &b) {
  FF D[3], S[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    D[d] = two_sum(b.p[d], -a.p[d]);
    S[d] = two_sum(a.v[d], b.v[d]);
  }
  const FF dd = ff_add(ff_add(ff_mul(D[0], D[0]), ff_mul(D[1], D[1])), ff_mul(D[2], D[2]));
  const FF ds = ff_add(ff_add(ff_mul(D[0], S[0]), ff_mul(D[1], S[1])), ff_mul(D[2], S[2]));
  const FF v01 = ff_add(ff_add(two_prod(a.v[0], b.v[0]), two_prod(a.v[1], b.v[1])),
                        two_prod(a.v[2], b.v[2]));
  const FF A0 = ff_mulf(dd, 12.0f), A0x3 = ff_mulf(dd, 36.0f);
  const FF A1 = ff_mulf(ds, -12.0f), A1x2 = ff_mulf(ds, -24.0f);
  const FF A2s = ff_add(ff_add(a.vv, v01), b.vv);
  const FF A3 = ff_mulf(two_sum(a.v[2], -b.v[2]), 2.0f * PUMP_G);
  const double g = (double)PUMP_G;
  PairQuartic r;
  r.f.A0 = A0.h;
  r.f.A1 = A1.h;
  r.f.A2 = 4.0f * A2s.h;
  r.f.A4 = fmaf(PUMP_G, PUMP_G, 1.0f);
  r.q.A0 = ff2d(A0);
  r.q.A1 = ff2d(A1);
  r.q.A2 = 4.0 * ff2d(A2s);
  r.q.A3 = ff2d(A3);
  r.q.A4 = 1.0 + g * g;
  r.q.A0x3 = ff2d(A0x3);
  r.q.A1x2 = ff2d(A1x2);
  return r;
}

// One Newton step from a binary32 root estimate x: the residual Q(x) in
// binary64, the slope and the step size test in binary32 (the step is ~1e-6
// of x, so a binary32 slope leaves ~1e-13 relative error).  Keeps x when the
// step is not small (a tiny slope).
__device__ __forceinline__ double refine(const PairQuartic &pq, float x) {
  const double xd = f2d_exact(x);
  const double f = pq.q.Q(xd);
  const float r = __fdividef(1.0f, pq.f.dQ(x));
  const bool ok = fabsf(d2f_rn(f) * r) <= 1e-3f * x;
  return ok ? fma(-f, f2d_exact(r), xd) : xd;
}

// Global minimiser of the cost on (0, tmax]: candidates from the binary32
// analysis, each refined by one Newton step (quadratic convergence takes a
// ~1e-6 relative root to ~1e-12) and compared by their binary64 cost.  In
// the common case of one candidate the binary64 work is the same
// straight-line sequence for every pair, so the FP64 pipe runs with full
// warps.
// Global minimiser on (0, tmax] in binary64 (*t) and its binary64 cost (*c).
__device__ __forceinline__ void precise_tau(const SampleF &a, const SampleF &b, float tmax,
                                            double *t_out, double *c_out) {
  const PairQuartic pq = make_pair_quartic(a, b);
  float cand[2] = {0.0f, 0.0f};
  bool tmax_cand = false;
  const int nc = minima_f32(pq.f, tmax, &cand[0], &cand[1], &tmax_cand);
  // primary candidate, evaluated by every lane with the same instructions
  const bool primary_root = nc > 0;
  const double tm = f2d_exact(tmax);
  const double xr = refine(pq, primary_root ? cand[0] : tmax);
  double best_t = primary_root ? xr : tm;
  double best_c = pq.q.cost(best_t);
  // rare: a second interior minimum, or the cost still falling at tmax
  if (nc > 1) {
    const double t2 = refine(pq, cand[1]);
    const double c2 = pq.q.cost(t2);
    if (c2 < best_c) { best_c = c2; best_t = t2; }
  }
  if (primary_root && tmax_cand) {
    const double c3 = pq.q.cost(tm);
    if (c3 < best_c) { best_c = c3; best_t = tm; }
  }
  *t_out = best_t;
  *c_out = best_c;
}

// The same for a pair given only in binary32.
__device__ __forceinline__ void precise_tau(const float *x0, const float *x1, float tmax,
                                            double *t_out, double *c_out) {
  precise_tau(to_sample_f(x0), to_sample_f(x1), tmax, t_out, c_out);
}

}  // namespace
}  // namespace pump
