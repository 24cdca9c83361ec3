// Edge trajectory states (pathPoint, 2pBVP.cu:117-131): shared by the
// waypoint kernels, the dense-path kernels and the search's edge checks.
// Translation units that include this file compile without multiply-add
// contraction, so every rounding is the reference's.
#pragma once

#include "common.cuh"
#include "ffcost.cuh"

namespace pump {

// pathPoint, 2pBVP.cu:117-131, in the expression's own evaluation types.
__device__ __forceinline__ void path_point(float t, float tau, const float *x0, const float *x1,
                                           float *x) {
  const double t2 = p2f(t), t3 = p3f(t), u2 = p2f(tau), u3 = p3f(tau);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int a = k, b = k + 3;
    double r = (double)(t * x0[b] + x0[a]);
    r = r + (t3 * (double)(2 * x0[a] - 2 * x1[a] + (x0[b] + x1[b]) * tau)) / u3;
    r = r - (t2 * (double)(3 * x0[a] - 3 * x1[a] + (2 * x0[b] + x1[b]) * tau)) / u2;
    x[k] = (float)r;
  }
  {
    double r = (double)(t * x0[5]) * u3 + (double)x0[2] * u3;
    double q1 = -3. * x0[2] + 3. * x1[2] - 2. * x0[5] * tau - 1. * x1[5] * tau;
    r = r + (t2 * (double)tau) * q1;
    double q2 = 2. * x0[2] - 2. * x1[2] + (double)((x0[5] + x1[5]) * tau);
    r = r + t3 * q2;
    x[2] = (float)(r / u3);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int a = k, b = k + 3;
    float f1 = -(2 * t * (3 * x0[a] - 3 * x1[a] + x1[b] * tau));
    double r = (double)f1 / u2;
    r = r + (3 * t2 * (double)(2 * x0[a] - 2 * x1[a] + x1[b] * tau)) / u3;
    double inner = 3 * t2 - (double)(4 * t * tau) + u2;
    r = r + ((double)x0[b] * inner) / u2;
    x[3 + k] = (float)r;
  }
  {
    double r = (double)x0[5] * u3;
    double q1 = -6. * x0[2] + 6. * x1[2] - 4. * x0[5] * tau - 2. * x1[5] * tau;
    r = r + (double)(t * tau) * q1;
    double q2 = 6. * x0[2] - 6. * x1[2] + 3. * x0[5] * tau + 3. * x1[5] * tau;
    r = r + t2 * q2;
    x[5] = (float)(r / u3);
  }
}

// path_point's binary32 results from float-float arithmetic (ffcost.cuh's
// operations), certified as in cost_ff: each state is the sum of a few terms
// (the position x0 + ... as A + t^3 X / tau^3 - t^2 Y / tau^2, with A, X and
// Y the binary32 values path_point converts), evaluated exactly enough in
// float-float; path_point's binary64 value differs from the exact sum of
// those terms by its roundings (at most 16 of them, each within 2^-53 of a
// partial result no larger than M, the sum of the terms' magnitudes, tau^3
// and t^3 included: 2^-49 M), and the float-float value by at most about
// 37 u^2 M = 2^-42.8 M (u = 2^-24; with the double-word error bounds of
// Joldes, Muller and Popescu, 2017: 1.5 u^2 per product by a binary32,
// 6 u^2 per product, 15 u^2 per quotient, 3 u^2 per sum, 25 to 28 u^2 for a
// term, 9 u^2 for the three sums).
// When the interval of half-width 2^-41 M around the float-float value lies
// inside the binary32 rounding cell of its high part, that is path_point's
// (float) conversion; otherwise (or for tau outside [2^-20, 2^20], values
// outside [2^-40, 2^60] and non-finite values) path_point runs.  The
// per-edge terms (path_ff_edge) are shared by the edge's waypoints.
struct PathFF {
  bool ok;                           // tau in range: the float-float path applies
  FF u2, ru2, ru3;                   // tau^2 (exact), 1 / tau^2, 1 / tau^3
  float X[2], Y[2], inner[2], Z[2];  // path_point's binary32 edge terms
  FF q1, q2, q1v, q2v;               // its binary64 edge sums, exactly
  float mq1, mq2, mq1v, mq2v;        // their terms' magnitudes
};

__device__ __forceinline__ FF ff_neg(FF x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ PathFF path_ff_edge(float tau, const float *x0, const float *x1) {
  PathFF e;
  e.ok = tau >= 0x1p-20f && tau <= 0x1p20f;
  e.u2 = ff_two_prod(tau, tau);
  const FF u3 = ff_mul_f(e.u2, tau);
  const FF one = {1.0f, 0.0f};
  e.ru2 = ff_div(one, e.u2);
  e.ru3 = ff_div(one, u3);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int a = k, b = k + 3;
    // the same binary32 expressions as path_point
    e.X[k] = 2 * x0[a] - 2 * x1[a] + (x0[b] + x1[b]) * tau;
    e.Y[k] = 3 * x0[a] - 3 * x1[a] + (2 * x0[b] + x1[b]) * tau;
    e.inner[k] = 3 * x0[a] - 3 * x1[a] + x1[b] * tau;
    e.Z[k] = 2 * x0[a] - 2 * x1[a] + x1[b] * tau;
  }
  // -3 x0z + 3 x1z - 2 x0vz tau - x1vz tau (each term exact in binary64)
  {
    const FF a = ff_two_prod(x0[2], -3.0f), b = ff_two_prod(x1[2], 3.0f);
    const FF c = ff_two_prod(2.0f * x0[5], -tau), d = ff_two_prod(x1[5], -tau);
    e.q1 = ff_add(ff_add(ff_add(a, b), c), d);
    e.mq1 = fabsf(a.hi) + fabsf(b.hi) + fabsf(c.hi) + fabsf(d.hi);
  }
  // 2 x0z - 2 x1z + (binary32 (x0vz + x1vz) tau)
  {
    const float w = (x0[5] + x1[5]) * tau;
    const FF ab = ff_two_sum(2.0f * x0[2], -2.0f * x1[2]);
    e.q2 = ff_add_f(ab, w);
    e.mq2 = fabsf(2.0f * x0[2]) + fabsf(2.0f * x1[2]) + fabsf(w);
  }
  // -6 x0z + 6 x1z - 4 x0vz tau - 2 x1vz tau
  {
    const FF a = ff_two_prod(x0[2], -6.0f), b = ff_two_prod(x1[2], 6.0f);
    const FF c = ff_two_prod(4.0f * x0[5], -tau), d = ff_two_prod(2.0f * x1[5], -tau);
    e.q1v = ff_add(ff_add(ff_add(a, b), c), d);
    e.mq1v = fabsf(a.hi) + fabsf(b.hi) + fabsf(c.hi) + fabsf(d.hi);
  }
  // 6 x0z - 6 x1z + 3 x0vz tau + 3 x1vz tau
  {
    const FF a = ff_two_prod(x0[2], 6.0f), b = ff_two_prod(x1[2], -6.0f);
    const FF c = ff_mul_f(ff_two_prod(x0[5], tau), 3.0f), d = ff_mul_f(ff_two_prod(x1[5], tau), 3.0f);
    e.q2v = ff_add(ff_add(ff_add(a, b), c), d);
    e.mq2v = fabsf(a.hi) + fabsf(b.hi) + fabsf(c.hi) + fabsf(d.hi);
  }
  return e;
}

// *out = the binary32 rounding of every value within 2^-41 M + 2^-80 of v
// (true), or false when the interval reaches a rounding boundary (or leaves
// range).  The absolute 2^-80 covers float-float parts that fall below
// binary32's normal range (each at most 2^-149 off, scaled by at most 2^60
// through 1 / tau^3).
__device__ __forceinline__ bool ff_certify(FF v, float M, float *out) {
  const float f = v.hi, af = fabsf(f);
  if (!(af >= 0x1p-40f && af <= 0x1p60f && M <= 0x1p60f)) return false;  // also NaN
  const unsigned bits = __float_as_uint(af);
  const float ulp = __uint_as_float((bits & 0x7f800000u) - (23u << 23));
  const float up = 0.5f * ulp, down = (bits & 0x7fffffu) ? 0.5f * ulp : 0.25f * ulp;
  const float a = f >= 0.0f ? v.lo : -v.lo;  // offset towards larger magnitude
  const float B = M * (0x1p-41f * 1.01f) + 0x1p-80f;
  *out = f;
  return a + B < up && B - a < down;
}

// x = path_point's values when every state is certified (true); false
// leaves x unspecified.
__device__ __forceinline__ bool path_point_try(float t, float tau, const float *x0,
                                               const float *x1, const PathFF &e, float *x) {
  bool ok = e.ok;
  const FF t2 = ff_two_prod(t, t);
  const FF t3 = ff_mul_f(t2, t);
  float v[kDim];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int a = k, b = k + 3;
    // position: A + t^3 X / tau^3 - t^2 Y / tau^2
    const float A = t * x0[b] + x0[a];
    const FF T1 = ff_mul(ff_mul_f(t3, e.X[k]), e.ru3);
    const FF T2 = ff_mul(ff_mul_f(t2, e.Y[k]), e.ru2);
    const FF V = ff_add(ff_add_f(T1, A), ff_neg(T2));
    ok = ff_certify(V, fabsf(A) + fabsf(T1.hi) + fabsf(T2.hi), &v[k]) && ok;
    // velocity: f1 / tau^2 + 3 t^2 Z / tau^3 + x0v (3 t^2 - F + tau^2) / tau^2
    const float f1 = -(2 * t * e.inner[k]);
    const float F = 4 * t * tau;
    const FF t2x3 = ff_mul_f(t2, 3.0f);
    const FF S1 = ff_mul_f(e.ru2, f1);
    const FF S2 = ff_mul(ff_mul_f(t2x3, e.Z[k]), e.ru3);
    const FF in = ff_add(ff_add_f(t2x3, -F), e.u2);
    const FF S3 = ff_mul(ff_mul_f(in, x0[b]), e.ru2);
    const FF W = ff_add(ff_add(S1, S2), S3);
    const float MW = fabsf(S1.hi) + fabsf(S2.hi) +
                     fabsf(x0[b]) * ((t2x3.hi + fabsf(F)) + e.u2.hi) * e.ru2.hi;
    ok = ff_certify(W, MW, &v[3 + k]) && ok;
  }
  {
    // z: t x0vz + x0z + t^2 q1 / tau^2 + t^3 q2 / tau^3
    const float P = t * x0[5];
    const FF T1 = ff_mul(ff_mul(t2, e.q1), e.ru2);
    const FF T2 = ff_mul(ff_mul(t3, e.q2), e.ru3);
    const FF V = ff_add(ff_add(ff_two_sum(P, x0[2]), T1), T2);
    const float M = fabsf(P) + fabsf(x0[2]) + t2.hi * e.ru2.hi * e.mq1 + t3.hi * e.ru3.hi * e.mq2;
    ok = ff_certify(V, M, &v[2]) && ok;
  }
  {
    // vz: x0vz + (t tau) q1v / tau^3 + t^2 q2v / tau^3
    const float tt = t * tau;
    const FF T1 = ff_mul(ff_mul_f(e.q1v, tt), e.ru3);
    const FF T2 = ff_mul(ff_mul(t2, e.q2v), e.ru3);
    const FF V = ff_add(ff_add_f(T1, x0[5]), T2);
    const float M = fabsf(x0[5]) + (fabsf(tt) * e.mq1v + t2.hi * e.mq2v) * e.ru3.hi;
    ok = ff_certify(V, M, &v[5]) && ok;
  }
#pragma unroll
  for (int d = 0; d < kDim; ++d) x[d] = v[d];
  return ok;
}

// path_point_try, else path_point; certified (when given): whether the
// float-float values were used.
__device__ __forceinline__ void path_point_ff(float t, float tau, const float *x0, const float *x1,
                                              const PathFF &e, float *x,
                                              bool *certified = nullptr) {
  const bool ok = path_point_try(t, tau, x0, x1, e, x);
  if (certified) *certified = ok;
  if (!ok) path_point(t, tau, x0, x1, x);
}

// path_point through path_point_ff, the edge terms computed here.
__device__ __forceinline__ void path_point_fast(float t, float tau, const float *x0,
                                                const float *x1, float *x) {
  path_point_ff(t, tau, x0, x1, path_ff_edge(tau, x0, x1), x);
}

// The same trajectory as path_point (cubic position, quadratic velocity,
// no gravity term) in binary32 Hermite form with s = t / tau; used by the
// precision mode, where FP64 is reserved for the optimal-time root.
__device__ __forceinline__ void path_point_f32(float t, float tau, const float *x0, const float *x1,
                                               float *x) {
  const float s = t / tau;
  const float s2 = s * s, s3 = s2 * s;
  const float h00 = fmaf(2.0f, s3, fmaf(-3.0f, s2, 1.0f)), h01 = fmaf(-2.0f, s3, 3.0f * s2);
  const float h10 = tau * (s3 - 2.0f * s2 + s), h11 = tau * (s3 - s2);
  const float g00 = (6.0f * s2 - 6.0f * s) / tau, g10 = fmaf(3.0f, s2, fmaf(-4.0f, s, 1.0f));
  const float g11 = fmaf(3.0f, s2, -2.0f * s);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    x[k] = fmaf(h00, x0[k], fmaf(h01, x1[k], fmaf(h10, x0[k + 3], h11 * x1[k + 3])));
    x[k + 3] = fmaf(g00, x0[k] - x1[k], fmaf(g10, x0[k + 3], g11 * x1[k + 3]));
  }
}

}  // namespace pump
