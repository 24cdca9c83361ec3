// Edge trajectory states (pathPoint, 2pBVP.cu:117-131): shared by the
// waypoint kernels, the dense-path kernels and the search's edge checks.
// Translation units that include this file compile without multiply-add
// contraction, so every rounding is the reference's.
#pragma once

#include "common.cuh"

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
