// Binary32 costs of the reference's 2pBVP cost expression from float-float
// arithmetic, certified against the binary64 evaluation (bvp.cu for the
// reference built for the CPU, bvp_refgpu.cu for its GPU kernel).
//
// The same bound holds for the reference's GPU kernel (bvp_refgpu.cu): there
// nvcc may fuse any of its binary64 multiply-adds (a fused operation rounds
// once, within the same 2^-53 of its result), and CUDA's pow, which the
// expression calls for tau^2, tau^3, tau^4 and the coordinates' squares, is
// within 2 ulp (2^-51) of the power, so the terms' magnitudes times 2^-50
// cover it (2^-46.9 with the roundings, inside the 2^-41 below).  Its one
// binary32 multiply-add, b + c tau in the last two terms, is written here as
// the reference writes it, and bvp_refgpu.cu is compiled with contraction as
// the reference is; the GPU tests compare every pair with the reference
// kernel's own results.
#pragma once
#include "common.cuh"

namespace pump {
namespace {

// cost_eval rounds 25 binary64 additions and about 15 binary64 products, and
// the GB300 executes binary64 at 1/64 of its binary32 rate, so the parity
// kernels are bound by that pipe.  cost_fast gets the same binary32 result
// from binary32 arithmetic in most evaluations: it evaluates the bracket sum
// V (the same terms; the t^2, t^3 and t^4 coefficients summed per pair) and
// V / t^3 in float-float arithmetic (Dekker's and Knuth's error-free
// TwoSum and TwoProduct; double-float addition, multiplication and division
// as in Bailey's double-double library, with binary32 parts), and bounds the
// distance of cost_eval's binary64 value from it:
//   - cost_eval's sum: each of its 31 additions (s7's six included) and ~15
//     products is rounded once (|error| <= 2^-53 of the partial sum or
//     product; t^3 and t^4 are themselves rounded products), so its error is
//     at most 2^-52 x 33 x (the sum of the terms' magnitudes) = 2^-47 x that
//     sum;
//   - the float-float evaluation, counted with worst-case constants per
//     operation (u = 2^-24; double-word bounds of Joldes, Muller and
//     Popescu, 2017, and 7 u^2 (|x| + |y|) for the fast sum): s7 and the
//     t^2 coefficient's sums (make_pair_ff) 21 u^2 and 30 u^2 with their
//     product, the t^3 and t^4 terms 7.5 u^2 and 14 u^2, the eight binary32
//     terms 16 u^2, the three fast sums 21 u^2, the last two terms 4 u^2:
//     at most 114 u^2 = 2^-41.2 x that sum;
//   - the bound below takes 2^-41 x 1.01 of the sum (129 u^2), above the
//     two together (116 u^2; the reference's GPU kernel's binary64 value is
//     within 2.1 u^2 of it, see above);
//   - the final 1 / t^3 and the product (three more binary64 roundings) and
//     the float-float division (its residual a fast sum): at most 2^-42 of
//     the result.
// When that interval around the float-float value lies inside the binary32
// rounding cell of its high part (it does not reach the midpoint to either
// neighbour), cost_eval's (float) conversion gives that high part, which is
// returned.  Otherwise (and for tau outside [1e-4, 1e4], or a non-finite or
// subnormal result) the binary64 evaluation runs.  The binary32 terms that
// the reference rounds are products written as __fmul_rn, which no compiler
// fuses into the sums that follow (bvp_refgpu.cu is compiled with
// contraction, and a product with a single use would otherwise become a
// multiply-add); TwoProduct calls fmaf explicitly.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ FF ff_two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ FF ff_add(FF x, FF y) {
  FF s = ff_two_sum(x.hi, y.hi);
  const FF t = ff_two_sum(x.lo, y.lo);
  s.lo = s.lo + t.hi;
  s = ff_fast_two_sum(s.hi, s.lo);
  s.lo = s.lo + t.lo;
  return ff_fast_two_sum(s.hi, s.lo);
}
// Double-word sum without the second TwoSum ("sloppy" addition): its error
// is at most about 8 u^2 (|x| + |y|), u = 2^-24, also under cancellation,
// which is all cost_ff's bound (taken over the terms' magnitudes) needs.
__device__ __forceinline__ FF ff_add_fast(FF x, FF y) {
  FF s = ff_two_sum(x.hi, y.hi);
  s.lo = s.lo + (x.lo + y.lo);
  return ff_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ FF ff_add_f(FF x, float b) {
  FF s = ff_two_sum(x.hi, b);
  s.lo = s.lo + x.lo;
  return ff_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ FF ff_mul(FF x, FF y) {
  FF p = ff_two_prod(x.hi, y.hi);
  p.lo = p.lo + (x.hi * y.lo + x.lo * y.hi);
  return ff_fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ FF ff_mul_f(FF x, float b) {
  FF p = ff_two_prod(x.hi, b);
  p.lo = p.lo + x.lo * b;
  return ff_fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ FF ff_div(FF x, FF y) {
  const float q1 = __fdiv_rn(x.hi, y.hi);
  const FF qy = ff_mul_f(y, q1);
  const FF r = ff_add(x, {-qy.hi, -qy.lo});
  const float q2 = __fdiv_rn(r.hi, y.hi);
  return ff_fast_two_sum(q1, q2);
}

// Per-pair data of cost_ff, built without binary64 arithmetic (the GB300's
// binary64 conversions and products would cost the pair kernel a quarter of
// its time): the binary32 coefficients of cost_eval's t-linear and last two
// terms; s7 as the float-float sum of its seven terms (each exact: 12 x^2 is
// a TwoProduct scaled by 4 and then by 3 with a TwoProduct, 24 x y is the
// binary32 product cost_eval converts) and the sum of their magnitudes; the
// sums of the t^2 and t^3 coefficients and their magnitudes.  cost_eval's
// own s7 differs from the exact sum by its six binary64 roundings, which
// cost_ff's bound covers.
struct PairFF {
  float k8, k9, k10, k11, k12, k13, k14, k15;
  float a29, b29, c29, a30, b30, c30;
  FF s7, d2, d3;
  float abs_s7, abs_d2, abs_d3;
  float abs_k;  // |k8| + ... + |k15| (times tau: the t-linear terms' magnitudes)
};
__device__ __forceinline__ FF ff_12sq(float x) {
  FF t = ff_two_prod(x, x);
  t.hi *= 4.0f;
  t.lo *= 4.0f;
  FF p = ff_two_prod(t.hi, 3.0f);
  p.lo = p.lo + t.lo * 3.0f;
  return ff_fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ PairFF make_pair_ff(const float *x0, const float *x1) {
  const float g = PUMP_G;
  PairFF f;
  // the binary32 terms, as make_coef computes them
  f.k8 = 12 * x0[4] * x0[1];
  f.k9 = 12 * x0[1] * x1[4];
  f.k10 = 12 * x0[3] * x1[0];
  f.k11 = 12 * x1[3] * x1[0];
  f.k12 = 12 * x0[5] * x1[2];
  f.k13 = 12 * x1[5] * x1[2];
  f.k14 = 12 * x0[4] * x1[1];
  f.k15 = 12 * x1[4] * x1[1];
  f.abs_k = ((fabsf(f.k8) + fabsf(f.k9)) + (fabsf(f.k10) + fabsf(f.k11))) +
            ((fabsf(f.k12) + fabsf(f.k13)) + (fabsf(f.k14) + fabsf(f.k15)));
  f.a29 = 12 * x0[0];
  f.b29 = -2 * x1[0];
  f.c29 = x0[3] + x1[3];
  f.a30 = 12 * x0[2];
  f.b30 = -2 * x1[2];
  f.c30 = x0[5] + x1[5];
  // s7, make_coef's first seven terms
  FF s = ff_12sq(x0[0]);
  float as = s.hi;
  const float sq[5] = {x0[2], x0[1], x1[0], x1[2], x1[1]};
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    if (q == 4) {
      const float c24 = __fmul_rn(24 * x0[1], x1[1]);
      s = ff_add_f(s, -c24);
      as += fabsf(c24);
    }
    const FF t = ff_12sq(sq[q]);
    s = ff_add(s, t);
    as += t.hi;
  }
  f.s7 = s;
  f.abs_s7 = as;
  // 4 x^2 (exact as a TwoProduct scaled by 4) and the float coefficients
  const float sq4[6] = {x0[4], x0[3], x0[5], x1[4], x1[3], x1[5]};
  FF d = {0.0f, 0.0f};
  float ad = 0.0f;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    FF t = ff_two_prod(sq4[q], sq4[q]);
    t.hi *= 4.0f;
    t.lo *= 4.0f;
    d = ff_add(d, t);
    ad += t.hi;
  }
  const float fl[3] = {__fmul_rn(4 * x0[4], x1[4]), __fmul_rn(4 * x0[3], x1[3]),
                       __fmul_rn(4 * x0[5], x1[5])};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    d = ff_add_f(d, fl[q]);
    ad += fabsf(fl[q]);
  }
  f.d2 = d;
  f.abs_d2 = ad;
  const float f25 = __fmul_rn(2 * g, x0[5]), f26 = __fmul_rn(2 * g, x1[5]);
  f.d3 = ff_two_sum(f25, -f26);
  f.abs_d3 = fabsf(f25) + fabsf(f26);
  return f;
}

// The certified value, or *ok = false (then cost_eval gives the result).
__device__ __forceinline__ float cost_ff(const PairFF &f, float tau, bool *ok) {
  *ok = false;
  if (!(tau >= 1e-4f && tau <= 1e4f)) return 0.0f;
  // the float terms, as cost_eval rounds them
  const float k[8] = {__fmul_rn(f.k8, tau),     __fmul_rn(f.k9, tau),
                      -__fmul_rn(f.k10, tau),    -__fmul_rn(f.k11, tau),
                      -__fmul_rn(f.k12, tau),    -__fmul_rn(f.k13, tau),
                      -__fmul_rn(f.k14, tau),    -__fmul_rn(f.k15, tau)};
  // b + c tau as the reference writes it (contracted where the reference's
  // build contracts it), the outer product rounded (the reference converts
  // it to binary64 before adding it)
  const float a29 = __fmul_rn(f.a29, f.b29 + f.c29 * tau);
  const float a30 = __fmul_rn(f.a30, f.b30 + f.c30 * tau);
  FF v = f.s7;
  // |k[q]| = |k_q| tau to within 2^-24 of each, and abs_k is the sum of the
  // |k_q| to within 2^-21: inside the bound's 1 % margin
  float mag = f.abs_s7 + f.abs_k * tau;
#pragma unroll
  for (int q = 0; q < 8; ++q) v = ff_add_f(v, k[q]);
  const FF t2 = ff_two_prod(tau, tau);
  const FF t3 = ff_mul_f(t2, tau);
  const FF t4 = ff_mul(t2, t2);
  // 1 + g^2, the t^4 coefficient (g^2 exact as a TwoProduct)
  const float g = PUMP_G;
  const FF g2 = ff_two_prod(g, g);
  const FF d4 = ff_add_f(g2, 1.0f);
  v = ff_add_fast(v, ff_mul(f.d2, t2));
  v = ff_add_fast(v, ff_mul(f.d3, t3));
  v = ff_add_fast(v, ff_mul(d4, t4));
  v = ff_add_f(v, a29);
  v = ff_add_f(v, a30);
  mag += f.abs_d2 * t2.hi + f.abs_d3 * t3.hi + d4.hi * t4.hi + fabsf(a29) + fabsf(a30);
  // v / t3 as ff_div, the residual v - q1 t3 with the fast sum (its error,
  // 8 u^2 of |v| + |q1 t3|, is 2^-44 of the quotient)
  FF w;
  {
    const float q1 = __fdiv_rn(v.hi, t3.hi);
    const FF qy = ff_mul_f(t3, q1);
    const FF r = ff_add_fast(v, {-qy.hi, -qy.lo});
    const float q2 = __fdiv_rn(r.hi, t3.hi);
    w = ff_fast_two_sum(q1, q2);
  }
  // the bound on |cost_eval's binary64 value - w| (margins for the binary32
  // evaluation of the bound itself)
  const float aw = fabsf(w.hi);
  const float bound = (mag * 1.01f) * 0x1p-41f / t3.hi + aw * 0x1p-42f;
  const unsigned int u = __float_as_uint(aw);
  const unsigned int e = u >> 23;
  if (e < 2u || e > 253u) return 0.0f;  // zero, subnormal, huge, inf, NaN
  const float ulp_up = __uint_as_float(u + 1u) - aw, ulp_dn = aw - __uint_as_float(u - 1u);
  const float room = 0.5f * fminf(ulp_up, ulp_dn) - fabsf(w.lo);
  *ok = bound < 0.99f * room;
  return w.hi;
}


}  // namespace
}  // namespace pump
