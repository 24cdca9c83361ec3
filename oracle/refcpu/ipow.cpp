/*
 * Correctly rounded integer powers for the oracle's CPU build of the
 * reference.
 *
 * The reference evaluates pow(float, int) through the C++ promotion to
 * pow(double, double) (2pBVP.cu:99-105, 2pBVP.cu:117-131).  glibc's pow is
 * not correctly rounded: for x = (double)float it differs from the correctly
 * rounded x^3 (or x^4) in about 0.24 % of inputs, and CUDA's device pow has
 * its own error pattern.  Parity is defined on one platform-independent
 * arithmetic: for a float-valued x, x*x is exact in binary64, so x^2, x^3 and
 * x^4 computed as (x*x), (x*x)*x and (x*x)*(x*x) are each rounded exactly
 * once, i.e. correctly rounded.  This override makes the reference's own code
 * compute exactly that; any other argument goes to the C library's pow.
 *
 * Test infrastructure only (linked into oracle/_ref builds of the reference).
 */
#include <dlfcn.h>

namespace {
typedef double (*pow_fn)(double, double);
pow_fn libm_pow() {
  static pow_fn f = (pow_fn)dlsym(RTLD_NEXT, "pow");
  return f;
}
}  // namespace

extern "C" double pow(double x, double y) {
  if ((double)(float)x == x) {
    if (y == 2.0) return x * x;
    if (y == 3.0) return (x * x) * x;
    if (y == 4.0) {
      double s = x * x;
      return s * s;
    }
  }
  return libm_pow()(x, y);
}
