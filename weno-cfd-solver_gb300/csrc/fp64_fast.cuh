// FAST FP64 reciprocal, reciprocal square root and square root.
//
// GB300 runs FP64 at 1/64 of the FP32 rate, and CUDA's correctly rounded FP64
// divide costs about ten FP64 pipe slots.  These forms take three
// (reciprocal) or five (reciprocal square root) FP64 operations; the rest is
// integer and FP32 work on pipes that the FP64-bound kernels leave idle.
//
// Method (Newton's iteration raised to third order, i.e. Householder's method
// of order 2, on a hardware seed):
//  * x = m 2^E is split on its integer bits: m in [1, 2) for the reciprocal,
//    m in [1, 4) with E even for the square roots;
//  * a seed y0 of 1/m or 1/sqrt(m) comes from the PTX instructions
//    rcp.approx.ftz.f32 / rsqrt.approx.ftz.f32 applied to the leading 23 bits
//    of m (relative error of y0 below 2^-21), widened to double on its bits;
//  * one step of the series
//      1/m       = y0 / (1 - e)        = y0 (1 + e + e^2 + ...),       e = 1 - m y0
//      1/sqrt(m) = y0 (1 - e)^(-1/2)   = y0 (1 + e/2 + 3e^2/8 + ...),   e = 1 - m y0^2
//    truncated after e^2 (truncation error below 2^-60 relative); e is formed
//    by one fused multiply-add, exactly rounded (y0^2 is exact: y0 has 24
//    significant bits);
//  * 2^-E (or 2^-E/2) is put back on the exponent bits of the result.
// The reciprocal and the reciprocal square root are within 1 ulp, the square
// root (x times its reciprocal square root) within 2 ulp.  Arguments whose
// exponent lies outside [-1000, 1000] (zero, subnormals, infinities, NaN) and
// negative arguments of the square roots take CUDA's IEEE operations.
//
// rcp2 stops the series after e (Newton's step, two FP64 operations): relative
// error below 2^-41 (the seed's error squared).  It serves quotients whose
// relative error only scales a small correction -- the normalisation of the
// WENO weights, which multiplies the weighted slope added to a centre value,
// and the shared 1/(rho_a rho_b) of two Euler fluxes.
#pragma once

#include <cuda_runtime.h>

namespace weno {
namespace f64fast {

constexpr int kExpLo = 1023 - 1000, kExpHi = 1023 + 1000;  // biased exponents of the fast range

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// A positive normal float as a double, on the bits (exact).
__device__ __forceinline__ double widen(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned hi = (((b >> 23) + (1023u - 127u)) << 20) | ((b & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)((b & 7u) << 29));
}

// The leading 23 mantissa bits of the double (hi, lo) under the float biased
// exponent fexp.
__device__ __forceinline__ float narrow(int hi, int lo, unsigned fexp) {
  return __uint_as_float((fexp << 23) | (((unsigned)hi & 0xfffffu) << 3) | ((unsigned)lo >> 29));
}

__device__ __forceinline__ int biased_exp(int hi) { return (hi >> 20) & 0x7ff; }

// 1/x for x with biased exponent in [kExpLo, kExpHi] (either sign).
__device__ __forceinline__ double rcp_core(int hi, int lo) {
  const int ex = biased_exp(hi);
  const double m = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, lo);
  const double y0 = widen(rcp_approx(narrow(hi, lo, 127u)));
  const double e = fma(-m, y0, 1.0);
  const double y = fma(y0, fma(e, e, e), y0);  // in [0.5, 1]
  const int yh = __double2hiint(y) - (ex - 1023) * (1 << 20);
  return __hiloint2double(yh | (hi & (int)0x80000000), __double2loint(y));
}

// The same with the series truncated after e.
__device__ __forceinline__ double rcp2_core(int hi, int lo) {
  const int ex = biased_exp(hi);
  const double m = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, lo);
  const double y0 = widen(rcp_approx(narrow(hi, lo, 127u)));
  const double y = fma(y0, fma(-m, y0, 1.0), y0);  // in [0.5, 1]
  const int yh = __double2hiint(y) - (ex - 1023) * (1 << 20);
  return __hiloint2double(yh | (hi & (int)0x80000000), __double2loint(y));
}

// 1/sqrt(x) for positive x with biased exponent in [kExpLo, kExpHi].
__device__ __forceinline__ double rsqrt_core(int hi, int lo) {
  const int e2 = biased_exp(hi) - 1023;
  const int odd = e2 & 1;
  const double m = __hiloint2double((hi & 0x000fffff) | ((1023 + odd) << 20), lo);
  const double y0 = widen(rsqrt_approx(narrow(hi, lo, 127u + (unsigned)odd)));
  const double e = fma(-m, y0 * y0, 1.0);
  const double y = fma(y0 * e, fma(0.375, e, 0.5), y0);  // in [0.5, 1]
  const int yh = __double2hiint(y) - ((e2 - odd) / 2) * (1 << 20);
  return __hiloint2double(yh, __double2loint(y));
}

__device__ __forceinline__ double rcp(double x) {
  const int hi = __double2hiint(x), lo = __double2loint(x);
  const int ex = biased_exp(hi);
  if (ex < kExpLo || ex > kExpHi) return 1.0 / x;
  return rcp_core(hi, lo);
}

__device__ __forceinline__ double rcp2(double x) {
  const int hi = __double2hiint(x), lo = __double2loint(x);
  const int ex = biased_exp(hi);
  if (ex < kExpLo || ex > kExpHi) return 1.0 / x;
  return rcp2_core(hi, lo);
}

__device__ __forceinline__ double rsqrt(double x) {
  const int hi = __double2hiint(x), lo = __double2loint(x);
  const int ex = biased_exp(hi);
  if (hi < 0 || ex < kExpLo || ex > kExpHi) return ::rsqrt(x);
  return rsqrt_core(hi, lo);
}

__device__ __forceinline__ double sqrt(double x) {
  const int hi = __double2hiint(x), lo = __double2loint(x);
  const int ex = biased_exp(hi);
  if (hi < 0 || ex < kExpLo || ex > kExpHi) return ::sqrt(x);
  return x * rsqrt_core(hi, lo);
}

}  // namespace f64fast
}  // namespace weno
