// df64: a double-float number (hi + lo, two IEEE floats, |lo| <= ulp(hi)/2),
// about 48 significant bits, evaluated on the FP32 pipes.
//
// GB300 issues FP32 FMAs at 64x the FP64 rate, so FP64-class arithmetic built
// from error-free float transformations runs several times faster than native
// doubles on this GPU.  The algorithms are the classical ones:
//   two_sum        Knuth, TAOCP vol. 2 (exact a + b = s + e)
//   quick_two_sum  Dekker 1971 (|a| >= |b|)
//   two_prod       with a fused multiply-add (exact a * b = p + e)
//   add / mul      the "accurate" double-double forms of Hida, Li and Bailey
//                  (QD library paper, 2001)
//   div, sqrt      one Newton step on a float approximation, as in the same paper.
// The exponent range is that of float (about 1e-38 .. 3e38); callers keep
// values inside it (see the range guard of the kernels that use this type).
#pragma once

#include <cuda_runtime.h>

namespace weno {
// The type and its functions live in their own namespace: argument-dependent
// lookup finds fmax/sqrt/... for df64 arguments, while unqualified calls on
// doubles inside namespace weno still reach the CUDA math functions.
namespace dfm {

struct df64 {
  float hi, lo;
  __host__ __device__ constexpr df64() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  // Rounded split of a double: hi = fl(x), lo = fl(x - hi).
  __host__ __device__ constexpr df64(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  __host__ __device__ constexpr df64(int x) : hi((float)x), lo(0.f) {}
  __host__ __device__ double to_double() const { return (double)hi + (double)lo; }
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};
static_assert(sizeof(df64) == 8, "df64 is stored as two floats");

namespace dfd {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void quick_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

}  // namespace dfd

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  float s, e, t, f;
  dfd::two_sum(a.hi, b.hi, s, e);
  dfd::two_sum(a.lo, b.lo, t, f);
  e = __fadd_rn(e, t);
  dfd::quick_two_sum(s, e, s, e);
  e = __fadd_rn(e, f);
  dfd::quick_two_sum(s, e, s, e);
  return df64(s, e);
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  float p, e;
  dfd::two_prod(a.hi, b.hi, p, e);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  dfd::quick_two_sum(p, e, p, e);
  return df64(p, e);
}
// Division: q1 = a.hi / b.hi (float), r = a - q1 * b, q2 = r.hi / b.hi, q1 + q2.
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df64 r = a - b * df64(q1, 0.f);
  const float q2 = __fdiv_rn(r.hi, b.hi);
  float s, e;
  dfd::quick_two_sum(q1, q2, s, e);
  return df64(s, e);
}
__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }

__device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }
__device__ __forceinline__ bool operator<=(df64 a, df64 b) { return !(b < a) && a.hi == a.hi && b.hi == b.hi; }
__device__ __forceinline__ bool operator>=(df64 a, df64 b) { return b <= a; }
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return !(a == b); }

// max / min with the IEEE maxNum rule of the reference's f64::max (a NaN
// operand yields the other operand).
__device__ __forceinline__ df64 fmax(df64 a, df64 b) {
  if (a.hi != a.hi) return b;
  if (b.hi != b.hi) return a;
  return (a < b) ? b : a;
}
__device__ __forceinline__ df64 fmin(df64 a, df64 b) {
  if (a.hi != a.hi) return b;
  if (b.hi != b.hi) return a;
  return (b < a) ? b : a;
}
__device__ __forceinline__ df64 fabs(df64 a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ df64 copysign(df64 mag, df64 sgn) {
  const df64 m = fabs(mag);
  return signbit(sgn.hi) ? -m : m;
}
// sqrt: x = sqrt(a.hi) (float), then one Newton correction
// s = x + (a - x*x) / (2x) in double-float arithmetic.
__device__ __forceinline__ df64 sqrt(df64 a) {
  if (!(a.hi > 0.f)) return df64(sqrtf(a.hi), 0.f);  // 0, negative (NaN) or NaN
  const float x = sqrtf(a.hi);
  float p, e;
  dfd::two_prod(x, x, p, e);
  const df64 r = a - df64(p, e);
  const float corr = __fdiv_rn(r.hi, 2.f * x);
  float s, t;
  dfd::quick_two_sum(x, corr, s, t);
  return df64(s, t);
}

}  // namespace dfm
using dfm::df64;
}  // namespace weno
