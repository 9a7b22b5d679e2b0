// f32x2: two independent FP32 values processed by the packed FP32x2
// instructions of sm_100-class GPUs (FADD2 / FMUL2 / FFMA2: one instruction,
// two IEEE-rounded results).
//
// The FP32 kernels are instruction-issue bound, so running the branch-free
// WENO arithmetic of two fields (or two components) at once halves its
// instruction count.  A product returns a proxy, and adding or subtracting
// the proxy emits one fused multiply-add, so the same `a * b + c` expressions
// that the scalar code compiles to FFMA compile to FFMA2 here.  Division and
// reciprocal are per lane (__fdividef, as in the scalar FAST float path).
#pragma once

#include <cuda_runtime.h>

namespace weno {
namespace px {

struct f32x2 {
  float2 v;
  __device__ __forceinline__ f32x2() : v(make_float2(0.f, 0.f)) {}
  __device__ __forceinline__ explicit f32x2(float2 x) : v(x) {}
  __device__ __forceinline__ f32x2(float a, float b) : v(make_float2(a, b)) {}
  // broadcast of a constant (the generic code writes T(0.5), T(kC43), ...)
  __device__ __forceinline__ f32x2(double c) : v(make_float2((float)c, (float)c)) {}
  __device__ __forceinline__ f32x2(float c) : v(make_float2(c, c)) {}
  __device__ __forceinline__ f32x2(int c) : v(make_float2((float)c, (float)c)) {}
};

struct f32x2_prod {
  float2 a, b;
  __device__ __forceinline__ operator f32x2() const { return f32x2(__fmul2_rn(a, b)); }
};

__device__ __forceinline__ float2 neg2(float2 x) { return make_float2(-x.x, -x.y); }
__device__ __forceinline__ float2 val(const f32x2_prod& p) { return __fmul2_rn(p.a, p.b); }

__device__ __forceinline__ f32x2 operator-(f32x2 a) { return f32x2(neg2(a.v)); }
__device__ __forceinline__ f32x2 operator+(f32x2 a, f32x2 b) { return f32x2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ f32x2 operator-(f32x2 a, f32x2 b) { return f32x2(__fadd2_rn(a.v, neg2(b.v))); }

__device__ __forceinline__ f32x2_prod operator*(f32x2 a, f32x2 b) { return f32x2_prod{a.v, b.v}; }
__device__ __forceinline__ f32x2_prod operator*(f32x2_prod p, f32x2 b) { return f32x2_prod{val(p), b.v}; }
__device__ __forceinline__ f32x2_prod operator*(f32x2 a, f32x2_prod p) { return f32x2_prod{a.v, val(p)}; }
__device__ __forceinline__ f32x2_prod operator*(f32x2_prod p, f32x2_prod q) { return f32x2_prod{val(p), val(q)}; }

__device__ __forceinline__ f32x2 operator+(f32x2_prod p, f32x2 c) { return f32x2(__ffma2_rn(p.a, p.b, c.v)); }
__device__ __forceinline__ f32x2 operator+(f32x2 c, f32x2_prod p) { return f32x2(__ffma2_rn(p.a, p.b, c.v)); }
__device__ __forceinline__ f32x2 operator+(f32x2_prod p, f32x2_prod q) { return f32x2(__ffma2_rn(p.a, p.b, val(q))); }
__device__ __forceinline__ f32x2 operator-(f32x2_prod p, f32x2 c) { return f32x2(__ffma2_rn(p.a, p.b, neg2(c.v))); }
__device__ __forceinline__ f32x2 operator-(f32x2 c, f32x2_prod p) { return f32x2(__ffma2_rn(neg2(p.a), p.b, c.v)); }
__device__ __forceinline__ f32x2 operator-(f32x2_prod p, f32x2_prod q) {
  return f32x2(__ffma2_rn(p.a, p.b, neg2(val(q))));
}
__device__ __forceinline__ f32x2 operator-(f32x2_prod p) { return f32x2(neg2(val(p))); }

// per-lane fast division and reciprocal (the scalar FAST float forms)
__device__ __forceinline__ f32x2 operator/(f32x2 a, f32x2 b) {
  return f32x2(__fdividef(a.v.x, b.v.x), __fdividef(a.v.y, b.v.y));
}

}  // namespace px
using px::f32x2;
}  // namespace weno
