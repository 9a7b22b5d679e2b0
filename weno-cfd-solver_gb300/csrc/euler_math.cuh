// Device arithmetic of the 2D Euler finite-volume residual.
//
// Every function follows the reference's Rust core (weno_ext/src/utils.rs,
// weno.rs, riemann.rs) and is templated on
//   T    -- double or float, the arithmetic type;
//   FAST -- false: the reference's operation order, so that a translation unit
//           compiled with --fmad=false reproduces the Rust IEEE-754 doubles bit
//           for bit; true: the same mathematics with fewer FP64 divisions
//           (shared reciprocals, a common-denominator form of the WENO weights)
//           and FMA contraction, checked against the oracle by tolerance.
//
// GB300 executes FP64 at 1/64 of the FP32 rate and a correctly rounded FP64
// divide costs about ten FMA slots, so the FAST forms are written to remove
// divides and square roots rather than memory traffic; the FP64 reciprocals
// and square roots that remain take the seeded Newton forms of fp64_fast.cuh
// (three and five FP64 operations, within 1-2 ulp).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "df64.cuh"
#include "f32x2.cuh"
#include "fp64_fast.cuh"

#ifndef WENO_TU_NS
#error "WENO_TU_NS names the translation unit's inline namespace (tu_exact or tu_fast)"
#endif

namespace weno {
// Each translation unit compiles its kernels into its own inline namespace, so
// the --fmad=false and --fmad=true builds of the same template never share a
// symbol (the linker would otherwise keep only one of them).
inline namespace WENO_TU_NS {

// utils.rs:3-6
constexpr double kEps = 1e-12;              // DEFAULT_EPS, RHO_MIN and P_MIN; also the default WENO epsilon
                                            // `weps` (weno.rs:223), which callers may change
constexpr double kSqrt3_12 = 0.1443375673;  // truncated literal, not sqrt(3)/12
// weno.rs:270 / weno.rs:292 (Gauss-point linear weights, 10 digits)
constexpr double kGqA0 = 0.1928406937, kGqA1 = 0.6111111111, kGqA2 = 0.1960481952;
constexpr double kC13 = 13.0 / 12.0;
// The non-linear weights d_k/(eps+b_k)^2 / sum are unchanged when every
// eps+b_k is multiplied by the same factor; the FAST forms use 4 (eps+b_k) =
// 4 eps + (13/3) D^2 + s^2, two fused multiply-adds per indicator.
constexpr double kC43 = 13.0 / 3.0;

// Arithmetic kinds: native double takes the common-denominator WENO form (its
// exponent range is ample); float and df64 (float exponent range) take the
// reciprocal form.
template <class T>
constexpr bool is_native_f64 = std::is_same<T, double>::value;
template <class T>
constexpr bool is_f32 = std::is_same<T, float>::value;

template <class T>
__device__ __forceinline__ T vmax(T a, T b) { return fmax(a, b); }
template <class T>
__device__ __forceinline__ T vmin(T a, T b) { return fmin(a, b); }
// a*b + c as one FMA where the type has one (the FAST forms that must round
// the same way in two kernels spell it out).
template <class T>
__device__ __forceinline__ T mul_add(T a, T b, T c) {
  if constexpr (is_native_f64<T> || is_f32<T>) return fma(a, b, c);
  else return a * b + c;
}

// Clamps and tests against a non-negative bound.  FAST native double reads the
// operands' bits as signed 64-bit integers: for non-negative doubles that order
// is the numeric order, and every value with the sign bit set (negatives, -0)
// reads below any non-negative bound, so the result is max(x, c) / x < c for
// every non-NaN x, on the integer pipe instead of an FP64 slot (GB300 issues
// FP64 compares and min/max at the FP64 rate).  A NaN x with the sign bit clear
// passes through where fmax would return the bound; NaN propagates through
// the neighbouring arithmetic either way.  Used by the fluxes and the Riemann
// solvers (pass 2); the pass-1 Roe average and limiter keep the FP64 forms:
// there the integer forms measured 1.6 % slower, at 5 resident CTAs per SM
// and equally when held to the FP64 build's 4.
template <class T, bool FAST>
__device__ __forceinline__ T cmax(T x, T c) {
  if constexpr (FAST && is_native_f64<T>) return __double_as_longlong(x) > __double_as_longlong(c) ? x : c;
  else return vmax(x, c);
}
template <class T, bool FAST>
__device__ __forceinline__ bool lt_bound(T x, T c) {
  if constexpr (FAST && is_native_f64<T>) return __double_as_longlong(x) < __double_as_longlong(c);
  else return x < c;
}
template <class T, bool FAST>
__device__ __forceinline__ bool gt_zero(T x) {
  if constexpr (FAST && is_native_f64<T>) return __double_as_longlong(x) > 0;
  else return x > T(0.0);
}

// a / b: the IEEE quotient except in FAST float (the SFU path) and FAST double
// (a times the three-FMA reciprocal of fp64_fast.cuh).
template <class T, bool FAST>
__device__ __forceinline__ T qdiv(T a, T b) {
  if constexpr (FAST && is_f32<T>) return __fdividef(a, b);
  else if constexpr (FAST && is_native_f64<T>) return a * f64fast::rcp(b);
  else return a / b;
}
template <class T, bool FAST>
__device__ __forceinline__ T qrcp(T b) {
  if constexpr (FAST && is_f32<T>) return __fdividef(1.0f, b);
  else if constexpr (FAST && is_native_f64<T>) return f64fast::rcp(b);
  else return T(1.0) / b;
}
template <class T, bool FAST>
__device__ __forceinline__ T qsqrt(T x) {
  if constexpr (FAST && is_native_f64<T>) return f64fast::sqrt(x);
  else return sqrt(x);
}
// 1/sqrt(x) of the FAST forms (x > 0): one reciprocal square root gives sqrt(x)
// = x * r and 1/x = r * r, replacing a square root and two divisions.  Double:
// fp64_fast.cuh (within 1 ulp); float: CUDA's rsqrtf (within 2 ulp); df64
// takes 1/sqrt.
template <class T>
__device__ __forceinline__ T frsqrt(T x) {
  if constexpr (is_native_f64<T>) return f64fast::rsqrt(x);
  else if constexpr (is_f32<T>) return rsqrtf(x);
  else return T(1.0) / sqrt(x);
}

// a*b + c*d with both products rounded on their own (never contracted into an
// FMA).  For mirror-image arguments (c*d = -(a*b) exactly) the sum is +0.0, as
// the reference's separately rounded products give; a fused form would leave
// the first product's rounding error, a tiny value of either sign.  Used where
// a sign decides a branch: the Roe-averaged normal velocity and the HLLC star
// speed at a reflecting wall, where the reference flux jumps from F_L to F_R as
// that sign changes (when the Roe sound speed is zero, e.g. a state whose
// energy has gone negative).
template <class T>
__device__ __forceinline__ T sum_prod_rn(T a, T b, T c, T d) {
  if constexpr (is_native_f64<T>) return __dadd_rn(__dmul_rn(a, b), __dmul_rn(c, d));
  else if constexpr (is_f32<T>) return __fadd_rn(__fmul_rn(a, b), __fmul_rn(c, d));
  else return a * b + c * d;
}

// ---------------------------------------------------------------------------
// Conserved state helpers (utils.rs:9-35, utils.rs:74-109)
// ---------------------------------------------------------------------------
// The kinetic energy term 0.5 rho (u^2 + v^2) of a pressure, with u = m/rho and
// v = n/rho for the (clamped) density rho: the reference's form, or in FAST the
// same quantity as 0.5 (m u + n v) (rho u = m), two operations fewer.
template <class T, bool FAST>
__device__ __forceinline__ T half_rho_speed2(T rho, T m, T n, T u, T v) {
  if constexpr (FAST) return T(0.5) * (m * u + n * v);
  else return T(0.5) * rho * (u * u + v * v);
}

// Euler flux normal to x (Y = false) or y (Y = true), utils.rs:74-109.  `rinv`
// (FAST only, when > 0) is 1/max(q[0], eps) computed by the caller.
template <class T, bool FAST, bool Y>
__device__ __forceinline__ void euler_flux(const T q[4], T gamma, T f[4], T rinv = T(0.0)) {
  const T rho = cmax<T, FAST>(q[0], T(kEps));
  T u, v;
  if constexpr (FAST) {
    const T r = gt_zero<T, FAST>(rinv) ? rinv : qrcp<T, FAST>(rho);
    u = q[1] * r;
    v = q[2] * r;
  } else {
    u = q[1] / rho;
    v = q[2] / rho;
  }
  const T p = (gamma - T(1.0)) * (q[3] - half_rho_speed2<T, FAST>(rho, q[1], q[2], u, v));
  if constexpr (!Y) {
    f[0] = q[1];
    f[1] = q[1] * u + p;
    f[2] = q[2] * u;
    f[3] = u * (q[3] + p);
  } else {
    f[0] = q[2];
    f[1] = q[1] * v;
    f[2] = q[2] * v + p;
    f[3] = v * (q[3] + p);
  }
}

// Two Euler fluxes (utils.rs:74-109).  FAST native double shares one division
// between the two densities: 1/(rho_a rho_b) (f64fast::rcp2, relative error
// below 2^-41), whose product stays in range for any clamped density below
// 1e150 (otherwise two divisions).
template <class T, bool FAST, bool Y>
__device__ __forceinline__ void euler_flux_pair(const T qa[4], const T qb[4], T gamma, T fa[4], T fb[4]) {
  if constexpr (FAST && is_native_f64<T>) {
    const T ra = cmax<T, FAST>(qa[0], T(kEps)), rb = cmax<T, FAST>(qb[0], T(kEps));
    const T prod = ra * rb;
    T ia, ib;
    if (lt_bound<T, FAST>(prod, T(1e300))) {
      const T inv = f64fast::rcp2(prod);
      ia = rb * inv;
      ib = ra * inv;
    } else {
      ia = f64fast::rcp(ra);
      ib = f64fast::rcp(rb);
    }
    euler_flux<T, FAST, Y>(qa, gamma, fa, ia);
    euler_flux<T, FAST, Y>(qb, gamma, fb, ib);
  } else {
    euler_flux<T, FAST, Y>(qa, gamma, fa);
    euler_flux<T, FAST, Y>(qb, gamma, fb);
  }
}

// utils.rs:9-35 con2primi_local for one cell.
template <class T, bool FAST>
__device__ __forceinline__ void con2prim(T q0, T q1, T q2, T q3, T gamma, T& p, T& a, T& rho, T& u, T& v, T& h) {
  rho = cmax<T, FAST>(q0, T(kEps));
  if constexpr (FAST) {
    const T r = qrcp<T, FAST>(rho);
    u = q1 * r;
    v = q2 * r;
    p = cmax<T, FAST>((gamma - T(1.0)) * (q3 - half_rho_speed2<T, FAST>(rho, q1, q2, u, v)), T(kEps));
    a = qsqrt<T, FAST>(gamma * p * r);
    h = (q3 + p) * r;
  } else {
    u = q1 / rho;
    v = q2 / rho;
    p = vmax((gamma - T(1.0)) * (q3 - T(0.5) * rho * (u * u + v * v)), T(kEps));
    a = sqrt(gamma * p / rho);
    h = (q3 + p) / rho;
  }
}

// Pressure of con2primi (clamped density and pressure) -- the quantity the
// shock sensor averages (riemann.rs:421-430).
template <class T, bool FAST>
__device__ __forceinline__ T clamped_pressure(const T q[4], T gamma) {
  const T rho = cmax<T, FAST>(q[0], T(kEps));
  T u, v;
  if constexpr (FAST) {
    const T r = qrcp<T, FAST>(rho);
    u = q[1] * r;
    v = q[2] * r;
  } else {
    u = q[1] / rho;
    v = q[2] / rho;
  }
  return cmax<T, FAST>((gamma - T(1.0)) * (q[3] - half_rho_speed2<T, FAST>(rho, q[1], q[2], u, v)), T(kEps));
}

// ---------------------------------------------------------------------------
// WENO5-JS (weno.rs:214-257) and the 2-point Gauss-quadrature pair
// (weno.rs:262-303).
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void js_betas(T u0, T u1, T u2, T u3, T u4, T& b0, T& b1, T& b2) {
  T t, s;
  t = u2 - T(2.0) * u3 + u4;
  s = T(3.0) * u2 - T(4.0) * u3 + u4;
  b0 = T(kC13) * (t * t) + T(0.25) * (s * s);
  t = u1 - T(2.0) * u2 + u3;
  s = u1 - u3;
  b1 = T(kC13) * (t * t) + T(0.25) * (s * s);
  t = u0 - T(2.0) * u1 + u2;
  s = u0 - T(4.0) * u1 + T(3.0) * u2;
  b2 = T(kC13) * (t * t) + T(0.25) * (s * s);
}

// Biased exponent of the largest of three positive doubles, from integer
// operations on the high words (no FP64 slot).
__device__ __forceinline__ int max_biased_exp3(double a, double b, double c) {
  const int ea = (__double2hiint(a) >> 20) & 0x7ff;
  const int eb = (__double2hiint(b) >> 20) & 0x7ff;
  const int ec = (__double2hiint(c) >> 20) & 0x7ff;
  return max(ea, max(eb, ec));
}

// Brings (eps + beta_k) into the range where the products of the
// common-denominator weights neither overflow nor lose the dominant weight.
// For a largest value within [2^-W, 2^W] (every practical stencil) nothing is
// done; otherwise all three are scaled by the same power of two that puts the
// largest into [0.5, 1) (exact).  NaN and infinity pass through.  W = 200 for
// the fourth-power products of the WENO5 weights, 120 for the Gauss-point
// pair, whose shared reciprocal takes an eighth-power product.
template <int W = 200>
__device__ __forceinline__ void weno_range(double& e0, double& e1, double& e2) {
  const int em = max_biased_exp3(e0, e1, e2);
  if (em >= 1023 - W && em <= 1023 + W) return;
  if (em == 0x7ff || em == 0) return;
  int b = 2045 - em;
  if (b < 1) b = 1;
  const double sc = __hiloint2double(b << 20, 0);
  e0 *= sc;
  e1 *= sc;
  e2 *= sc;
}

// Non-linear weighting of three candidate values with linear weights d.
// Exact: the reference's a_k = d_k/(eps+b_k)^2, w_k = a_k/sum.  FAST (float
// and df64, whose float exponent range rules out products of fourth powers):
// reciprocals.  FAST native double uses weno_nd instead.
template <class T, bool FAST>
__device__ __forceinline__ T weno_combine(T e0, T e1, T e2, T d0, T d1, T d2, T p0, T p1, T p2, T scale) {
  if constexpr (!FAST) {
    const T a0 = d0 / (e0 * e0);
    const T a1 = d1 / (e1 * e1);
    const T a2 = d2 / (e2 * e2);
    const T sum = a0 + a1 + a2;
    const T w0 = a0 / sum, w1 = a1 / sum, w2 = a2 / sum;
    const T r = w0 * p0 + w1 * p1 + w2 * p2;
    return scale == T(1.0) ? r : r / scale;
  } else {
    static_assert(!is_native_f64<T>, "FAST double takes the common-denominator form (weno_nd)");
    const T a0 = d0 * qrcp<T, FAST>(e0 * e0);
    const T a1 = d1 * qrcp<T, FAST>(e1 * e1);
    const T a2 = d2 * qrcp<T, FAST>(e2 * e2);
    const T num = a0 * p0 + a1 * p1 + a2 * p2;
    return qdiv<T, FAST>(num, (a0 + a1 + a2) * scale);
  }
}

// FAST native double: the weights in a common-denominator form,
// d_k prod_{j != k} (eps+b_j)^2, returned as numerator and denominator so that
// a caller can share one divide between two reconstructions; the (eps+b_k)
// are first brought into a safe range (weno_range), so the products neither
// overflow nor lose the dominant weight whatever the magnitude of the values.
__device__ __forceinline__ void weno_nd_products(double e0, double e1, double e2, double& P0, double& P1,
                                                 double& P2) {
  weno_range(e0, e1, e2);
  const double s0 = e0 * e0, s1 = e1 * e1, s2 = e2 * e2;
  P0 = s1 * s2;
  P1 = s0 * s2;
  P2 = s0 * s1;
}
// Numerator and denominator of the weighted slope from the products, linear
// weights (3, 6, 1) (the reference's 0.3, 0.6, 0.1 scaled by 10), each
// operation spelled out: two reconstructions that share the products (the
// same three stencils seen from both sides of a cell) round exactly as two
// separate evaluations would.
__device__ __forceinline__ void weno_nd_combine(double P0, double P1, double P2, double g0, double g1, double g2,
                                                double& num, double& den) {
  const double c0 = 3.0 * P0, c1 = 6.0 * P1;
  num = fma(P2, g2, fma(c1, g1, c0 * g0));
  den = (c0 + c1) + P2;
}

// x = x0 + a/(k b) and y = y0 + c/(k d) with one divide, 1/(k b d), when b d is
// a normal number well inside the double range (tested on its exponent bits, no
// FP64 slot); otherwise two divides.
__device__ __forceinline__ void div_pair(double a, double b, double c, double d, double& x, double& y,
                                         double k = 1.0, double x0 = 0.0, double y0 = 0.0) {
  const double bd = b * d;
  const int e = (__double2hiint(bd) >> 20) & 0x7ff;
  if (e > 64 && e < 1983) {
    const double inv = f64fast::rcp2(bd * k);  // scales the slopes only
    x = fma(a * d, inv, x0);
    y = fma(c * b, inv, y0);
  } else {
    x = x0 + a / (b * k);
    y = y0 + c / (d * k);
  }
}

// weno.rs:214-233 (left-biased, value at the right face of u2)
template <class T, bool FAST>
__device__ __forceinline__ T weno5_left(T u0, T u1, T u2, T u3, T u4, T weps) {
  T b0, b1, b2;
  js_betas(u0, u1, u2, u3, u4, b0, b1, b2);
  const T p0 = -u4 + T(5.0) * u3 + T(2.0) * u2;
  const T p1 = -u1 + T(5.0) * u2 + T(2.0) * u3;
  const T p2 = T(2.0) * u0 - T(7.0) * u1 + T(11.0) * u2;
  return weno_combine<T, FAST>(weps + b0, weps + b1, weps + b2, T(0.3), T(0.6), T(0.1), p0, p1, p2, T(6.0));
}

// weno.rs:238-257 (right-biased, value at the left face of u3)
template <class T, bool FAST>
__device__ __forceinline__ T weno5_right(T u1, T u2, T u3, T u4, T u5, T weps) {
  T b0, b1, b2;
  T t, s;
  t = u3 - T(2.0) * u4 + u5;
  s = T(3.0) * u3 - T(4.0) * u4 + u5;
  b0 = T(kC13) * (t * t) + T(0.25) * (s * s);
  t = u2 - T(2.0) * u3 + u4;
  s = u2 - u4;
  b1 = T(kC13) * (t * t) + T(0.25) * (s * s);
  t = u1 - T(2.0) * u2 + u3;
  s = u1 - T(4.0) * u2 + T(3.0) * u3;
  b2 = T(kC13) * (t * t) + T(0.25) * (s * s);
  const T p0 = T(2.0) * u5 - T(7.0) * u4 + T(11.0) * u3;
  const T p1 = -u4 + T(5.0) * u3 + T(2.0) * u2;
  const T p2 = -u1 + T(5.0) * u2 + T(2.0) * u3;
  return weno_combine<T, FAST>(weps + b0, weps + b1, weps + b2, T(0.1), T(0.6), T(0.3), p0, p1, p2, T(6.0));
}

// weno5_left and weno5_right of one field at one face (the right stencil is
// the left one shifted by a cell), FAST: native double shares one divide
// between the two; float and df64 take reciprocal weights.
template <class T>
__device__ __forceinline__ void weno5_lr_fast(T u0, T u1, T u2, T u3, T u4, T u5, T weps, T& left, T& right) {
  // first differences d_m = u_{m+1} - u_m, second differences D_m = d_m - d_{m-1}
  // (centred on u_m), shared by the two stencils; each Jiang-Shu indicator is
  // 13/12 D^2 + 1/4 s^2 with s a combination of two first differences.
  const T d0 = u1 - u0, d1 = u2 - u1, d2 = u3 - u2, d3 = u4 - u3, d4 = u5 - u4;
  const T D1 = d1 - d0, D2 = d2 - d1, D3 = d3 - d2, D4 = d4 - d3;
  // indicators scaled by 4 (see kC43): 4 eps + (13/3) D^2 + s^2
  const T w4 = T(4.0) * weps;
  const T C1 = T(kC43) * D1 * D1 + w4, C2 = T(kC43) * D2 * D2 + w4, C3 = T(kC43) * D3 * D3 + w4,
          C4 = T(kC43) * D4 * D4 + w4;
  const T sl0 = d3 - T(3.0) * d2, sl1 = d1 + d2, sl2 = T(3.0) * d1 - d0;  // left:  stencils 2-4, 1-3, 0-2
  const T sr0 = d4 - T(3.0) * d3, sr1 = d2 + d3, sr2 = T(3.0) * d2 - d1;  // right: stencils 3-5, 2-4, 1-3
  const T el0 = sl0 * sl0 + C3, el1 = sl1 * sl1 + C2, el2 = sl2 * sl2 + C1;
  const T er0 = sr0 * sr0 + C4, er1 = sr1 * sr1 + C3, er2 = sr2 * sr2 + C2;
  // Candidate polynomials (x6) less six times the centre value, from the same
  // differences: left 6 u2 + (4 d2 - d3, d1 + 2 d2, 5 d1 - 2 d0), right 6 u3 +
  // (d1 - 4 d2, -(2 d2 + d3), 2 d4 - 5 d3); each face state is its centre value
  // plus the weighted slope / 6 (no 6 u2 formed and cancelled).
  const T gl0 = d2 - sl0, gl1 = sl1 + d2, gl2 = T(2.0) * sl2 - d1;
  const T gr2 = -d2 - sr2, gr1 = -d2 - sr1, gr0 = T(2.0) * sr0 + d3;
  // The right reconstruction takes its stencils in the mirror order of the left
  // one (1-3, 2-4, 3-5 against 2-4, 1-3, 0-2), so that for mirror-image inputs
  // (u_k -> u_{5-k}, as across a reflecting wall: d_m -> -d_{4-m}) it performs
  // the left one's operations on bit-identical values and the two face states
  // are exact mirrors, as in the reference's arithmetic.
  if constexpr (is_native_f64<T>) {
    // linear weights scaled by 10 -- (3, 6, 1) -- and the 1/6 of the candidate
    // polynomials applied once to the shared divide
    double P0, P1, P2, nl, dl, nr, dr;
    weno_nd_products(el0, el1, el2, P0, P1, P2);
    weno_nd_combine(P0, P1, P2, gl0, gl1, gl2, nl, dl);
    weno_nd_products(er2, er1, er0, P0, P1, P2);
    weno_nd_combine(P0, P1, P2, gr2, gr1, gr0, nr, dr);
    div_pair(nl, dl, nr, dr, left, right, 6.0, u2, u3);
  } else {
    left = u2 + weno_combine<T, true>(el0, el1, el2, T(0.3), T(0.6), T(0.1), gl0, gl1, gl2, T(6.0));
    right = u3 + weno_combine<T, true>(er2, er1, er0, T(0.3), T(0.6), T(0.1), gr2, gr1, gr0, T(6.0));
  }
}

// weno5_lr_fast of two neighbouring faces of one field (A between u2 and u3,
// B between u3 and u4; FAST native double), sharing what the two faces have in
// common: the differences, and -- since A's right state and B's left state are
// both reconstructions about cell u3 from the stencils 1-3, 2-4, 3-5 -- their
// indicators and weight products.  Every shared value is computed with the
// operations weno5_lr_fast performs for each face on its own, so A and B get
// the bits of two separate calls (the component-wise pass 1 of the FAST
// double solver).
__device__ __forceinline__ void weno5_lr_fast_two(double u0, double u1, double u2, double u3, double u4, double u5,
                                                  double u6, double weps, double& lA, double& rA, double& lB,
                                                  double& rB) {
  const double d0 = u1 - u0, d1 = u2 - u1, d2 = u3 - u2, d3 = u4 - u3, d4 = u5 - u4, d5 = u6 - u5;
  const double D1 = d1 - d0, D2 = d2 - d1, D3 = d3 - d2, D4 = d4 - d3, D5 = d5 - d4;
  const double w4 = 4.0 * weps;
  const double C1 = kC43 * D1 * D1 + w4, C2 = kC43 * D2 * D2 + w4, C3 = kC43 * D3 * D3 + w4,
               C4 = kC43 * D4 * D4 + w4, C5 = kC43 * D5 * D5 + w4;
  // face A: as weno5_lr_fast(u0..u5)
  const double sl0 = d3 - 3.0 * d2, sl1 = d1 + d2, sl2 = 3.0 * d1 - d0;
  const double sr0 = d4 - 3.0 * d3, sr1 = d2 + d3, sr2 = 3.0 * d2 - d1;
  const double el0 = sl0 * sl0 + C3, el1 = sl1 * sl1 + C2, el2 = sl2 * sl2 + C1;
  const double er0 = sr0 * sr0 + C4, er1 = sr1 * sr1 + C3, er2 = sr2 * sr2 + C2;
  const double gl0 = d2 - sl0, gl1 = sl1 + d2, gl2 = 2.0 * sl2 - d1;
  const double gr2 = -d2 - sr2, gr1 = -d2 - sr1, gr0 = 2.0 * sr0 + d3;
  // face B: as weno5_lr_fast(u1..u6); its left stencils and indicators are A's right ones
  const double tr0 = d5 - 3.0 * d4, tr1 = d3 + d4, tr2 = 3.0 * d3 - d2;
  const double fr0 = tr0 * tr0 + C5, fr1 = tr1 * tr1 + C4, fr2 = tr2 * tr2 + C3;
  const double hl0 = d3 - sr0, hl1 = sr1 + d3, hl2 = 2.0 * sr2 - d2;
  const double hr2 = -d3 - tr2, hr1 = -d3 - tr1, hr0 = 2.0 * tr0 + d4;
  double P0, P1, P2, nl, dl, nr, dr;
  weno_nd_products(el0, el1, el2, P0, P1, P2);
  weno_nd_combine(P0, P1, P2, gl0, gl1, gl2, nl, dl);
  weno_nd_products(er2, er1, er0, P0, P1, P2);
  weno_nd_combine(P0, P1, P2, gr2, gr1, gr0, nr, dr);
  div_pair(nl, dl, nr, dr, lA, rA, 6.0, u2, u3);
  // B's left from the same products in the other order (products commute)
  weno_nd_combine(P2, P1, P0, hl0, hl1, hl2, nl, dl);
  weno_nd_products(fr2, fr1, fr0, P0, P1, P2);
  weno_nd_combine(P0, P1, P2, hr2, hr1, hr0, nr, dr);
  div_pair(nl, dl, nr, dr, lB, rB, 6.0, u3, u4);
}

// FAST float: the four fields' left/right reconstructions as two packed pairs
// (fields 0,1 and 2,3) on the FP32x2 instructions; field 2 takes weps2.
__device__ __forceinline__ void weno5_lr_fast_f32_pairs(const float c[6][4], float weps, float left[4],
                                                        float right[4], float weps2) {
#pragma unroll
  for (int f = 0; f < 4; f += 2) {
    f32x2 l, r;
    weno5_lr_fast<f32x2>(f32x2(c[0][f], c[0][f + 1]), f32x2(c[1][f], c[1][f + 1]), f32x2(c[2][f], c[2][f + 1]),
                         f32x2(c[3][f], c[3][f + 1]), f32x2(c[4][f], c[4][f + 1]), f32x2(c[5][f], c[5][f + 1]),
                         f == 0 ? f32x2(weps) : f32x2(weps2, weps), l, r);
    left[f] = l.v.x;
    left[f + 1] = l.v.y;
    right[f] = r.v.x;
    right[f + 1] = r.v.y;
  }
}

// weno.rs:262-303: both Gauss-point values from one 5-cell stencil.  The
// smoothness indicators are shared (the reference recomputes identical values).
// FAST Gauss-point pair from the centre value, the slopes h_k of the three
// candidate polynomials and the (scaled) indicators f_k: native double in the
// common-denominator form, float and df64 with reciprocals.  The candidates
// are q2 +- S h_k, so each weighted value is q2 plus S times a weighted slope.
template <class T>
__device__ __forceinline__ void gq_weights(T q2, T h0, T h1, T h2, T f0, T f1, T f2, T& ra, T& rb) {
  const T S = T(kSqrt3_12);
  if constexpr (is_native_f64<T>) {
    weno_range<120>(f0, f1, f2);
    const double s0 = f0 * f0, s1 = f1 * f1, s2 = f2 * f2;
    const double P0 = s1 * s2, P1 = s0 * s2, P2 = s0 * s1;
    // linear weights divided by the centre one (a common factor): point a
    // weighs (r0 P0, P1, r2 P2), point b the mirror (r2 P0, P1, r0 P2)
    constexpr double r0 = kGqA0 / kGqA1, r2 = kGqA2 / kGqA1;
    const double u0 = P0 * h0, u1 = P1 * h1, u2 = P2 * h2;
    const double sa = fma(r0, P0, fma(r2, P2, P1)), sb = fma(r2, P0, fma(r0, P2, P1));
    const double t = S * f64fast::rcp2(sa * sb);  // scales the weighted slopes only
    // point a: candidates (q2 + S h0, q2 - S h1, q2 - S h2); point b: the mirror
    ra = fma(r0, u0, fma(-r2, u2, -u1)) * (sb * t) + q2;
    rb = fma(r0, u2, fma(-r2, u0, u1)) * (sa * t) + q2;
  } else {
    const T r0 = qrcp<T, true>(f0 * f0), r1 = qrcp<T, true>(f1 * f1), r2 = qrcp<T, true>(f2 * f2);
    const T ca0 = T(kGqA0 / kGqA1) * r0, ca1 = r1, ca2 = T(kGqA2 / kGqA1) * r2;
    const T cb0 = T(kGqA2 / kGqA1) * r0, cb2 = T(kGqA0 / kGqA1) * r2;
    ra = qdiv<T, true>((ca0 * h0 - ca1 * h1 - ca2 * h2) * S, ca0 + ca1 + ca2) + q2;
    rb = qdiv<T, true>((ca1 * h1 + cb2 * h2 - cb0 * h0) * S, cb0 + ca1 + cb2) + q2;
  }
}

// Two neighbouring 5-cell stencils (q0..q4 and q1..q5), FAST: both
// Gauss-point pairs, sharing the first and second differences.
template <class T>
__device__ __forceinline__ void weno5_gq_two(T q0, T q1, T q2, T q3, T q4, T q5, T weps, T& raA, T& rbA, T& raB,
                                             T& rbB) {
  const T d0 = q1 - q0, d1 = q2 - q1, d2 = q3 - q2, d3 = q4 - q3, d4 = q5 - q4;
  const T D1 = d1 - d0, D2 = d2 - d1, D3 = d3 - d2, D4 = d4 - d3;
  const T w4 = T(4.0) * weps;
  const T C1 = T(kC43) * D1 * D1 + w4, C2 = T(kC43) * D2 * D2 + w4, C3 = T(kC43) * D3 * D3 + w4,
          C4 = T(kC43) * D4 * D4 + w4;
  const T hA0 = d3 - T(3.0) * d2, hA1 = d1 + d2, hA2 = T(3.0) * d1 - d0;
  const T hB0 = d4 - T(3.0) * d3, hB1 = d2 + d3, hB2 = T(3.0) * d2 - d1;
  gq_weights<T>(q2, hA0, hA1, hA2, hA0 * hA0 + C3, hA1 * hA1 + C2, hA2 * hA2 + C1, raA, rbA);
  gq_weights<T>(q3, hB0, hB1, hB2, hB0 * hB0 + C4, hB1 * hB1 + C3, hB2 * hB2 + C2, raB, rbB);
}

template <class T, bool FAST>
__device__ __forceinline__ void weno5_gq_pair(T q0, T q1, T q2, T q3, T q4, T& ra, T& rb, T weps) {
  const T S = T(kSqrt3_12);
  if constexpr (FAST) {
    // difference form (as in weno5_lr_fast): the one-sided indicator terms are
    // the polynomial slopes g0, g2 and the centred one is g1/S
    const T d0 = q1 - q0, d1 = q2 - q1, d2 = q3 - q2, d3 = q4 - q3;
    const T D1 = d1 - d0, D2 = d2 - d1, D3 = d3 - d2;
    const T h0 = d3 - T(3.0) * d2;  // 3 q2 - 4 q3 + q4
    const T h1 = d1 + d2;           // q3 - q1
    const T h2 = T(3.0) * d1 - d0;  // 3 q2 - 4 q1 + q0
    // indicators scaled by 4 (see kC43): 4 eps + (13/3) D^2 + h^2
    const T w4 = T(4.0) * weps;
    const T f0 = h0 * h0 + (T(kC43) * D3 * D3 + w4);
    const T f1 = h1 * h1 + (T(kC43) * D2 * D2 + w4);
    const T f2 = h2 * h2 + (T(kC43) * D1 * D1 + w4);
    gq_weights<T>(q2, h0, h1, h2, f0, f1, f2, ra, rb);
  } else {
    T b0, b1, b2;
    js_betas(q0, q1, q2, q3, q4, b0, b1, b2);
    const T e0 = weps + b0, e1 = weps + b1, e2 = weps + b2;
    const T g0 = T(3.0) * q2 - T(4.0) * q3 + q4;
    const T g2 = T(3.0) * q2 - T(4.0) * q1 + q0;
    const T pa0 = q2 + g0 * S;
    const T pa1 = q2 - (-q1 + q3) * S;
    const T pa2 = q2 - g2 * S;
    ra = weno_combine<T, FAST>(e0, e1, e2, T(kGqA0), T(kGqA1), T(kGqA2), pa0, pa1, pa2, T(1.0));
    const T pb0 = q2 - g0 * S;
    const T pb1 = q2 - (q1 - q3) * S;
    const T pb2 = q2 + g2 * S;
    rb = weno_combine<T, FAST>(e0, e1, e2, T(kGqA2), T(kGqA1), T(kGqA0), pb0, pb1, pb2, T(1.0));
  }
}

// ---------------------------------------------------------------------------
// Characteristic projection (weno.rs:13-205)
// ---------------------------------------------------------------------------
// FAST Roe-average inputs of one cell: with r = 1/sqrt(rho) (one reciprocal
// square root), sqrt(rho) = rho r, 1/rho = r r, sqrt(rho) u = m r and
// sqrt(rho) v = n r; E + p with the clamped pressure.
template <class T>
struct RoeSide {
  T sq, r, i, a, b, ep;  // sqrt(rho), 1/sqrt(rho), 1/rho, m r, n r, E + p
};

template <class T>
__device__ __forceinline__ RoeSide<T> roe_side(const T u[4], T gamma) {
  RoeSide<T> s;
  const T rho = vmax(u[0], T(kEps));
  s.r = frsqrt(rho);
  s.sq = rho * s.r;
  s.i = s.r * s.r;
  // kinetic energy (m^2 + n^2) / (2 rho): the velocities themselves are not needed
  const T p = vmax((gamma - T(1.0)) * (u[3] - T(0.5) * ((u[1] * u[1] + u[2] * u[2]) * s.i)), T(kEps));
  s.a = u[1] * s.r;
  s.b = u[2] * s.r;
  s.ep = u[3] + p;
  return s;
}

// Roe average of the face between sides L and R (weno.rs:13-52), FAST: m_l,
// n_l are the left cell's momenta.  Also returns 1/c_roe and 1/rho_roe (ic,
// irho) for the eigenvectors; 1/rho_roe = r_l r_r.
template <class T>
__device__ __forceinline__ void roe_face(const RoeSide<T>& L, const RoeSide<T>& R, T m_l, T n_l, T gamma,
                                         T& rho_roe, T& u_roe, T& v_roe, T& h_roe, T& c_roe, T& ic, T& irho) {
  const T id = qrcp<T, true>(L.sq + R.sq);
  u_roe = mul_add(m_l, L.r, R.a) * id;
  v_roe = mul_add(n_l, L.r, R.b) * id;
  h_roe = mul_add(L.ep, L.r, R.ep * R.r) * id;
  const T kin = T(0.5) * (u_roe * u_roe + v_roe * v_roe);
  const T c2 = vmax((gamma - T(1.0)) * (h_roe - kin), T(kEps) * vmax(L.i, R.i));
  ic = frsqrt(c2);
  c_roe = c2 * ic;
  rho_roe = L.sq * R.sq;
  irho = L.r * R.r;
}

// Roe average of two conserved cells, weno.rs:13-52 (FAST: roe_side and
// roe_face, two reciprocal square roots, one divide and one more reciprocal
// square root for c).
template <class T, bool FAST>
__device__ __forceinline__ void roe_avg(const T ul[4], const T ur[4], T gamma, T& rho_roe, T& u_roe, T& v_roe,
                                        T& h_roe, T& c_roe, T& ic, T& irho) {
  if constexpr (FAST) {
    roe_face(roe_side(ul, gamma), roe_side(ur, gamma), ul[1], ul[2], gamma, rho_roe, u_roe, v_roe, h_roe, c_roe, ic,
             irho);
  } else {
    (void)ic;
    (void)irho;
    const T rho_l = vmax(ul[0], T(kEps));
    const T rho_r = vmax(ur[0], T(kEps));
    const T sqrt_l = sqrt(rho_l);
    const T sqrt_r = sqrt(rho_r);
    const T denom = sqrt_l + sqrt_r;
    const T u_l = ul[1] / rho_l, v_l = ul[2] / rho_l;
    const T u_r = ur[1] / rho_r, v_r = ur[2] / rho_r;
    const T p_l = vmax((gamma - T(1.0)) * (ul[3] - T(0.5) * rho_l * (u_l * u_l + v_l * v_l)), T(kEps));
    const T p_r = vmax((gamma - T(1.0)) * (ur[3] - T(0.5) * rho_r * (u_r * u_r + v_r * v_r)), T(kEps));
    const T h_l = (ul[3] + p_l) / rho_l;
    const T h_r = (ur[3] + p_r) / rho_r;
    u_roe = (sqrt_l * u_l + sqrt_r * u_r) / denom;
    v_roe = (sqrt_l * v_l + sqrt_r * v_r) / denom;
    h_roe = (sqrt_l * h_l + sqrt_r * h_r) / denom;
    const T kin = T(0.5) * (u_roe * u_roe + v_roe * v_roe);
    const T c2 = vmax((gamma - T(1.0)) * (h_roe - kin), T(kEps) / vmin(rho_l, rho_r));
    c_roe = sqrt(c2);
    rho_roe = sqrt_l * sqrt_r;
  }
}

// Left eigenvectors, weno.rs:76-107 (x) and weno.rs:136-167 (y), in the
// reference's operation order (FAST callers use CharScalars / project_left).
template <class T, bool Y>
__device__ __forceinline__ void left_eig(T rho, T u, T v, T c, T gamma, T L[4][4]) {
  const T g1 = gamma - T(1.0);
  const T kin = T(0.5) * (u * u + v * v);
  const T vn = Y ? v : u;
  const T rc = rho * c;
  const T inv_rc = T(1.0) / rc;
  const T inv_c2 = T(1.0) / (c * c);
  const T a = g1 * kin / (T(2.0) * c * c);
  const T b = vn / (T(2.0) * c);
  const T gu = -g1 * u * inv_c2 / T(2.0);
  const T gv = -g1 * v * inv_c2 / T(2.0);
  const T gg = g1 * inv_c2 / T(2.0);
  const T hr = T(0.5) * inv_rc;
  L[0][0] = a + b;
  L[3][0] = a - b;
  if constexpr (!Y) {
    L[0][1] = gu - hr; L[0][2] = gv; L[0][3] = gg;
    L[3][1] = gu + hr; L[3][2] = gv; L[3][3] = gg;
    L[2][0] = -v / rho; L[2][1] = T(0.0); L[2][2] = T(1.0) / rho; L[2][3] = T(0.0);
  } else {
    L[0][1] = gu; L[0][2] = gv - hr; L[0][3] = gg;
    L[3][1] = gu; L[3][2] = gv + hr; L[3][3] = gg;
    L[2][0] = -u / rho; L[2][1] = T(1.0) / rho; L[2][2] = T(0.0); L[2][3] = T(0.0);
  }
  L[1][0] = T(1.0) - g1 * kin * inv_c2;
  L[1][1] = g1 * u * inv_c2;
  L[1][2] = g1 * v * inv_c2;
  L[1][3] = -g1 * inv_c2;
}

// Right eigenvectors, weno.rs:113-131 (x) and weno.rs:171-189 (y).
template <class T, bool Y>
__device__ __forceinline__ void right_eig(T rho, T u, T v, T h, T c, T R[4][4]) {
  const T kin = T(0.5) * (u * u + v * v);
  R[0][0] = T(1.0); R[0][1] = T(1.0); R[0][2] = T(0.0); R[0][3] = T(1.0);
  if constexpr (!Y) {
    R[1][0] = u - c; R[1][1] = u; R[1][2] = T(0.0); R[1][3] = u + c;
    R[2][0] = v; R[2][1] = v; R[2][2] = rho; R[2][3] = v;
    R[3][0] = h - u * c; R[3][1] = kin; R[3][2] = rho * v; R[3][3] = h + u * c;
  } else {
    R[1][0] = u; R[1][1] = u; R[1][2] = rho; R[1][3] = u;
    R[2][0] = v - c; R[2][1] = v; R[2][2] = T(0.0); R[2][3] = v + c;
    R[3][0] = h - v * c; R[3][1] = kin; R[3][2] = rho * u; R[3][3] = h + v * c;
  }
}

// weno.rs:197-205 mat4_vec4: every product accumulated from 0.0 in column
// order, as the reference does (FAST callers use project_left / project_right).
template <class T>
__device__ __forceinline__ void mat4_vec4(const T M[4][4], const T x[4], T out[4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    T acc = T(0.0);
#pragma unroll
    for (int c = 0; c < 4; ++c) acc = acc + M[r][c] * x[c];
    out[r] = acc;
  }
}

// FAST products with the eigenvector matrices of weno.rs:76-189, written from
// their structure instead of a 4x4 product.  With G = (gamma-1)/c^2,
// kin = (u^2+v^2)/2, b = u_n/(2c), hr = 1/(2 rho c) and Z = kin q0 - u q1 - v q2 + q3:
//   L q = ( G Z/2 + (b q0 - hr q_n),  q0 - G Z,  (q_t - u_t q0)/rho,  G Z/2 - (b q0 - hr q_n) )
// (n the normal and t the tangential momentum index), and with s = w0+w1+w3:
//   R w = ( s,  u s + [c (w3-w0) | rho w2],  v s + [rho w2 | c (w3-w0)],  R3 . w ).
// The shear field is carried as rho w2 = q_t - u_t q0: WENO5 is homogeneous
// when its epsilon scales with the square of the field (the indicators are
// quadratic, the candidates linear), so reconstructing rho w2 with
// eps rho^2 gives rho times the reconstruction of w2, which is what R needs;
// the 1/rho of L and the rho of R drop out.
template <class T>
struct CharScalars {
  T u, v, c, rho, kin, G, G2, b, hr, h;
};

template <class T, bool Y>
__device__ __forceinline__ void project_left(const CharScalars<T>& k, const T q[4], T w[4]) {
  // Z from q3 upwards and G Z / 2 +- Yv as one FMA each: nine operations
  const T Z = (k.kin * q[0] + q[3]) - k.u * q[1] - k.v * q[2];
  const T Yv = k.b * q[0] - k.hr * q[Y ? 2 : 1];
  w[0] = k.G2 * Z + Yv;
  w[1] = q[0] - k.G * Z;
  w[2] = q[Y ? 1 : 2] - (Y ? k.u : k.v) * q[0];  // rho w2
  w[3] = k.G2 * Z - Yv;
}
template <class T, bool Y>
__device__ __forceinline__ void project_right(const CharScalars<T>& k, const T w[4], T out[4]) {
  const T s = w[0] + w[1] + w[3];
  const T d = w[3] - w[0];
  const T un = Y ? k.v : k.u;
  out[0] = s;
  if constexpr (!Y) {
    out[1] = k.u * s + k.c * d;
    out[2] = k.v * s + w[2];
  } else {
    out[1] = k.u * s + w[2];
    out[2] = k.v * s + k.c * d;
  }
  out[3] = (k.h - un * k.c) * w[0] + k.kin * w[1] + (Y ? k.u : k.v) * w[2] + (k.h + un * k.c) * w[3];
}

// weno.rs:312-315 pressure ; weno.rs:327-352 Zhang-Shu limiter toward `ub`.
template <class T, bool FAST>
__device__ __forceinline__ T pp_pressure(const T q[4], T gamma) {
  if (q[0] <= T(0.0)) return T(0.0);
  return (gamma - T(1.0)) * (q[3] - qdiv<T, FAST>(T(0.5) * (q[1] * q[1] + q[2] * q[2]), q[0]));
}
template <class T, bool FAST>
__device__ __forceinline__ void pp_limit(T q[4], const T ub[4], T gamma) {
  if (q[0] < T(kEps)) {
    const T rho_bar = vmax(ub[0], T(kEps));
    const T theta = vmax(vmin(qdiv<T, FAST>(rho_bar - T(kEps), rho_bar - q[0]), T(1.0)), T(0.0));
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] = theta * (q[k] - ub[k]) + ub[k];
  }
  if constexpr (FAST) {
    // p < eps  <=>  (gamma-1)(E rho - |m|^2/2) < eps rho for rho > 0 (pp_pressure
    // is 0 for rho <= 0): the divide is only needed when the limiter acts.
    if (q[0] > T(0.0) &&
        !((gamma - T(1.0)) * (q[3] * q[0] - T(0.5) * (q[1] * q[1] + q[2] * q[2])) < T(kEps) * q[0]))
      return;
  }
  const T p_q = pp_pressure<T, FAST>(q, gamma);
  if (p_q < T(kEps)) {
    const T p_bar = vmax(pp_pressure<T, FAST>(ub, gamma), T(kEps));
    const T theta = vmax(vmin(qdiv<T, FAST>(p_bar - T(kEps), p_bar - p_q), T(1.0)), T(0.0));
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] = theta * (q[k] - ub[k]) + ub[k];
  }
}

// ---------------------------------------------------------------------------
// Pass 1: normal-direction reconstruction of the two states at the interface
// between stencil cells 2 and 3 (weno.rs:390-454 characteristic,
// weno.rs:654-717 component-wise).  c[0..5] are the six cells along the normal.
// ---------------------------------------------------------------------------
template <class T, bool FAST, bool Y, bool CHAR>
__device__ __forceinline__ void pass1_face(const T c[6][4], T gamma, T ql[4], T qr[4], T weps) {
  if constexpr (!CHAR && FAST && is_f32<T>) {
    weno5_lr_fast_f32_pairs(c, weps, ql, qr, weps);
  } else if constexpr (!CHAR) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if constexpr (FAST) {
        weno5_lr_fast<T>(c[0][k], c[1][k], c[2][k], c[3][k], c[4][k], c[5][k], weps, ql[k], qr[k]);
      } else {
        ql[k] = weno5_left<T, FAST>(c[0][k], c[1][k], c[2][k], c[3][k], c[4][k], weps);
        qr[k] = weno5_right<T, FAST>(c[1][k], c[2][k], c[3][k], c[4][k], c[5][k], weps);
      }
    }
  } else {
    T rho_a, u_a, v_a, h_a, c_a, ic_a = T(0.0), irho_a = T(0.0);
    roe_avg<T, FAST>(c[2], c[3], gamma, rho_a, u_a, v_a, h_a, c_a, ic_a, irho_a);
    // The reference projects cells 0..4 for the left state and 1..5 for the
    // right state with the same matrix (both faces use the Roe average of
    // cells 2|3), so six projections cover both.
    T w[6][4];
    T chl[4], chr[4];
    if constexpr (FAST) {
      CharScalars<T> k;
      k.u = u_a;
      k.v = v_a;
      k.c = c_a;
      k.rho = rho_a;
      k.h = h_a;
      k.kin = T(0.5) * (u_a * u_a + v_a * v_a);
      k.G = (gamma - T(1.0)) * (ic_a * ic_a);
      k.G2 = T(0.5) * k.G;
      const T ich = T(0.5) * ic_a;
      k.b = (Y ? v_a : u_a) * ich;
      k.hr = ich * irho_a;
#pragma unroll
      for (int s = 0; s < 6; ++s) project_left<T, Y>(k, c[s], w[s]);
      const T weps2 = weps * (rho_a * rho_a);  // epsilon of the shear field rho w2
      if constexpr (is_f32<T>) {
        weno5_lr_fast_f32_pairs(w, weps, chl, chr, weps2);
      } else {
#pragma unroll
        for (int f = 0; f < 4; ++f)
          weno5_lr_fast<T>(w[0][f], w[1][f], w[2][f], w[3][f], w[4][f], w[5][f], f == 2 ? weps2 : weps, chl[f],
                           chr[f]);
      }
      project_right<T, Y>(k, chl, ql);
      project_right<T, Y>(k, chr, qr);
    } else {
      T Lm[4][4];
      left_eig<T, Y>(rho_a, u_a, v_a, c_a, gamma, Lm);
#pragma unroll
      for (int s = 0; s < 6; ++s) mat4_vec4<T>(Lm, c[s], w[s]);
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        chl[f] = weno5_left<T, FAST>(w[0][f], w[1][f], w[2][f], w[3][f], w[4][f], weps);
        chr[f] = weno5_right<T, FAST>(w[1][f], w[2][f], w[3][f], w[4][f], w[5][f], weps);
      }
      T Rm[4][4];
      right_eig<T, Y>(rho_a, u_a, v_a, h_a, c_a, Rm);
      mat4_vec4<T>(Rm, chl, ql);
      mat4_vec4<T>(Rm, chr, qr);
    }
    pp_limit<T, FAST>(ql, c[2], gamma);
    pp_limit<T, FAST>(qr, c[3], gamma);
  }
}

// ---------------------------------------------------------------------------
// Interface Riemann solvers (riemann.rs:6-349).  Inputs are the face-averaged
// states and fluxes; `ql`/`qr` are the raw (unclamped) states.
// ---------------------------------------------------------------------------
template <class T, bool FAST, bool Y>
struct RiemannPre {
  T ql0, qr0, u_l, v_l, u_r, v_r, p_l, p_r, s_l, s_r, un_l, un_r;
};

// S = 2 (FAST): ql, qr are twice the face states (the sums of the two Gauss-point
// values, which saves the halving multiplies); the clamps then take 2 eps, so
// densities and pressures are exactly twice the clamped values and every
// velocity, enthalpy and wave speed is a ratio that the factor leaves alone.
template <class T, bool FAST, bool Y, int S = 1>
__device__ __forceinline__ RiemannPre<T, FAST, Y> riemann_pre(const T ql[4], const T qr[4], T gamma) {
  static_assert(S == 1 || FAST, "doubled states are a FAST form");
  RiemannPre<T, FAST, Y> r;
  r.ql0 = cmax<T, FAST>(ql[0], T(kEps * S));
  r.qr0 = cmax<T, FAST>(qr[0], T(kEps * S));
  T h_l, h_r, u_t, v_t, h_t;
  T rsl = T(0.0), rsr = T(0.0);  // FAST: 1/sqrt(rho) per side
  if constexpr (!FAST) {
    r.u_l = ql[1] / r.ql0; r.v_l = ql[2] / r.ql0;
    r.u_r = qr[1] / r.qr0; r.v_r = qr[2] / r.qr0;
  } else {
    rsl = frsqrt(r.ql0);
    rsr = frsqrt(r.qr0);
    const T il = rsl * rsl, ir = rsr * rsr;
    r.u_l = ql[1] * il; r.v_l = ql[2] * il;
    r.u_r = qr[1] * ir; r.v_r = qr[2] * ir;
  }
  // FAST: sqrt(rho)*u = q1/sqrt(rho) and sqrt(rho)*h = (E+p)/sqrt(rho); the
  // kinetic energy is (m^2 + n^2) / (2 rho), without the velocities.
  if constexpr (!FAST) {
    r.p_l = (gamma - T(1.0)) * (ql[3] - half_rho_speed2<T, FAST>(r.ql0, ql[1], ql[2], r.u_l, r.v_l));
    r.p_r = (gamma - T(1.0)) * (qr[3] - half_rho_speed2<T, FAST>(r.qr0, qr[1], qr[2], r.u_r, r.v_r));
  } else {
    r.p_l = (gamma - T(1.0)) * (ql[3] - T(0.5) * ((ql[1] * ql[1] + ql[2] * ql[2]) * (rsl * rsl)));
    r.p_r = (gamma - T(1.0)) * (qr[3] - T(0.5) * ((qr[1] * qr[1] + qr[2] * qr[2]) * (rsr * rsr)));
  }
  r.p_l = cmax<T, FAST>(r.p_l, T(kEps * S));
  r.p_r = cmax<T, FAST>(r.p_r, T(kEps * S));
  if constexpr (!FAST) {
    const T srl = sqrt(r.ql0), srr = sqrt(r.qr0);
    const T denom_r = srl + srr;
    h_l = (ql[3] + r.p_l) / r.ql0;
    h_r = (qr[3] + r.p_r) / r.qr0;
    u_t = (srl * r.u_l + srr * r.u_r) / denom_r;
    v_t = (srl * r.v_l + srr * r.v_r) / denom_r;
    h_t = (srl * h_l + srr * h_r) / denom_r;
  } else {
    // sqrt(rho) = rho r and sqrt(rho)*h = (E+p) r with r = 1/sqrt(rho) per side.
    const T id = qrcp<T, FAST>(r.ql0 * rsl + r.qr0 * rsr);
    u_t = sum_prod_rn<T>(ql[1], rsl, qr[1], rsr) * id;
    v_t = sum_prod_rn<T>(ql[2], rsl, qr[2], rsr) * id;
    h_t = ((ql[3] + r.p_l) * rsl + (qr[3] + r.p_r) * rsr) * id;
  }
  const T tmp = h_t - T(0.5) * (u_t * u_t + v_t * v_t);
  const T a_t = qsqrt<T, FAST>(cmax<T, FAST>((gamma - T(1.0)) * tmp, T(0.0)));
  const T un_t = Y ? v_t : u_t;
  r.un_l = Y ? r.v_l : r.u_l;
  r.un_r = Y ? r.v_r : r.u_r;
  r.s_l = un_t - a_t;
  r.s_r = un_t + a_t;
  return r;
}

template <class T, bool FAST>
__device__ __forceinline__ T guard_denom(T d) {
  bool small;
  if constexpr (FAST && is_native_f64<T>)
    small = (__double_as_longlong(d) & 0x7fffffffffffffffLL) < __double_as_longlong(kEps);
  else
    small = fabs(d) < T(kEps);
  if (small) d = copysign(T(kEps), d) + T(kEps);
  return d;
}

// riemann.rs:191-349 HLLE.  S = 2: states and fluxes are doubled (riemann_pre),
// the flux is halved on the way out.
template <class T, bool FAST, bool Y, int S = 1>
__device__ __forceinline__ void hlle_flux(const RiemannPre<T, FAST, Y>& r, const T ql[4], const T fl[4],
                                          const T qr[4], const T fr[4], T F[4]) {
  const T denom = guard_denom<T, FAST>(r.s_r - r.s_l);
  if (r.s_l >= T(0.0)) {
#pragma unroll
    for (int k = 0; k < 4; ++k) F[k] = S == 1 ? fl[k] : T(0.5) * fl[k];
  } else if (r.s_r < T(0.0)) {
#pragma unroll
    for (int k = 0; k < 4; ++k) F[k] = S == 1 ? fr[k] : T(0.5) * fr[k];
  } else {
    const T qlv[4] = {r.ql0, ql[1], ql[2], ql[3]};
    const T qrv[4] = {r.qr0, qr[1], qr[2], qr[3]};
    const T srsl = r.s_r * r.s_l;
    if constexpr (!FAST) {
#pragma unroll
      for (int k = 0; k < 4; ++k) F[k] = (r.s_r * fl[k] - r.s_l * fr[k] + srsl * (qrv[k] - qlv[k])) / denom;
    } else {
      const T id = qrcp<T, FAST>(S == 1 ? denom : T(S) * denom);
#pragma unroll
      for (int k = 0; k < 4; ++k) F[k] = (r.s_r * fl[k] - r.s_l * fr[k] + srsl * (qrv[k] - qlv[k])) * id;
    }
  }
}

// riemann.rs:6-189 HLLC
template <class T, bool FAST, bool Y>
__device__ __forceinline__ void hllc_flux(const RiemannPre<T, FAST, Y>& r, const T ql[4], const T fl[4],
                                          const T qr[4], const T fr[4], T F[4]) {
  if (r.s_l >= T(0.0)) {
#pragma unroll
    for (int k = 0; k < 4; ++k) F[k] = fl[k];
    return;
  }
  const T denom = guard_denom<T, FAST>(r.ql0 * (r.s_l - r.un_l) - r.qr0 * (r.s_r - r.un_r));
  // FAST: the two momentum terms rounded on their own, so mirror-image states give
  // S* = +0.0 exactly, as the reference's arithmetic does
  const T s_star = FAST ? qdiv<T, FAST>((r.p_r - r.p_l) + sum_prod_rn<T>(r.ql0 * r.un_l, r.s_l - r.un_l,
                                                                           -(r.qr0 * r.un_r), r.s_r - r.un_r),
                                        denom)
                        : qdiv<T, FAST>(r.p_r - r.p_l + r.ql0 * r.un_l * (r.s_l - r.un_l) -
                                            r.qr0 * r.un_r * (r.s_r - r.un_r),
                                        denom);
  if (r.s_l < T(0.0) && s_star >= T(0.0)) {
    // left star state
    const T m_l = r.ql0 * (r.s_l - r.un_l);
    const T coeff = qdiv<T, FAST>(m_l, r.s_l - s_star);
    const T e_spec = qdiv<T, FAST>(ql[3], r.ql0);
    const T e_star = e_spec + (s_star - r.un_l) * (s_star + qdiv<T, FAST>(r.p_l, m_l));
    T qs[4];
    qs[0] = coeff;
    qs[1] = Y ? coeff * r.u_l : coeff * s_star;
    qs[2] = Y ? coeff * s_star : coeff * r.v_l;
    qs[3] = coeff * e_star;
#pragma unroll
    for (int k = 0; k < 4; ++k) F[k] = fl[k] + r.s_l * (qs[k] - ql[k]);
  } else if (s_star < T(0.0) && r.s_r > T(0.0)) {
    const T m_r = r.qr0 * (r.s_r - r.un_r);
    const T coeff = qdiv<T, FAST>(m_r, r.s_r - s_star);
    const T e_spec = qdiv<T, FAST>(qr[3], r.qr0);
    const T e_star = e_spec + (s_star - r.un_r) * (s_star + qdiv<T, FAST>(r.p_r, m_r));
    T qs[4];
    qs[0] = coeff;
    qs[1] = Y ? coeff * r.u_r : coeff * s_star;
    qs[2] = Y ? coeff * s_star : coeff * r.v_r;
    qs[3] = coeff * e_star;
#pragma unroll
    for (int k = 0; k < 4; ++k) F[k] = fr[k] + r.s_r * (qs[k] - qr[k]);
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) F[k] = fr[k];
  }
}

// riemann.rs:394-405: blend weight from the normalised pressure gradient.
template <class T, bool FAST>
__device__ __forceinline__ T sensor_weight(T dpdx, T dpdy, T p, T jp_lo, T jp_hi) {
  const T grad = qsqrt<T, FAST>(dpdx * dpdx + dpdy * dpdy);
  const T jp = qdiv<T, FAST>(grad, vmax(p, T(kEps)));
  if (jp <= jp_lo) return T(1.0);
  if (jp >= jp_hi) return T(0.0);
  return T(1.0) - qdiv<T, FAST>(jp - jp_lo, jp_hi - jp_lo);
}

}  // inline namespace WENO_TU_NS
}  // namespace weno
