// ORACLE -- test infrastructure only.  Never linked into the product library.
//
// CPU restatement of the reference's Rust residual core (weno_ext/src/utils.rs,
// weno_ext/src/weno.rs, weno_ext/src/riemann.rs) and of the numpy driver
// arithmetic around it (Rie_prob_2d_rs.py, unitest.py, double_mach_reflection.py).
// It keeps the reference's whole-array pass structure, operation order and
// constants (including the truncated SQRT3_12 and the 10-digit Gauss weights)
// so that, compiled with -ffp-contract=off, every value is the IEEE-754 double
// the reference computes.  Only tests/, the smoke check and bench.py's CPU
// baseline leg load it, and only as the checker.
//
// Parity pinning: the component-wise + HLLE path, flux, con2primi and the
// pressure-gradient sensor are checked against golden vectors produced by the
// reference's own numpy twin (WENO_HLLC_2d.py) and the driver helpers
// (Rie_prob_2d_rs.py, unitest.py) -- see tests/golden/make_golden.py.  The
// characteristic projection and the HLLC star-right branch have no independent
// implementation in the reference and are pinned by restatement plus the
// invariant tests (free stream, L*R = I, mirror symmetry).
//
// The numerical core is a template over the scalar type so that the same code
// also runs on a counting scalar (exact per-operation tallies for the roofline's
// algorithmic FLOP figure).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

// ---------------------------------------------------------------------------
// Counting scalar: every arithmetic operation bumps a tally.
// ---------------------------------------------------------------------------
struct Tally {
  uint64_t add = 0, mul = 0, div = 0, sqrt = 0, cmp = 0;
};
static Tally g_tally;

struct Cnt {
  double v;
  Cnt() : v(0.0) {}
  Cnt(double x) : v(x) {}
};
static inline Cnt operator+(Cnt a, Cnt b) { g_tally.add++; return Cnt(a.v + b.v); }
static inline Cnt operator-(Cnt a, Cnt b) { g_tally.add++; return Cnt(a.v - b.v); }
static inline Cnt operator*(Cnt a, Cnt b) { g_tally.mul++; return Cnt(a.v * b.v); }
static inline Cnt operator/(Cnt a, Cnt b) { g_tally.div++; return Cnt(a.v / b.v); }
static inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
static inline bool operator<(Cnt a, Cnt b) { g_tally.cmp++; return a.v < b.v; }
static inline bool operator<=(Cnt a, Cnt b) { g_tally.cmp++; return a.v <= b.v; }
static inline bool operator>(Cnt a, Cnt b) { g_tally.cmp++; return a.v > b.v; }
static inline bool operator>=(Cnt a, Cnt b) { g_tally.cmp++; return a.v >= b.v; }
static inline Cnt& operator+=(Cnt& a, Cnt b) { a = a + b; return a; }

// Rust f64::max / f64::min return the non-NaN operand, like C fmax / fmin.
static inline double vmax(double a, double b) { return std::fmax(a, b); }
static inline double vmin(double a, double b) { return std::fmin(a, b); }
static inline double vsqrt(double a) { return std::sqrt(a); }
static inline double vabs(double a) { return std::fabs(a); }
static inline double vcopysign(double a, double b) { return std::copysign(a, b); }
static inline double val(double a) { return a; }
static inline Cnt vmax(Cnt a, Cnt b) { g_tally.cmp++; return Cnt(std::fmax(a.v, b.v)); }
static inline Cnt vmin(Cnt a, Cnt b) { g_tally.cmp++; return Cnt(std::fmin(a.v, b.v)); }
static inline Cnt vsqrt(Cnt a) { g_tally.sqrt++; return Cnt(std::sqrt(a.v)); }
static inline Cnt vabs(Cnt a) { return Cnt(std::fabs(a.v)); }
static inline Cnt vcopysign(Cnt a, Cnt b) { return Cnt(std::copysign(a.v, b.v)); }
static inline double val(Cnt a) { return a.v; }

// utils.rs:3-6
const double DEFAULT_EPS = 1e-12;
const double SQRT3_12 = 0.1443375673;
const double RHO_MIN = 1e-12;
const double P_MIN = 1e-12;
// The WENO smoothness epsilon: DEFAULT_EPS in the reference (weno.rs:223);
// configurable for configurations that name another value.
static double g_weno_eps = DEFAULT_EPS;

// Dense (m, n, 4) array with the layout of an ndarray Array3 in C order.
template <class T>
struct A3 {
  int64_t m = 0, n = 0, c = 0;
  std::vector<T> d;
  A3() {}
  A3(int64_t m_, int64_t n_, int64_t c_) : m(m_), n(n_), c(c_), d((size_t)(m_ * n_ * c_), T(0.0)) {}
  T& at(int64_t i, int64_t j, int64_t k) { return d[(size_t)((i * n + j) * c + k)]; }
  const T& at(int64_t i, int64_t j, int64_t k) const { return d[(size_t)((i * n + j) * c + k)]; }
};
template <class T>
struct A2 {
  int64_t m = 0, n = 0;
  std::vector<T> d;
  A2() {}
  A2(int64_t m_, int64_t n_) : m(m_), n(n_), d((size_t)(m_ * n_), T(0.0)) {}
  T& at(int64_t i, int64_t j) { return d[(size_t)(i * n + j)]; }
  const T& at(int64_t i, int64_t j) const { return d[(size_t)(i * n + j)]; }
};

// Read-only strided view of caller memory (an ndarray ArrayView3).
struct View3 {
  const double* p;
  int64_t m, n, c, s0, s1, s2;
  double at(int64_t i, int64_t j, int64_t k) const { return p[i * s0 + j * s1 + k * s2]; }
};

template <class T>
static A3<T> copy4(const View3& u) {
  A3<T> o(u.m, u.n, 4);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < u.m; ++i)
    for (int64_t j = 0; j < u.n; ++j)
      for (int k = 0; k < 4; ++k) o.at(i, j, k) = T(u.at(i, j, k));
  return o;
}

// ---------------------------------------------------------------------------
// utils.rs:9-35  con2primi_local
// ---------------------------------------------------------------------------
template <class T>
static void con2primi(const A3<T>& q, T gamma, A2<T>& p, A2<T>& a, A2<T>& rs, A2<T>& u, A2<T>& v, A2<T>& h) {
  p = A2<T>(q.m, q.n); a = A2<T>(q.m, q.n); rs = A2<T>(q.m, q.n);
  u = A2<T>(q.m, q.n); v = A2<T>(q.m, q.n); h = A2<T>(q.m, q.n);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < q.m; ++i)
    for (int64_t j = 0; j < q.n; ++j) {
      T rho = vmax(q.at(i, j, 0), T(DEFAULT_EPS));
      rs.at(i, j) = rho;
      T uval = q.at(i, j, 1) / rho;
      T vval = q.at(i, j, 2) / rho;
      u.at(i, j) = uval;
      v.at(i, j) = vval;
      T pval = vmax((gamma - T(1.0)) * (q.at(i, j, 3) - T(0.5) * rho * (uval * uval + vval * vval)), T(DEFAULT_EPS));
      p.at(i, j) = pval;
      a.at(i, j) = vsqrt(gamma * pval / rho);
      h.at(i, j) = (q.at(i, j, 3) + pval) / rho;
    }
}

// utils.rs:74-90 flux_x_local ; utils.rs:93-109 flux_y_local
template <class T>
static A3<T> flux_dir(const A3<T>& q, T gamma, bool ydir) {
  A3<T> f(q.m, q.n, 4);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < q.m; ++i)
    for (int64_t j = 0; j < q.n; ++j) {
      T rho = vmax(q.at(i, j, 0), T(DEFAULT_EPS));
      T u = q.at(i, j, 1) / rho;
      T v = q.at(i, j, 2) / rho;
      T p = (gamma - T(1.0)) * (q.at(i, j, 3) - T(0.5) * rho * (u * u + v * v));
      if (!ydir) {
        f.at(i, j, 0) = q.at(i, j, 1);
        f.at(i, j, 1) = q.at(i, j, 1) * u + p;
        f.at(i, j, 2) = q.at(i, j, 2) * u;
        f.at(i, j, 3) = u * (q.at(i, j, 3) + p);
      } else {
        f.at(i, j, 0) = q.at(i, j, 2);
        f.at(i, j, 1) = q.at(i, j, 1) * v;
        f.at(i, j, 2) = q.at(i, j, 2) * v + p;
        f.at(i, j, 3) = v * (q.at(i, j, 3) + p);
      }
    }
  return f;
}

// ---------------------------------------------------------------------------
// weno.rs:13-52 roe_avg_x (roe_avg_y at :57-63 is the same arithmetic)
// ---------------------------------------------------------------------------
template <class T>
static void roe_avg(const T* ul, const T* ur, T gamma, T& rho_roe, T& u_roe, T& v_roe, T& h_roe, T& c_roe) {
  T rho_l = vmax(ul[0], T(RHO_MIN));
  T rho_r = vmax(ur[0], T(RHO_MIN));
  T sqrt_l = vsqrt(rho_l);
  T sqrt_r = vsqrt(rho_r);
  T denom = sqrt_l + sqrt_r;
  T u_l = ul[1] / rho_l;
  T v_l = ul[2] / rho_l;
  T u_r = ur[1] / rho_r;
  T v_r = ur[2] / rho_r;
  T p_l = vmax((gamma - T(1.0)) * (ul[3] - T(0.5) * rho_l * (u_l * u_l + v_l * v_l)), T(P_MIN));
  T p_r = vmax((gamma - T(1.0)) * (ur[3] - T(0.5) * rho_r * (u_r * u_r + v_r * v_r)), T(P_MIN));
  T h_l = (ul[3] + p_l) / rho_l;
  T h_r = (ur[3] + p_r) / rho_r;
  u_roe = (sqrt_l * u_l + sqrt_r * u_r) / denom;
  v_roe = (sqrt_l * v_l + sqrt_r * v_r) / denom;
  h_roe = (sqrt_l * h_l + sqrt_r * h_r) / denom;
  T kin = T(0.5) * (u_roe * u_roe + v_roe * v_roe);
  T c2 = vmax((gamma - T(1.0)) * (h_roe - kin), T(P_MIN) / vmin(rho_l, rho_r));
  c_roe = vsqrt(c2);
  rho_roe = sqrt_l * sqrt_r;
}

// weno.rs:76-107 left_eigenvectors_x ; weno.rs:136-167 left_eigenvectors_y
template <class T>
static void left_eig(bool ydir, T rho, T u, T v, T c, T gamma, T L[4][4]) {
  T g1 = gamma - T(1.0);
  T kin = T(0.5) * (u * u + v * v);
  T rc = rho * c;
  T inv_rc = T(1.0) / rc;
  T inv_c2 = T(1.0) / (c * c);
  T vn = ydir ? v : u;  // normal velocity
  T a = g1 * kin / (T(2.0) * c * c);
  T b = vn / (T(2.0) * c);
  T gu = -g1 * u * inv_c2 / T(2.0);
  T gv = -g1 * v * inv_c2 / T(2.0);
  T gg = g1 * inv_c2 / T(2.0);
  if (!ydir) {
    L[0][0] = a + b; L[0][1] = gu - T(0.5) * inv_rc; L[0][2] = gv; L[0][3] = gg;
    L[3][0] = a - b; L[3][1] = gu + T(0.5) * inv_rc; L[3][2] = gv; L[3][3] = gg;
    L[2][0] = -v / rho; L[2][1] = T(0.0); L[2][2] = T(1.0) / rho; L[2][3] = T(0.0);
  } else {
    L[0][0] = a + b; L[0][1] = gu; L[0][2] = gv - T(0.5) * inv_rc; L[0][3] = gg;
    L[3][0] = a - b; L[3][1] = gu; L[3][2] = gv + T(0.5) * inv_rc; L[3][3] = gg;
    L[2][0] = -u / rho; L[2][1] = T(1.0) / rho; L[2][2] = T(0.0); L[2][3] = T(0.0);
  }
  L[1][0] = T(1.0) - g1 * kin * inv_c2;
  L[1][1] = g1 * u * inv_c2;
  L[1][2] = g1 * v * inv_c2;
  L[1][3] = -g1 * inv_c2;
}

// weno.rs:113-131 right_eigenvectors_x ; weno.rs:171-189 right_eigenvectors_y
template <class T>
static void right_eig(bool ydir, T rho, T u, T v, T h, T c, T R[4][4]) {
  T kin = T(0.5) * (u * u + v * v);
  R[0][0] = T(1.0); R[0][1] = T(1.0); R[0][2] = T(0.0); R[0][3] = T(1.0);
  if (!ydir) {
    R[1][0] = u - c; R[1][1] = u; R[1][2] = T(0.0); R[1][3] = u + c;
    R[2][0] = v; R[2][1] = v; R[2][2] = rho; R[2][3] = v;
    R[3][0] = h - u * c; R[3][1] = kin; R[3][2] = rho * v; R[3][3] = h + u * c;
  } else {
    R[1][0] = u; R[1][1] = u; R[1][2] = rho; R[1][3] = u;
    R[2][0] = v - c; R[2][1] = v; R[2][2] = T(0.0); R[2][3] = v + c;
    R[3][0] = h - v * c; R[3][1] = kin; R[3][2] = rho * u; R[3][3] = h + v * c;
  }
}

// weno.rs:197-205 mat4_vec4 (accumulation from 0.0 in column order)
template <class T>
static void mat4_vec4(const T M[4][4], const T* x, T* out) {
  for (int r = 0; r < 4; ++r) {
    T acc = T(0.0);
    for (int c = 0; c < 4; ++c) acc += M[r][c] * x[c];
    out[r] = acc;
  }
}

// weno.rs:214-233 weno5_left (also the q_l part of weno.rs:664-688)
template <class T>
static T weno5_left(T u0, T u1, T u2, T u3, T u4) {
  const T c13 = T(13.0 / 12.0);
  T t;
  t = u2 - T(2.0) * u3 + u4; T s = T(3.0) * u2 - T(4.0) * u3 + u4;
  T beta0 = c13 * (t * t) + T(0.25) * (s * s);
  t = u1 - T(2.0) * u2 + u3; s = u1 - u3;
  T beta1 = c13 * (t * t) + T(0.25) * (s * s);
  t = u0 - T(2.0) * u1 + u2; s = u0 - T(4.0) * u1 + T(3.0) * u2;
  T beta2 = c13 * (t * t) + T(0.25) * (s * s);
  T e0 = T(g_weno_eps) + beta0, e1 = T(g_weno_eps) + beta1, e2 = T(g_weno_eps) + beta2;
  T a0 = T(0.3) / (e0 * e0);
  T a1 = T(0.6) / (e1 * e1);
  T a2 = T(0.1) / (e2 * e2);
  T sum = a0 + a1 + a2;
  T w0 = a0 / sum, w1 = a1 / sum, w2 = a2 / sum;
  T p0 = -u4 + T(5.0) * u3 + T(2.0) * u2;
  T p1 = -u1 + T(5.0) * u2 + T(2.0) * u3;
  T p2 = T(2.0) * u0 - T(7.0) * u1 + T(11.0) * u2;
  return (w0 * p0 + w1 * p1 + w2 * p2) / T(6.0);
}

// weno.rs:238-257 weno5_right (also the q_r part of weno.rs:690-714)
template <class T>
static T weno5_right(T u1, T u2, T u3, T u4, T u5) {
  const T c13 = T(13.0 / 12.0);
  T t, s;
  t = u3 - T(2.0) * u4 + u5; s = T(3.0) * u3 - T(4.0) * u4 + u5;
  T beta0 = c13 * (t * t) + T(0.25) * (s * s);
  t = u2 - T(2.0) * u3 + u4; s = u2 - u4;
  T beta1 = c13 * (t * t) + T(0.25) * (s * s);
  t = u1 - T(2.0) * u2 + u3; s = u1 - T(4.0) * u2 + T(3.0) * u3;
  T beta2 = c13 * (t * t) + T(0.25) * (s * s);
  T e0 = T(g_weno_eps) + beta0, e1 = T(g_weno_eps) + beta1, e2 = T(g_weno_eps) + beta2;
  T a0 = T(0.1) / (e0 * e0);
  T a1 = T(0.6) / (e1 * e1);
  T a2 = T(0.3) / (e2 * e2);
  T sum = a0 + a1 + a2;
  T w0 = a0 / sum, w1 = a1 / sum, w2 = a2 / sum;
  T p0 = T(2.0) * u5 - T(7.0) * u4 + T(11.0) * u3;
  T p1 = -u4 + T(5.0) * u3 + T(2.0) * u2;
  T p2 = -u1 + T(5.0) * u2 + T(2.0) * u3;
  return (w0 * p0 + w1 * p1 + w2 * p2) / T(6.0);
}

// weno.rs:262-281 weno5_gq_left_a and weno.rs:284-303 weno5_gq_left_b
// (the cons pass at weno.rs:737-782 evaluates the same expressions).
template <class T>
static T weno5_gq(T q0, T q1, T q2, T q3, T q4, bool second) {
  const T c13 = T(13.0 / 12.0);
  T t, s;
  t = q2 - T(2.0) * q3 + q4; s = T(3.0) * q2 - T(4.0) * q3 + q4;
  T beta0 = c13 * (t * t) + T(0.25) * (s * s);
  t = q1 - T(2.0) * q2 + q3; s = q1 - q3;
  T beta1 = c13 * (t * t) + T(0.25) * (s * s);
  t = q0 - T(2.0) * q1 + q2; s = q0 - T(4.0) * q1 + T(3.0) * q2;
  T beta2 = c13 * (t * t) + T(0.25) * (s * s);
  T d0 = second ? T(0.1960481952) : T(0.1928406937);
  T d1 = T(0.6111111111);
  T d2 = second ? T(0.1928406937) : T(0.1960481952);
  T e0 = T(g_weno_eps) + beta0, e1 = T(g_weno_eps) + beta1, e2 = T(g_weno_eps) + beta2;
  T a0 = d0 / (e0 * e0);
  T a1 = d1 / (e1 * e1);
  T a2 = d2 / (e2 * e2);
  T sum = a0 + a1 + a2;
  T w0 = a0 / sum, w1 = a1 / sum, w2 = a2 / sum;
  const T S = T(SQRT3_12);
  T p0, p1, p2;
  if (!second) {
    p0 = q2 + (T(3.0) * q2 - T(4.0) * q3 + q4) * S;
    p1 = q2 - (-q1 + q3) * S;
    p2 = q2 - (T(3.0) * q2 - T(4.0) * q1 + q0) * S;
  } else {
    p0 = q2 - (T(3.0) * q2 - T(4.0) * q3 + q4) * S;
    p1 = q2 - (q1 - q3) * S;
    p2 = q2 + (T(3.0) * q2 - T(4.0) * q1 + q0) * S;
  }
  return w0 * p0 + w1 * p1 + w2 * p2;
}

// weno.rs:312-315 pressure ; weno.rs:327-352 pp_limit
template <class T>
static T pressure4(const T* q, T gamma) {
  if (q[0] <= T(0.0)) return T(0.0);
  return (gamma - T(1.0)) * (q[3] - T(0.5) * (q[1] * q[1] + q[2] * q[2]) / q[0]);
}
template <class T>
static void pp_limit(T* q, const T* ub, T gamma) {
  if (q[0] < T(RHO_MIN)) {
    T rho_bar = vmax(ub[0], T(RHO_MIN));
    T theta = vmax(vmin((rho_bar - T(RHO_MIN)) / (rho_bar - q[0]), T(1.0)), T(0.0));
    for (int k = 0; k < 4; ++k) q[k] = theta * (q[k] - ub[k]) + ub[k];
  }
  T p_q = pressure4(q, gamma);
  if (p_q < T(P_MIN)) {
    T p_bar = vmax(pressure4(ub, gamma), T(P_MIN));
    T theta = vmax(vmin((p_bar - T(P_MIN)) / (p_bar - p_q), T(1.0)), T(0.0));
    for (int k = 0; k < 4; ++k) q[k] = theta * (q[k] - ub[k]) + ub[k];
  }
}

// Reconstruction result: face states and face fluxes.
template <class T>
struct Faces { A3<T> ql, fl, qr, fr; };

// ---------------------------------------------------------------------------
// weno.rs:367-502 weno_x_reconstruct_local, weno.rs:508-632 weno_y_reconstruct_local,
// weno.rs:635-852 weno_x_reconstruct_local_cons, weno.rs:854-1071 _y_ _cons.
// `ydir` selects the sweep direction, `cons` the component-wise variant.
// ---------------------------------------------------------------------------
template <class T>
static Faces<T> reconstruct(const A3<T>& uc, T gamma, bool ydir, bool cons) {
  const int64_t m = uc.m, n = uc.n;
  const int64_t om = ydir ? m : m - 5;
  const int64_t on = ydir ? n - 5 : n;
  A3<T> q_l(om, on, 4), q_r(om, on, 4);
  // Pass 1: normal-direction WENO5 over a 6-cell stencil.
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < om; ++i)
    for (int64_t j = 0; j < on; ++j) {
      T cells[6][4];
      for (int s = 0; s < 6; ++s)
        for (int k = 0; k < 4; ++k) cells[s][k] = ydir ? uc.at(i, j + s, k) : uc.at(i + s, j, k);
      T cl[4], cr[4];
      if (cons) {
        for (int k = 0; k < 4; ++k) {
          cl[k] = weno5_left(cells[0][k], cells[1][k], cells[2][k], cells[3][k], cells[4][k]);
          cr[k] = weno5_right(cells[1][k], cells[2][k], cells[3][k], cells[4][k], cells[5][k]);
        }
      } else {
        // Left face: Roe average at cells[2|3] (weno.rs:409-425)
        T rho_a, u_a, v_a, h_a, c_a;
        roe_avg(cells[2], cells[3], gamma, rho_a, u_a, v_a, h_a, c_a);
        T Lm[4][4], Rm[4][4];
        left_eig(ydir, rho_a, u_a, v_a, c_a, gamma, Lm);
        right_eig(ydir, rho_a, u_a, v_a, h_a, c_a, Rm);
        T wl[5][4];
        for (int s = 0; s < 5; ++s) mat4_vec4(Lm, cells[s], wl[s]);
        T chl[4];
        for (int k = 0; k < 4; ++k) chl[k] = weno5_left(wl[0][k], wl[1][k], wl[2][k], wl[3][k], wl[4][k]);
        mat4_vec4(Rm, chl, cl);
        // Right face: the reference recomputes the same Roe average (weno.rs:428-444)
        roe_avg(cells[2], cells[3], gamma, rho_a, u_a, v_a, h_a, c_a);
        left_eig(ydir, rho_a, u_a, v_a, c_a, gamma, Lm);
        right_eig(ydir, rho_a, u_a, v_a, h_a, c_a, Rm);
        T wr[5][4];
        for (int s = 0; s < 5; ++s) mat4_vec4(Lm, cells[s + 1], wr[s]);
        T chr[4];
        for (int k = 0; k < 4; ++k) chr[k] = weno5_right(wr[0][k], wr[1][k], wr[2][k], wr[3][k], wr[4][k]);
        mat4_vec4(Rm, chr, cr);
        pp_limit(cl, cells[2], gamma);
        pp_limit(cr, cells[3], gamma);
      }
      for (int k = 0; k < 4; ++k) { q_l.at(i, j, k) = cl[k]; q_r.at(i, j, k) = cr[k]; }
    }
  // Pass 2: transverse 2-point Gauss-quadrature WENO over a 5-cell stencil.
  const int64_t m1 = ydir ? om - 6 : om;
  const int64_t n1 = ydir ? on : on - 6;
  A3<T> ql1(m1, n1, 4), ql2(m1, n1, 4), qr1(m1, n1, 4), qr2(m1, n1, 4);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m1; ++i)
    for (int64_t j = 0; j < n1; ++j)
      for (int k = 0; k < 4; ++k) {
        T a[5], b[5];
        for (int s = 0; s < 5; ++s) {
          a[s] = ydir ? q_l.at(i + 1 + s, j, k) : q_l.at(i, j + 1 + s, k);
          b[s] = ydir ? q_r.at(i + 1 + s, j, k) : q_r.at(i, j + 1 + s, k);
        }
        ql1.at(i, j, k) = weno5_gq(a[0], a[1], a[2], a[3], a[4], false);
        ql2.at(i, j, k) = weno5_gq(a[0], a[1], a[2], a[3], a[4], true);
        qr1.at(i, j, k) = weno5_gq(b[0], b[1], b[2], b[3], b[4], false);
        qr2.at(i, j, k) = weno5_gq(b[0], b[1], b[2], b[3], b[4], true);
      }
  A3<T> fl1 = flux_dir(ql1, gamma, ydir), fl2 = flux_dir(ql2, gamma, ydir);
  A3<T> fr1 = flux_dir(qr1, gamma, ydir), fr2 = flux_dir(qr2, gamma, ydir);
  Faces<T> out;
  out.ql = A3<T>(m1, n1, 4); out.fl = A3<T>(m1, n1, 4);
  out.qr = A3<T>(m1, n1, 4); out.fr = A3<T>(m1, n1, 4);
  for (size_t e = 0; e < out.ql.d.size(); ++e) {
    out.fl.d[e] = T(0.5) * (fl1.d[e] + fl2.d[e]);
    out.fr.d[e] = T(0.5) * (fr2.d[e] + fr1.d[e]);
    out.ql.d[e] = T(0.5) * (ql1.d[e] + ql2.d[e]);
    out.qr.d[e] = T(0.5) * (qr1.d[e] + qr2.d[e]);
  }
  return out;
}

// ---------------------------------------------------------------------------
// riemann.rs:6-96 hllc_x_local, :99-189 hllc_y_local,
// riemann.rs:191-269 hlle_x_local, :271-349 hlle_y_local
// ---------------------------------------------------------------------------
template <class T>
static A3<T> riemann(const A3<T>& q_l, const A3<T>& f_l, const A3<T>& q_r, const A3<T>& f_r, T gamma, bool ydir, bool hlle) {
  A3<T> out(q_l.m, q_l.n, 4);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < q_l.m; ++i)
    for (int64_t j = 0; j < q_l.n; ++j) {
      T ql0 = vmax(q_l.at(i, j, 0), T(DEFAULT_EPS));
      T ql1 = q_l.at(i, j, 1), ql2 = q_l.at(i, j, 2), ql3 = q_l.at(i, j, 3);
      T qr0 = vmax(q_r.at(i, j, 0), T(DEFAULT_EPS));
      T qr1 = q_r.at(i, j, 1), qr2 = q_r.at(i, j, 2), qr3 = q_r.at(i, j, 3);
      T u_l = ql1 / ql0, v_l = ql2 / ql0, u_r = qr1 / qr0, v_r = qr2 / qr0;
      T p_l = (gamma - T(1.0)) * (ql3 - T(0.5) * ql0 * (u_l * u_l + v_l * v_l));
      T p_r = (gamma - T(1.0)) * (qr3 - T(0.5) * qr0 * (u_r * u_r + v_r * v_r));
      p_l = vmax(p_l, T(DEFAULT_EPS));
      p_r = vmax(p_r, T(DEFAULT_EPS));
      T h_l = (ql3 + p_l) / ql0;
      T h_r = (qr3 + p_r) / qr0;
      T srl = vsqrt(ql0), srr = vsqrt(qr0);
      T denom_r = srl + srr;
      T u_t = (srl * u_l + srr * u_r) / denom_r;
      T v_t = (srl * v_l + srr * v_r) / denom_r;
      T h_t = (srl * h_l + srr * h_r) / denom_r;
      T tmp = h_t - T(0.5) * (u_t * u_t + v_t * v_t);
      T a_t = vsqrt(vmax((gamma - T(1.0)) * tmp, T(0.0)));
      T un_l = ydir ? v_l : u_l, un_r = ydir ? v_r : u_r, un_t = ydir ? v_t : u_t;
      T s_l = un_t - a_t, s_r = un_t + a_t;
      T fl[4], fr[4], fij[4];
      for (int k = 0; k < 4; ++k) { fl[k] = f_l.at(i, j, k); fr[k] = f_r.at(i, j, k); }
      if (hlle) {
        T denom = s_r - s_l;
        if (vabs(denom) < T(DEFAULT_EPS)) denom = vcopysign(T(DEFAULT_EPS), denom) + T(DEFAULT_EPS);
        T qlv[4] = {ql0, ql1, ql2, ql3}, qrv[4] = {qr0, qr1, qr2, qr3};
        if (s_l >= T(0.0)) {
          for (int k = 0; k < 4; ++k) fij[k] = fl[k];
        } else if (s_r < T(0.0)) {
          for (int k = 0; k < 4; ++k) fij[k] = fr[k];
        } else {
          for (int k = 0; k < 4; ++k) fij[k] = (s_r * fl[k] - s_l * fr[k] + s_r * s_l * (qrv[k] - qlv[k])) / denom;
        }
      } else {
        T denom = ql0 * (s_l - un_l) - qr0 * (s_r - un_r);
        if (vabs(denom) < T(DEFAULT_EPS)) denom = vcopysign(T(DEFAULT_EPS), denom) + T(DEFAULT_EPS);
        T s_star = (p_r - p_l + ql0 * un_l * (s_l - un_l) - qr0 * un_r * (s_r - un_r)) / denom;
        T coeff_l = ql0 * (s_l - un_l) / (s_l - s_star);
        T el_spec = ql3 / ql0;
        T e_star_l = el_spec + (s_star - un_l) * (s_star + p_l / (ql0 * (s_l - un_l)));
        T coeff_r = qr0 * (s_r - un_r) / (s_r - s_star);
        T er_spec = qr3 / qr0;
        T e_star_r = er_spec + (s_star - un_r) * (s_star + p_r / (qr0 * (s_r - un_r)));
        T qsl[4], qsr[4];
        qsl[0] = coeff_l; qsr[0] = coeff_r;
        if (!ydir) {
          qsl[1] = coeff_l * s_star; qsl[2] = coeff_l * v_l;
          qsr[1] = coeff_r * s_star; qsr[2] = coeff_r * v_r;
        } else {
          qsl[1] = coeff_l * u_l; qsl[2] = coeff_l * s_star;
          qsr[1] = coeff_r * u_r; qsr[2] = coeff_r * s_star;
        }
        qsl[3] = coeff_l * e_star_l; qsr[3] = coeff_r * e_star_r;
        if (s_l >= T(0.0)) {
          for (int k = 0; k < 4; ++k) fij[k] = fl[k];
        } else if (s_l < T(0.0) && s_star >= T(0.0)) {
          for (int k = 0; k < 4; ++k) fij[k] = fl[k] + s_l * (qsl[k] - q_l.at(i, j, k));
        } else if (s_star < T(0.0) && s_r > T(0.0)) {
          for (int k = 0; k < 4; ++k) fij[k] = fr[k] + s_r * (qsr[k] - q_r.at(i, j, k));
        } else {
          for (int k = 0; k < 4; ++k) fij[k] = fr[k];
        }
      }
      for (int k = 0; k < 4; ++k) out.at(i, j, k) = fij[k];
    }
  return out;
}

// riemann.rs:352-410 shock_sensor_grad_p.  Requires m >= 2 and n >= 2 (the
// reference indexes p[1] and p[m-2] unconditionally).
template <class T>
static A2<T> shock_sensor(const A2<T>& p, T jp_low, T jp_high) {
  const int64_t m = p.m, n = p.n;
  double min_dim = (double)std::max<int64_t>(std::min(m, n), 1);
  T dx = T(1.0) / T(min_dim);
  A2<T> dpdx(m, n), dpdy(m, n), phi(m, n);
  for (int64_t i = 1; i < m - 1; ++i)
    for (int64_t j = 0; j < n; ++j) dpdx.at(i, j) = (p.at(i + 1, j) - p.at(i - 1, j)) / (T(2.0) * dx);
  for (int64_t j = 0; j < n; ++j) {
    dpdx.at(0, j) = (p.at(1, j) - p.at(0, j)) / (T(2.0) * dx);
    dpdx.at(m - 1, j) = (p.at(m - 1, j) - p.at(m - 2, j)) / (T(2.0) * dx);
  }
  for (int64_t i = 0; i < m; ++i) {
    for (int64_t j = 1; j < n - 1; ++j) dpdy.at(i, j) = (p.at(i, j + 1) - p.at(i, j - 1)) / (T(2.0) * dx);
    dpdy.at(i, 0) = (p.at(i, 1) - p.at(i, 0)) / (T(2.0) * dx);
    dpdy.at(i, n - 1) = (p.at(i, n - 1) - p.at(i, n - 2)) / (T(2.0) * dx);
  }
  for (int64_t i = 0; i < m; ++i)
    for (int64_t j = 0; j < n; ++j) {
      T gx = dpdx.at(i, j), gy = dpdy.at(i, j);
      T grad = vsqrt(gx * gx + gy * gy);
      T jp = grad / vmax(p.at(i, j), T(DEFAULT_EPS));
      T w;
      if (jp <= jp_low) w = T(1.0);
      else if (jp >= jp_high) w = T(0.0);
      else w = T(1.0) - (jp - jp_low) / (jp_high - jp_low);
      phi.at(i, j) = w;
    }
  return phi;
}

// riemann.rs:412-448 hllc_hlle_blend_x_local, :450-486 _y_
template <class T>
static A3<T> blend(const A3<T>& q_l, const A3<T>& f_l, const A3<T>& q_r, const A3<T>& f_r, T gamma, bool ydir, T jp_low, T jp_high) {
  A2<T> pl, al, rl, ul, vl, hl, pr, ar, rr, ur, vr, hr;
  con2primi(q_l, gamma, pl, al, rl, ul, vl, hl);
  con2primi(q_r, gamma, pr, ar, rr, ur, vr, hr);
  A2<T> p(pl.m, pl.n);
  for (size_t e = 0; e < p.d.size(); ++e) p.d[e] = T(0.5) * (pl.d[e] + pr.d[e]);
  A2<T> phi = shock_sensor(p, jp_low, jp_high);
  A3<T> fc = riemann(q_l, f_l, q_r, f_r, gamma, ydir, false);
  A3<T> fe = riemann(q_l, f_l, q_r, f_r, gamma, ydir, true);
  A3<T> flux(fc.m, fc.n, 4);
  for (int64_t i = 0; i < fc.m; ++i)
    for (int64_t j = 0; j < fc.n; ++j) {
      T w = phi.at(i, j);
      for (int k = 0; k < 4; ++k) flux.at(i, j, k) = w * fc.at(i, j, k) + (T(1.0) - w) * fe.at(i, j, k);
    }
  return flux;
}

// riemann.rs:489-541 l_local
template <class T>
static A3<T> l_local(const A3<T>& uc, T dx, T gamma, bool force_hlle, T jp_lo, T jp_hi, bool cons) {
  Faces<T> fx = reconstruct(uc, gamma, false, cons);
  Faces<T> fy = reconstruct(uc, gamma, true, cons);
  A3<T> Fx = force_hlle ? riemann(fx.ql, fx.fl, fx.qr, fx.fr, gamma, false, true)
                        : blend(fx.ql, fx.fl, fx.qr, fx.fr, gamma, false, jp_lo, jp_hi);
  A3<T> Fy = force_hlle ? riemann(fy.ql, fy.fl, fy.qr, fy.fr, gamma, true, true)
                        : blend(fy.ql, fy.fl, fy.qr, fy.fr, gamma, true, jp_lo, jp_hi);
  const int64_t mo = Fx.m - 1, no = Fy.n - 1;
  A3<T> out(mo, no, 4);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < mo; ++i)
    for (int64_t j = 0; j < no; ++j)
      for (int k = 0; k < 4; ++k) {
        T dfdx = (Fx.at(i + 1, j, k) - Fx.at(i, j, k)) / dx;
        T dgdy = (Fy.at(i, j + 1, k) - Fy.at(i, j, k)) / dx;
        out.at(i, j, k) = -(dfdx + dgdy);
      }
  return out;
}

}  // namespace oracle

// ===========================================================================
// C ABI used by the test harness (ctypes).  Inputs are strided views in
// elements; outputs are dense C-order arrays owned by the caller.
// Return 0 on success, 1 on a shape error.
// ===========================================================================
using namespace oracle;

static View3 mkview(const double* p, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2) {
  View3 v{p, m, n, c, s0, s1, s2};
  return v;
}
template <class T>
static void store3(const A3<T>& a, double* out) {
  for (size_t e = 0; e < a.d.size(); ++e) out[e] = val(a.d[e]);
}
static A3<double> dense4(const double* p, int64_t m, int64_t n, int64_t c) {
  return copy4<double>(mkview(p, m, n, c, n * c, c, 1));
}

extern "C" {

void orc_set_weno_eps(double eps) { g_weno_eps = eps > 0.0 ? eps : DEFAULT_EPS; }

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int orc_flux(const double* q, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2, double gamma, int ydir, double* out) {
  if (c < 4) return 1;
  A3<double> uc = copy4<double>(mkview(q, m, n, c, s0, s1, s2));
  store3(flux_dir(uc, gamma, ydir != 0), out);
  return 0;
}

int orc_con2primi(const double* q, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2, double gamma,
                  double* p, double* a, double* rho, double* u, double* v, double* h) {
  if (c < 4) return 1;
  A3<double> uc = copy4<double>(mkview(q, m, n, c, s0, s1, s2));
  A2<double> P, A, R, U, V, H;
  con2primi(uc, gamma, P, A, R, U, V, H);
  size_t ne = (size_t)(m * n);
  std::memcpy(p, P.d.data(), ne * 8); std::memcpy(a, A.d.data(), ne * 8);
  std::memcpy(rho, R.d.data(), ne * 8); std::memcpy(u, U.d.data(), ne * 8);
  std::memcpy(v, V.d.data(), ne * 8); std::memcpy(h, H.d.data(), ne * 8);
  return 0;
}

// Outputs are (m-5, n-6, 4) for x and (m-6, n-5, 4) for y.
int orc_reconstruct(const double* u, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2, double gamma,
                    int ydir, int cons, double* ql, double* fl, double* qr, double* fr) {
  if (c < 4 || m < 6 || n < 6) return 1;
  A3<double> uc = copy4<double>(mkview(u, m, n, c, s0, s1, s2));
  Faces<double> f = reconstruct(uc, gamma, ydir != 0, cons != 0);
  store3(f.ql, ql); store3(f.fl, fl); store3(f.qr, qr); store3(f.fr, fr);
  return 0;
}

// kind: 0 = HLLC, 1 = HLLE, 2 = HLLC/HLLE blend.  Inputs dense (m, n, 4).
int orc_riemann(const double* ql, const double* fl, const double* qr, const double* fr, int64_t m, int64_t n,
                double gamma, int ydir, int kind, double jp_lo, double jp_hi, double* out) {
  if (kind == 2 && (m < 2 || n < 2)) return 1;
  A3<double> QL = dense4(ql, m, n, 4), FL = dense4(fl, m, n, 4), QR = dense4(qr, m, n, 4), FR = dense4(fr, m, n, 4);
  A3<double> F = kind == 2 ? blend(QL, FL, QR, FR, gamma, ydir != 0, jp_lo, jp_hi)
                           : riemann(QL, FL, QR, FR, gamma, ydir != 0, kind == 1);
  store3(F, out);
  return 0;
}

int orc_shock_sensor(const double* p, int64_t m, int64_t n, double jp_lo, double jp_hi, double* phi) {
  if (m < 2 || n < 2) return 1;
  A2<double> P(m, n);
  std::memcpy(P.d.data(), p, (size_t)(m * n) * 8);
  A2<double> F = shock_sensor(P, jp_lo, jp_hi);
  std::memcpy(phi, F.d.data(), (size_t)(m * n) * 8);
  return 0;
}

// Output (m-6, n-6, 4).
int orc_l_local(const double* u, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2, double dx,
                double gamma, int force_hlle, double jp_lo, double jp_hi, int cons, double* out) {
  if (c < 4 || m < 6 || n < 6) return 1;
  if (!force_hlle && (m < 8 || n < 8)) return 1;
  A3<double> uc = copy4<double>(mkview(u, m, n, c, s0, s1, s2));
  store3(l_local<double>(uc, dx, gamma, force_hlle != 0, jp_lo, jp_hi, cons != 0), out);
  return 0;
}

// Exact operation tallies of one l_local call (per call, not per cell).
int orc_count_l_local(const double* u, int64_t m, int64_t n, int64_t c, double dx, double gamma, int force_hlle,
                      double jp_lo, double jp_hi, int cons, uint64_t* tally5) {
  if (c < 4 || m < 8 || n < 8) return 1;
#ifdef _OPENMP
  int saved = omp_get_max_threads();
  omp_set_num_threads(1);
#endif
  g_tally = Tally();
  A3<Cnt> uc(m, n, 4);
  for (int64_t i = 0; i < m; ++i)
    for (int64_t j = 0; j < n; ++j)
      for (int k = 0; k < 4; ++k) uc.at(i, j, k) = Cnt(u[(i * n + j) * c + k]);
  A3<Cnt> o = l_local<Cnt>(uc, Cnt(dx), Cnt(gamma), force_hlle != 0, Cnt(jp_lo), Cnt(jp_hi), cons != 0);
  (void)o;
  tally5[0] = g_tally.add; tally5[1] = g_tally.mul; tally5[2] = g_tally.div;
  tally5[3] = g_tally.sqrt; tally5[4] = g_tally.cmp;
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  return 0;
}

// ---------------------------------------------------------------------------
// Driver arithmetic.  q is a dense (M, N, C) array, modified in place.
// ---------------------------------------------------------------------------

// Rie_prob_2d_rs.py:123-152 apply_bc_zero_gradient (mirror copy, no sign flip;
// the j-ghosts are filled first for every i, then the i-ghosts for every j).
void orc_bc_transmissive(double* q, int64_t M, int64_t N, int64_t C) {
  const int ng = 3;
  auto cell = [&](int64_t i, int64_t j) { return q + (i * N + j) * C; };
  for (int g = 0; g < ng; ++g) {
    int64_t mirror = 2 * ng - 1 - g;
    for (int64_t i = 0; i < M; ++i) std::memmove(cell(i, g), cell(i, mirror), C * 8);
  }
  for (int g = 0; g < ng; ++g) {
    int64_t interior = N - 2 * ng + g, ghost = N - 1 - g;
    for (int64_t i = 0; i < M; ++i) std::memmove(cell(i, ghost), cell(i, interior), C * 8);
  }
  for (int g = 0; g < ng; ++g) {
    int64_t mirror = 2 * ng - 1 - g;
    std::memmove(cell(g, 0), cell(mirror, 0), N * C * 8);
  }
  for (int g = 0; g < ng; ++g) {
    int64_t interior = M - 2 * ng + g, ghost = M - 1 - g;
    std::memmove(cell(ghost, 0), cell(interior, 0), N * C * 8);
  }
}

// Rie_prob_2d_rs.py:42-120 apply_bc_reflecting.  The reference names the axis-1
// extent `m` and the axis-0 extent `n` and indexes axis 0 with `m`; for M != N
// that raises IndexError in numpy, so only square arrays are accepted here
// (return 1 otherwise).  C must be 8 (the sign masks have 8 entries).
int orc_bc_reflecting(double* q, int64_t M, int64_t N, int64_t C) {
  if (M != N || C != 8) return 1;
  static const double SY[8] = {1, 1, -1, 1, 1, 1, -1, 1};
  static const double SX[8] = {1, -1, 1, 1, 1, -1, 1, 1};
  static const double SC[8] = {1, -1, -1, 1, 1, -1, -1, 1};
  const int ng = 3;
  const int64_t m = N, n = M;  // as in the reference: m = shape[1], n = shape[0]
  auto cell = [&](int64_t i, int64_t j) { return q + (i * N + j) * C; };
  auto copy_row_range = [&](int64_t dst_i, int64_t src_i, int64_t j0, int64_t j1, const double* s) {
    j1 = std::min(j1, N);
    std::vector<double> tmp;
    for (int64_t j = j0; j < j1; ++j)
      for (int64_t k = 0; k < C; ++k) tmp.push_back(cell(src_i, j)[k] * s[k]);
    size_t t = 0;
    for (int64_t j = j0; j < j1; ++j)
      for (int64_t k = 0; k < C; ++k) cell(dst_i, j)[k] = tmp[t++];
  };
  auto copy_col_range = [&](int64_t dst_j, int64_t src_j, int64_t i0, int64_t i1, const double* s) {
    i1 = std::min(i1, M);
    std::vector<double> tmp;
    for (int64_t i = i0; i < i1; ++i)
      for (int64_t k = 0; k < C; ++k) tmp.push_back(cell(i, src_j)[k] * s[k]);
    size_t t = 0;
    for (int64_t i = i0; i < i1; ++i)
      for (int64_t k = 0; k < C; ++k) cell(i, dst_j)[k] = tmp[t++];
  };
  for (int g = 0; g < ng; ++g) copy_row_range(g, 2 * ng - 1 - g, ng, n - ng, SY);
  for (int g = 0; g < ng; ++g) copy_row_range(m - 1 - g, m - 2 * ng + g, ng, n - ng, SY);
  for (int g = 0; g < ng; ++g) copy_col_range(g, 2 * ng - 1 - g, ng, m - ng, SX);
  for (int g = 0; g < ng; ++g) copy_col_range(n - 1 - g, n - 2 * ng + g, ng, m - ng, SX);
  for (int gi = 0; gi < ng; ++gi)
    for (int gj = 0; gj < ng; ++gj) {
      int64_t mi = 2 * ng - 1 - gi, mj = 2 * ng - 1 - gj;
      int64_t int_j = n - 2 * ng + gj, gh_j = n - ng + gj;
      int64_t int_i = m - 2 * ng + gi, gh_i = m - ng + gi;
      auto put = [&](int64_t di, int64_t dj, int64_t si, int64_t sj) {
        double tmp[64];
        for (int64_t k = 0; k < C; ++k) tmp[k] = cell(si, sj)[k] * SC[k];
        for (int64_t k = 0; k < C; ++k) cell(di, dj)[k] = tmp[k];
      };
      put(gi, gj, mi, mj);
      put(gi, gh_j, mi, int_j);
      put(gh_i, gj, int_i, mj);
      put(gh_i, gh_j, int_i, int_j);
    }
  return 0;
}

// unitest.py:207-227 apply_bc_refac (oblique-shock / DMR boundary), executed
// statement by statement.  `post` is the 8-channel inflow vector; C must be 8.
void orc_bc_dmr(double* q, int64_t M, int64_t N, int64_t C, int64_t nx, int64_t ny, int64_t bound, const double* post) {
  auto cell = [&](int64_t i, int64_t j) { return q + (i * N + j) * C; };
  for (int i = 0; i < 3; ++i) {
    for (int64_t j = 0; j < N; ++j) std::memcpy(cell(i, j), post, C * 8);
    for (int64_t r = 0; r < M; ++r) std::memmove(cell(r, ny + 3 + i), cell(r, ny + 2), C * 8);
    std::memmove(cell(nx + 3 + i, 0), cell(nx + 2, 0), N * C * 8);
    for (int64_t r = 0; r < std::min<int64_t>(bound + 1, M); ++r) std::memcpy(cell(r, i), post, C * 8);
    for (int64_t r = bound + 1; r < std::min<int64_t>(bound + 10, M); ++r) std::memmove(cell(r, i), cell(r, 3), C * 8);
    for (int64_t r = bound + 10; r < M; ++r) {
      std::memmove(cell(r, i), cell(r, 5 - i), C * 8);
      cell(r, i)[2] *= -1.0;
      cell(r, i)[6] *= -1.0;
    }
  }
}

// Rie_prob_2d_rs.py:157-163 _sync_primitives (channels 4..7 = rho_safe, u, v, p)
void orc_sync_primitives(double* q, int64_t M, int64_t N, int64_t C, double gamma) {
  A3<double> uc = dense4(q, M, N, C);
  A2<double> P, A, R, U, V, H;
  con2primi(uc, gamma, P, A, R, U, V, H);
  for (int64_t i = 0; i < M; ++i)
    for (int64_t j = 0; j < N; ++j) {
      double* c = q + (i * N + j) * C;
      c[4] = R.at(i, j); c[5] = U.at(i, j); c[6] = V.at(i, j); c[7] = P.at(i, j);
    }
}

// Rie_prob_2d_rs.py:311-319 _cfl_dt (returns c_max + 1e-16; the caller forms
// dt = CFL*dx / that and clips it to the remaining time).
double orc_cfl_cmax(const double* q, int64_t M, int64_t N, int64_t C, int64_t nx, int64_t ny, double gamma) {
  (void)M;
  double cmax = -INFINITY;
  bool nan = false;
  for (int64_t i = 3; i < 3 + nx; ++i)
    for (int64_t j = 3; j < 3 + ny; ++j) {
      const double* c = q + (i * N + j) * C;
      double speed = std::sqrt(c[5] * c[5] + c[6] * c[6]);
      // np.maximum propagates NaN (a NaN density makes the wave speed NaN)
      const double rden = c[0] != c[0] ? c[0] : std::fmax(c[0], 1e-14);
      double cs = std::sqrt(gamma * c[7] / rden);
      double x = cs + speed;
      if (x != x) nan = true;
      if (x > cmax) cmax = x;
    }
  if (nan) return NAN;
  return cmax + 1e-16;
}

// One SSP-RK3 step of Rie_prob_2d_rs.py:169-207 (bc_kind 0: apply_bc_zero_gradient,
// including the in-place fill of the input) or of double_mach_reflection.py:97-134
// (bc_kind 1: apply_bc_refac with `bound` and `post`).  q (M, N, 8) is updated in
// place to q_next.
int orc_rk3_step(double* q, int64_t M, int64_t N, int64_t C, int64_t nx, int64_t ny, double dx, double dt,
                 double gamma, int force_hlle, double jp_lo, double jp_hi, int cons, int bc_kind, int64_t bound,
                 const double* post) {
  if (C != 8 || M != nx + 6 || N != ny + 6) return 1;
  auto bc = [&](double* a) {
    if (bc_kind == 0) orc_bc_transmissive(a, M, N, C);
    else orc_bc_dmr(a, M, N, C, nx, ny, bound, post);
  };
  const size_t tot = (size_t)(M * N * C);
  const double third = 1.0 / 3.0, two_third = 2.0 / 3.0;
  auto residual = [&](const double* a) {
    A3<double> uc = dense4(a, M, N, C);
    return l_local<double>(uc, dx, gamma, force_hlle != 0, jp_lo, jp_hi, cons != 0);
  };
  if (bc_kind == 0) bc(q);
  A3<double> l0 = residual(q);
  std::vector<double> q1(q, q + tot);
  for (int64_t i = 0; i < nx; ++i)
    for (int64_t j = 0; j < ny; ++j)
      for (int k = 0; k < 4; ++k) {
        size_t e = (size_t)(((i + 3) * N + (j + 3)) * C + k);
        q1[e] = q[e] + dt * l0.at(i, j, k);
      }
  bc(q1.data());
  if (bc_kind == 0) { orc_sync_primitives(q1.data(), M, N, C, gamma); bc(q1.data()); }
  A3<double> l1 = residual(q1.data());
  std::vector<double> q2(q, q + tot);
  for (int64_t i = 0; i < nx; ++i)
    for (int64_t j = 0; j < ny; ++j)
      for (int k = 0; k < 4; ++k) {
        size_t e = (size_t)(((i + 3) * N + (j + 3)) * C + k);
        q2[e] = 0.75 * q[e] + 0.25 * q1[e] + (0.25 * dt) * l1.at(i, j, k);
      }
  bc(q2.data());
  if (bc_kind == 0) { orc_sync_primitives(q2.data(), M, N, C, gamma); bc(q2.data()); }
  A3<double> l2 = residual(q2.data());
  std::vector<double> qn(q, q + tot);
  for (int64_t i = 0; i < nx; ++i)
    for (int64_t j = 0; j < ny; ++j)
      for (int k = 0; k < 4; ++k) {
        size_t e = (size_t)(((i + 3) * N + (j + 3)) * C + k);
        qn[e] = third * q[e] + two_third * q2[e] + (two_third * dt) * l2.at(i, j, k);
      }
  bc(qn.data());
  orc_sync_primitives(qn.data(), M, N, C, gamma);
  bc(qn.data());
  std::memcpy(q, qn.data(), tot * 8);
  return 0;
}

}  // extern "C"
