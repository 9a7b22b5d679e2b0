// Kernels of the residual L(U) and of the SSP-RK3 step around it.
//
// Data layout.  The caller's state is a strided 3-D array (i, j, channel)
// addressed as p[i*s0 + j*s1 + k*s2] -- the reference's (nx+6, ny+6, C) C-order
// array (s0 = (ny+6)*C, s1 = C, s2 = 1) or the solver's structure-of-arrays
// planes (s0 = ny+6, s1 = 1, s2 = plane).  j is the contiguous axis and maps to
// threadIdx.x.  Intermediate face data live in workspace planes of one
// component each (`Planes`), so every warp load and store is a contiguous run.
//
// Residual pipeline for one direction (x shown; y swaps the roles of i and j):
//   pass1   (m-5) x n   faces x columns : normal WENO5 (char or cons) -> q_l, q_r
//   pass2   (m-5) x (n-6) faces        : transverse 2-point Gauss WENO of q_l,
//           q_r, Euler fluxes of the four Gauss states, face averages (the FAST
//           HLLE takes their doubles, the Gauss-point sums), then the HLLE
//           flux, or HLLC + HLLE + mean pressure for the sensor blend
//   blend   (sensor blend only)        : pressure-gradient weight, F
//   residual (m-6) x (n-6) cells       : -(dF/dx + dG/dy), optionally fused
//           with the SSP-RK3 stage combination.
#pragma once

#include "euler_math.cuh"
#include "step_ctl.h"

namespace weno {
inline namespace WENO_TU_NS {

template <class T>
struct CView {
  const T* p;
  int64_t s0, s1, s2;
  __device__ __forceinline__ T at(int64_t i, int64_t j, int k) const { return p[i * s0 + j * s1 + k * s2]; }
};

// A set of planes: component k, element (r, c) at p[k*ps + r*ld + c].
template <class T>
struct Planes {
  T* p;
  int64_t ps, ld;
  __device__ __forceinline__ T& at(int k, int64_t r, int64_t c) const { return p[k * ps + r * ld + c]; }
};

// ---------------------------------------------------------------------------
// Pass 1 (weno.rs:390-454 characteristic, weno.rs:654-717 component-wise)
// ---------------------------------------------------------------------------
template <class T, bool FAST, bool Y, bool CHAR>
__global__ void __launch_bounds__(128) k_pass1(CView<T> u, int64_t rows, int64_t cols, T gamma, Planes<T> PL,
                                                Planes<T> PR, T weps) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (row >= rows || col >= cols) return;
  T c[6][4];
#pragma unroll
  for (int s = 0; s < 6; ++s)
#pragma unroll
    for (int k = 0; k < 4; ++k) c[s][k] = Y ? u.at(row, col + s, k) : u.at(row + s, col, k);
  T ql[4], qr[4];
  if constexpr (std::is_same<T, df64>::value) {
    // df64 has the float exponent range: a face whose stencil holds a tiny
    // density or a huge value (near vacuum the characteristic projection scales
    // by 1/(rho*c)) is reconstructed in native double instead.
    bool safe = true;
#pragma unroll
    for (int s = 0; s < 6; ++s) {
      safe = safe && c[s][0].hi > 1e-6f;
#pragma unroll
      for (int k = 0; k < 4; ++k) safe = safe && fabsf(c[s][k].hi) < 1e15f;
    }
    if (safe) {
      pass1_face<T, FAST, Y, CHAR>(c, gamma, ql, qr, weps);
    } else {
      double cd[6][4], l[4], r[4];
#pragma unroll
      for (int s = 0; s < 6; ++s)
#pragma unroll
        for (int k = 0; k < 4; ++k) cd[s][k] = (double)c[s][k];
      pass1_face<double, FAST, Y, CHAR>(cd, (double)gamma, l, r, (double)weps);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        ql[k] = T(l[k]);
        qr[k] = T(r[k]);
      }
    }
  } else {
    pass1_face<T, FAST, Y, CHAR>(c, gamma, ql, qr, weps);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    PL.at(k, row, col) = ql[k];
    PR.at(k, row, col) = qr[k];
  }
}

// Component-wise pass 1, FAST double: two neighbouring faces per thread along
// the sweep (rows for x, columns for y), whose seven cells and shared
// reconstructions about the middle cell serve both (weno5_lr_fast_two; the
// same bits as one face per thread).
template <bool Y>
__global__ void __launch_bounds__(128) k_pass1_cons2(CView<double> u, int64_t rows, int64_t cols,
                                                      Planes<double> PL, Planes<double> PR, double weps) {
  int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t row = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if constexpr (Y) col *= 2;
  else row *= 2;
  if (row >= rows || col >= cols) return;
  const bool two = Y ? (col + 1 < cols) : (row + 1 < rows);
  const int64_t rowB = Y ? row : row + 1, colB = Y ? col + 1 : col;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double v[7];
#pragma unroll
    for (int s = 0; s < 6; ++s) v[s] = Y ? u.at(row, col + s, k) : u.at(row + s, col, k);
    // the seventh cell exists only when face B does
    v[6] = two ? (Y ? u.at(row, col + 6, k) : u.at(row + 6, col, k)) : v[5];
    double lA, rA, lB, rB;
    weno5_lr_fast_two(v[0], v[1], v[2], v[3], v[4], v[5], v[6], weps, lA, rA, lB, rB);
    PL.at(k, row, col) = lA;
    PR.at(k, row, col) = rA;
    if (two) {
      PL.at(k, rowB, colB) = lB;
      PR.at(k, rowB, colB) = rB;
    }
  }
}

// ---------------------------------------------------------------------------
// Pass 2 (weno.rs:460-501 / :587-631) + Riemann solver (riemann.rs)
// ---------------------------------------------------------------------------
enum Pass2Out : int {
  P2_STATES = 0,  // q_l, f_l, q_r, f_r as four dense (rows, cols, 4) arrays
  P2_HLLE = 1,    // HLLE flux planes F[4]
  P2_BLEND = 2,   // HLLC planes Fc[4], HLLE planes Fe[4], mean pressure plane
};

struct Pass2Dst {
  void* a;  // P2_STATES: q_l ; P2_HLLE: F planes ; P2_BLEND: Fc planes
  void* b;  // P2_STATES: f_l ;                      P2_BLEND: Fe planes
  void* c;  // P2_STATES: q_r ;                      P2_BLEND: pbar plane
  void* d;  // P2_STATES: f_r
  int64_t ps, ld;
};

template <class T, bool FAST, bool Y>
__device__ __forceinline__ void gq_face(const Planes<T>& P, int64_t row, int64_t col, T q1[4], T q2[4], T weps) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    T s[5];
#pragma unroll
    for (int t = 0; t < 5; ++t) s[t] = Y ? P.at(k, row + 1 + t, col) : P.at(k, row, col + 1 + t);
    weno5_gq_pair<T, FAST>(s[0], s[1], s[2], s[3], s[4], q1[k], q2[k], weps);
  }
}

// The Riemann solver and the stores of one pass-2 face (row, col).
// S = 2 (FAST, P2_HLLE): the states and fluxes are twice the face averages.
template <class T, bool FAST, bool Y, int OUT, int S = 1>
__device__ __forceinline__ void pass2_emit(const T ql[4], const T fl[4], const T qr[4], const T fr[4], T gamma,
                                           const Pass2Dst& dst, int64_t row, int64_t col, int64_t cols) {
  static_assert(S == 1 || OUT == P2_HLLE, "doubled states feed the HLLE flux only");
  const int64_t e = row * dst.ld + col;
  if constexpr (OUT == P2_STATES) {
    const int64_t o = (row * cols + col) * 4;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      static_cast<T*>(dst.a)[o + k] = ql[k];
      static_cast<T*>(dst.b)[o + k] = fl[k];
      static_cast<T*>(dst.c)[o + k] = qr[k];
      static_cast<T*>(dst.d)[o + k] = fr[k];
    }
  } else {
    const RiemannPre<T, FAST, Y> r = riemann_pre<T, FAST, Y, S>(ql, qr, gamma);
    T F[4];
    hlle_flux<T, FAST, Y, S>(r, ql, fl, qr, fr, F);
    if constexpr (OUT == P2_HLLE) {
#pragma unroll
      for (int k = 0; k < 4; ++k) static_cast<T*>(dst.a)[k * dst.ps + e] = F[k];
    } else {
      T G[4];
      hllc_flux<T, FAST, Y>(r, ql, fl, qr, fr, G);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        static_cast<T*>(dst.a)[k * dst.ps + e] = G[k];
        static_cast<T*>(dst.b)[k * dst.ps + e] = F[k];
      }
      // con2primi pressure of q_l and q_r is the clamped p of the solver
      // preamble (utils.rs:28 == riemann.rs:33-36).
      static_cast<T*>(dst.c)[e] = T(0.5) * (r.p_l + r.p_r);
    }
  }
}

template <class T, bool FAST, bool Y, int OUT>
__global__ void __launch_bounds__(128) k_pass2(Planes<T> PL, Planes<T> PR, int64_t rows, int64_t cols, T gamma,
                                                Pass2Dst dst, T weps) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (row >= rows || col >= cols) return;
  T ql[4], qr[4], fl[4], fr[4];
  {
    T a1[4], a2[4], f1[4], f2[4];
    gq_face<T, FAST, Y>(PL, row, col, a1, a2, weps);
    euler_flux_pair<T, FAST, Y>(a1, a2, gamma, f1, f2);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      fl[k] = T(0.5) * (f1[k] + f2[k]);
      ql[k] = T(0.5) * (a1[k] + a2[k]);
    }
    gq_face<T, FAST, Y>(PR, row, col, a1, a2, weps);
    euler_flux_pair<T, FAST, Y>(a1, a2, gamma, f1, f2);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      fr[k] = T(0.5) * (f2[k] + f1[k]);
      qr[k] = T(0.5) * (a1[k] + a2[k]);
    }
  }
  pass2_emit<T, FAST, Y, OUT>(ql, fl, qr, fr, gamma, dst, row, col, cols);
}

// Face-averaged states and fluxes of two neighbouring faces (along the
// transverse direction) from one side's pass-1 planes, FAST arithmetic.  SUM:
// twice the averages (the Gauss-point sums), for the doubled-state HLLE.
template <class T, bool Y, bool SUM = false>
__device__ __forceinline__ void gq_side_two(const Planes<T>& P, int64_t row, int64_t col, T gamma, T weps, T qA[4],
                                            T fA[4], T qB[4], T fB[4]) {
  T a1A[4], a2A[4], a1B[4], a2B[4];
  if constexpr (is_f32<T>) {
    // components (0,1) and (2,3) as packed pairs on the FP32x2 instructions
#pragma unroll
    for (int k = 0; k < 4; k += 2) {
      f32x2 v[6];
#pragma unroll
      for (int t = 0; t < 6; ++t)
        v[t] = Y ? f32x2(P.at(k, row + 1 + t, col), P.at(k + 1, row + 1 + t, col))
                 : f32x2(P.at(k, row, col + 1 + t), P.at(k + 1, row, col + 1 + t));
      f32x2 raA, rbA, raB, rbB;
      weno5_gq_two<f32x2>(v[0], v[1], v[2], v[3], v[4], v[5], f32x2(weps), raA, rbA, raB, rbB);
      a1A[k] = raA.v.x, a1A[k + 1] = raA.v.y, a2A[k] = rbA.v.x, a2A[k + 1] = rbA.v.y;
      a1B[k] = raB.v.x, a1B[k + 1] = raB.v.y, a2B[k] = rbB.v.x, a2B[k + 1] = rbB.v.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      T v[6];
#pragma unroll
      for (int t = 0; t < 6; ++t) v[t] = Y ? P.at(k, row + 1 + t, col) : P.at(k, row, col + 1 + t);
      weno5_gq_two<T>(v[0], v[1], v[2], v[3], v[4], v[5], weps, a1A[k], a2A[k], a1B[k], a2B[k]);
    }
  }
  const T h = SUM ? T(1.0) : T(0.5);
  T f1[4], f2[4];
  euler_flux_pair<T, true, Y>(a1A, a2A, gamma, f1, f2);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    fA[k] = SUM ? f1[k] + f2[k] : h * (f1[k] + f2[k]);
    qA[k] = SUM ? a1A[k] + a2A[k] : h * (a1A[k] + a2A[k]);
  }
  euler_flux_pair<T, true, Y>(a1B, a2B, gamma, f1, f2);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    fB[k] = SUM ? f1[k] + f2[k] : h * (f1[k] + f2[k]);
    qB[k] = SUM ? a1B[k] + a2B[k] : h * (a1B[k] + a2B[k]);
  }
}

// FAST pass 2 with two faces per thread along the transverse direction
// (columns for the x sweep, rows for the y sweep): the six transverse values
// of each component serve both faces, whose Gauss-point reconstructions share
// their first and second differences.
template <class T, bool Y, int OUT>
__global__ void __launch_bounds__(128) k_pass2_two(Planes<T> PL, Planes<T> PR, int64_t rows, int64_t cols, T gamma,
                                                    Pass2Dst dst, T weps) {
  int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t row = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if constexpr (Y) row *= 2;
  else col *= 2;
  if (row >= rows || col >= cols) return;
  const bool two = Y ? (row + 1 < rows) : (col + 1 < cols);
  // the HLLE flux takes the Gauss-point sums (twice the face averages)
  constexpr bool SUM = OUT == P2_HLLE;
  constexpr int S = SUM ? 2 : 1;
  T qlA[4], flA[4], qlB[4], flB[4], qrA[4], frA[4], qrB[4], frB[4];
  gq_side_two<T, Y, SUM>(PL, row, col, gamma, weps, qlA, flA, qlB, flB);
  gq_side_two<T, Y, SUM>(PR, row, col, gamma, weps, qrA, frA, qrB, frB);
  pass2_emit<T, true, Y, OUT, S>(qlA, flA, qrA, frA, gamma, dst, row, col, cols);
  if (two)
    pass2_emit<T, true, Y, OUT, S>(qlB, flB, qrB, frB, gamma, dst, Y ? row + 1 : row, Y ? col : col + 1, cols);
}

// Riemann solver on caller-provided dense (rows, cols, 4) face arrays
// (hllc_x_rs_py & co, lib.rs:54-132).  KIND 0: HLLC -> out dense;
// KIND 1: HLLE -> out dense; KIND 2: HLLC, HLLE and mean pressure -> planes
// for k_blend.
template <class T, bool FAST, bool Y, int KIND>
__global__ void __launch_bounds__(128) k_riemann(const T* QL, const T* FL, const T* QR, const T* FR, int64_t rows,
                                                  int64_t cols, T gamma, T* out, Planes<T> Fc, Planes<T> Fe,
                                                  Planes<T> Pbar) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (row >= rows || col >= cols) return;
  const int64_t o = (row * cols + col) * 4;
  T ql[4], qr[4], fl[4], fr[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    ql[k] = QL[o + k]; fl[k] = FL[o + k]; qr[k] = QR[o + k]; fr[k] = FR[o + k];
  }
  const RiemannPre<T, FAST, Y> r = riemann_pre<T, FAST, Y>(ql, qr, gamma);
  T F[4];
  if constexpr (KIND == 0) {
    hllc_flux<T, FAST, Y>(r, ql, fl, qr, fr, F);
#pragma unroll
    for (int k = 0; k < 4; ++k) out[o + k] = F[k];
  } else if constexpr (KIND == 1) {
    hlle_flux<T, FAST, Y>(r, ql, fl, qr, fr, F);
#pragma unroll
    for (int k = 0; k < 4; ++k) out[o + k] = F[k];
  } else {
    T G[4];
    hllc_flux<T, FAST, Y>(r, ql, fl, qr, fr, G);
    hlle_flux<T, FAST, Y>(r, ql, fl, qr, fr, F);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      Fc.at(k, row, col) = G[k];
      Fe.at(k, row, col) = F[k];
    }
    Pbar.at(0, row, col) = T(0.5) * (r.p_l + r.p_r);
  }
}

// ---------------------------------------------------------------------------
// Sensor blend (riemann.rs:352-410 shock_sensor_grad_p and riemann.rs:412-448).
// The derivative spacing is 1/min(rows, cols) of the face array, with one-sided
// differences (still divided by 2*dx) on its edges.  rows, cols >= 2.
// Output: planes (DENSE = false) or a dense (rows, cols, 4) array.
// ---------------------------------------------------------------------------
template <class T, bool FAST, bool DENSE>
__global__ void __launch_bounds__(128) k_blend(Planes<T> Fc, Planes<T> Fe, Planes<T> Pbar, int64_t rows,
                                                int64_t cols, T jp_lo, T jp_hi, T* out, Planes<T> Fout) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (row >= rows || col >= cols) return;
  const int64_t min_dim = rows < cols ? rows : cols;
  const T dx = T(1.0) / T((double)min_dim);
  const T two_dx = T(2.0) * dx;
  const int64_t ra = row == 0 ? 0 : (row == rows - 1 ? rows - 2 : row - 1);
  const int64_t rb = row == 0 ? 1 : (row == rows - 1 ? rows - 1 : row + 1);
  const int64_t ca = col == 0 ? 0 : (col == cols - 1 ? cols - 2 : col - 1);
  const int64_t cb = col == 0 ? 1 : (col == cols - 1 ? cols - 1 : col + 1);
  const T p = Pbar.at(0, row, col);
  const T dpdx = qdiv<T, FAST>(Pbar.at(0, rb, col) - Pbar.at(0, ra, col), two_dx);
  const T dpdy = qdiv<T, FAST>(Pbar.at(0, row, cb) - Pbar.at(0, row, ca), two_dx);
  const T w = sensor_weight<T, FAST>(dpdx, dpdy, p, jp_lo, jp_hi);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T f = w * Fc.at(k, row, col) + (T(1.0) - w) * Fe.at(k, row, col);
    if constexpr (DENSE) out[(row * cols + col) * 4 + k] = f;
    else Fout.at(k, row, col) = f;
  }
}

// ---------------------------------------------------------------------------
// Residual (riemann.rs:513-540) fused with the SSP-RK3 stage combination of
// Rie_prob_2d_rs.py:183-202 in numpy's evaluation order:
//   STAGE 0: out[i,j,k] dense = L                       (l_local_py)
//   STAGE 1: q1 = q + dt*L
//   STAGE 2: q2 = (0.75*q + 0.25*q1) + (0.25*dt)*L
//   STAGE 3: qn = ((1/3)*q + (2/3)*q2) + ((2/3)*dt)*L
// Fx planes are (m-5) x (n-6) faces, Fy planes (m-6) x (n-5).
// ---------------------------------------------------------------------------

template <class T, bool FAST, int STAGE>
__global__ void __launch_bounds__(128) k_residual(Planes<T> Fx, Planes<T> Fy, int64_t rows, int64_t cols, T dx,
                                                   T* out, Planes<T> Qn, Planes<T> Qs, Planes<T> Qo,
                                                   const StepCtl* ctl) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (row >= rows || col >= cols) return;
  if constexpr (STAGE > 0) {
    if (!ctl->active) return;
  }
  T L[4];
  if constexpr (FAST) {
    // one reciprocal instead of eight divides (riemann.rs:527 divides both
    // differences by the same dx)
    const T idx = qrcp<T, FAST>(dx);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      L[k] = -((Fx.at(k, row + 1, col) - Fx.at(k, row, col)) + (Fy.at(k, row, col + 1) - Fy.at(k, row, col))) * idx;
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const T dfdx = (Fx.at(k, row + 1, col) - Fx.at(k, row, col)) / dx;
      const T dgdy = (Fy.at(k, row, col + 1) - Fy.at(k, row, col)) / dx;
      L[k] = -(dfdx + dgdy);
    }
  }
  if constexpr (STAGE == 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k) out[(row * cols + col) * 4 + k] = L[k];
  } else {
    const double dt = ctl->dt;
    const int64_t r = row + 3, c = col + 3;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const T qn = Qn.at(k, r, c);
      T v;
      if constexpr (STAGE == 1) {
        v = qn + T(dt) * L[k];
      } else if constexpr (STAGE == 2) {
        v = T(0.75) * qn + T(0.25) * Qs.at(k, r, c) + T(0.25 * dt) * L[k];
      } else {
        v = T(1.0 / 3.0) * qn + T(2.0 / 3.0) * Qs.at(k, r, c) + T((2.0 / 3.0) * dt) * L[k];
      }
      Qo.at(k, r, c) = v;
    }
  }
}

// ---------------------------------------------------------------------------
// Boundary fills, in place, on NC channels of a strided array (the solver's
// 4 conserved planes, or the driver's 8-channel array).  Each ghost value
// depends only on interior values, so the fill is one pointwise pass.
// Requires nx, ny >= 3.
// ---------------------------------------------------------------------------
template <class T>
struct S3 {
  T* p;
  int64_t s0, s1, s2;
  __device__ __forceinline__ T& at(int64_t i, int64_t j, int k) const { return p[i * s0 + j * s1 + k * s2]; }
};

// Rie_prob_2d_rs.py:123-152 apply_bc_zero_gradient: ghost g <- 5-g on the low
// side and the mirror about the last interior cell on the high side; the
// corners end up mirrored in both directions.
__device__ __forceinline__ int64_t mirror_idx(int64_t i, int64_t M) {
  if (i < 3) return 5 - i;
  if (i >= M - 3) return 2 * M - 7 - i;
  return i;
}

template <class T, int NC>
__global__ void k_bc_transmissive(S3<T> Q, int64_t M, int64_t N, const StepCtl* ctl) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= M || j >= N) return;
  if (ctl && !ctl->active) return;
  const int64_t si = mirror_idx(i, M), sj = mirror_idx(j, N);
  if (si == i && sj == j) return;
#pragma unroll
  for (int k = 0; k < NC; ++k) Q.at(i, j, k) = Q.at(si, sj, k);
}

// The inflow state of the oblique-shock boundary, all eight driver channels.
template <class T>
struct Post8 {
  T v[8];
};

// unitest.py:207-227 apply_bc_refac, the oblique-shock / double-Mach boundary:
// rows 0..2 take the inflow state; top ghost columns copy column ny+2; right
// ghost rows copy row nx+2; bottom ghost columns take the inflow state for rows
// <= bound, a copy of column 3 for rows bound+1..bound+9 and a mirror with the
// normal momentum (and v) negated beyond.  The reference fills these with
// sequential numpy slices; right ghost row nx+3+k takes its first k
// bottom-ghost values from row nx+2's band and the rest from its own band,
// which the pointwise form below reproduces.
template <class T, int NC>
__global__ void k_bc_dmr(S3<T> Q, int64_t nx, int64_t ny, int64_t bound, Post8<T> post, const StepCtl* ctl) {
  const int64_t M = nx + 6, N = ny + 6;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= M || j >= N) return;
  if (ctl && !ctl->active) return;
  T v[NC];
  if (i < 3) {
#pragma unroll
    for (int k = 0; k < NC; ++k) v[k] = post.v[k];
  } else if (j >= ny + 3) {
    const int64_t s = i < nx + 3 ? i : nx + 2;
#pragma unroll
    for (int k = 0; k < NC; ++k) v[k] = Q.at(s, ny + 2, k);
  } else if (j < 3) {
    const int64_t s = i < nx + 3 ? i : nx + 2;
    const int64_t band_row = (i >= nx + 3 && j < i - nx - 3) ? nx + 2 : i;
    if (band_row <= bound) {
#pragma unroll
      for (int k = 0; k < NC; ++k) v[k] = post.v[k];
    } else if (band_row <= bound + 9) {
#pragma unroll
      for (int k = 0; k < NC; ++k) v[k] = Q.at(s, 3, k);
    } else {
#pragma unroll
      for (int k = 0; k < NC; ++k) v[k] = Q.at(s, 5 - j, k);
      v[2] = -v[2];
      if constexpr (NC == 8) v[6] = -v[6];
    }
  } else if (i >= nx + 3) {
#pragma unroll
    for (int k = 0; k < NC; ++k) v[k] = Q.at(nx + 2, j, k);
  } else {
    return;
  }
#pragma unroll
  for (int k = 0; k < NC; ++k) Q.at(i, j, k) = v[k];
}

// ---------------------------------------------------------------------------
// CFL wave-speed maximum (Rie_prob_2d_rs.py:311-319): max over interior cells
// of sqrt(u^2+v^2) + sqrt(gamma*p/max(rho, 1e-14)), with u, v, p the primitive
// channels as con2primi writes them (utils.rs:22-29) and rho the raw density.
// AOS = true reads the primitives from channels 5, 6, 7 of a (M, N, C>=8)
// array instead (the first step of a run starting from the driver's array).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* a, double x) {
  atomicMax(a, (unsigned long long)__double_as_longlong(x));
}

// np.maximum(rho, 1e-14) of the driver's CFL (Rie_prob_2d_rs.py:314): NaN in,
// NaN out (fmax would return the bound).
template <class T>
__device__ __forceinline__ T np_maximum(T x, T c) { return x != x ? x : fmax(x, c); }

// np.max propagates NaN (and inf dominates), so a non-finite wave speed makes
// the maximum non-finite and dt follows, as in the driver; NaN's bit pattern
// orders above +inf under the unsigned atomicMax.
__device__ __forceinline__ double nan_max(double a, double b) { return (a != a || b != b) ? __longlong_as_double(0x7ff8000000000000ll) : fmax(a, b); }

template <class T, bool AOS>
__global__ void __launch_bounds__(256) k_cfl_max(CView<T> q, int64_t nx, int64_t ny, T gamma, StepCtl* ctl) {
  if (!ctl->active || ctl->cmax_preset) return;
  double best = 0.0;
  bool nonpos = false;  // FP64 positivity check of the recovered density and pressure
  const int64_t total = nx * ny;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / ny + 3, j = e % ny + 3;
    if constexpr (!AOS && std::is_same<T, float>::value) {
      // FP32 state: the wave speed in FP32 (the state's own precision; the
      // maximum and dt stay FP64), the positivity of the recovered density and
      // pressure in FP64 without a divide: rho > 0 and E rho - |m|^2/2 > 0.
      const float r0 = q.at(i, j, 0), m1 = q.at(i, j, 1), m2 = q.at(i, j, 2), E = q.at(i, j, 3);
      const double rd = r0, m1d = m1, m2d = m2;
      if (!(rd > 0.0) || !((double)E * rd - 0.5 * (m1d * m1d + m2d * m2d) > 0.0)) nonpos = true;
      const float rho = fmaxf(r0, float(kEps));
      const float ir = __fdividef(1.0f, rho);
      const float uu = m1 * ir, vv = m2 * ir;
      const float pp = fmaxf(((float)gamma - 1.0f) * (E - 0.5f * rho * (uu * uu + vv * vv)), float(kEps));
      const float w = sqrtf(uu * uu + vv * vv) + sqrtf((float)gamma * pp * __fdividef(1.0f, np_maximum(r0, 1e-14f)));
      best = nan_max(best, (double)w);
    } else {
      double uu, vv, pp;
      const double r0 = (double)q.at(i, j, 0);
      if constexpr (AOS) {
        uu = (double)q.at(i, j, 5);
        vv = (double)q.at(i, j, 6);
        pp = (double)q.at(i, j, 7);
      } else {
        const double rho = fmax(r0, kEps);
        uu = (double)q.at(i, j, 1) / rho;
        vv = (double)q.at(i, j, 2) / rho;
        const double praw = ((double)gamma - 1.0) * ((double)q.at(i, j, 3) - 0.5 * rho * (uu * uu + vv * vv));
        pp = fmax(praw, kEps);
        if (!(r0 > 0.0) || !(praw > 0.0)) nonpos = true;
      }
      const double speed = sqrt(uu * uu + vv * vv);
      const double c = sqrt((double)gamma * pp / np_maximum(r0, 1e-14));
      best = nan_max(best, c + speed);
    }
  }
  nonpos = __any_sync(0xffffffffu, nonpos);
  if (nonpos && (threadIdx.x & 31) == 0) atomicOr(&ctl->status, 2);
  for (int off = 16; off > 0; off >>= 1) best = nan_max(best, __shfl_xor_sync(0xffffffffu, best, off));
  __shared__ double sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = sm[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) b = nan_max(b, sm[w]);
    atomic_max_nonneg(&ctl->cmax_bits, b);
    if (!(b < INFINITY)) atomicOr(&ctl->status, 1);
  }
}

// FP64 sums of the four conserved planes over the interior (conservation
// diagnostics); one block-partial per block, added with atomicAdd.
template <class T>
__global__ void __launch_bounds__(256) k_totals(CView<T> q, int64_t nx, int64_t ny, double* out4) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const int64_t total = nx * ny;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / ny + 3, j = e % ny + 3;
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] += (double)q.at(i, j, k);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], off);
    if ((threadIdx.x & 31) == 0) atomicAdd(out4 + k, acc[k]);
  }
}

// dt = CFL*dx / (cmax + 1e-16), clipped to the time left (Rie_prob_2d_rs.py:315-318).
__global__ void k_dt(StepCtl* ctl) {
  if (!ctl->active) return;
  ctl->cmax_preset = 0;
  const double cmax = __longlong_as_double((long long)ctl->cmax_bits) + 1e-16;
  double dt = ctl->cfl_dx / cmax;
  if (ctl->t_final >= 0.0) {
    const double remaining = ctl->t_final - ctl->t;
    if (remaining < dt) dt = remaining;
  }
  ctl->dt = dt;
}

// Start of a run of `add` steps: the loop condition of Rie_prob_2d_rs.py:335.
__global__ void k_run_begin(StepCtl* ctl, double t_final, long long add) {
  ctl->t_final = t_final;
  ctl->max_steps = ctl->steps + add;
  bool go = ctl->steps < ctl->max_steps;
  if (t_final >= 0.0) go = go && (ctl->t < t_final - 1e-12);
  ctl->active = go ? 1 : 0;
}

// End of a step: advance the clock, reset the reduction, decide whether the
// next step runs (Rie_prob_2d_rs.py:335, loop condition T < t_final - 1e-12).
__global__ void k_step_end(StepCtl* ctl) {
  if (!ctl->active) return;
  ctl->t += ctl->dt;
  ctl->steps += 1;
  ctl->cmax_bits = 0ull;
  bool more = ctl->steps < ctl->max_steps;
  if (ctl->t_final >= 0.0) more = more && (ctl->t < ctl->t_final - 1e-12);
  ctl->active = more ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Small element-wise kernels of the drop-in API
// ---------------------------------------------------------------------------
template <class T, bool FAST, bool Y>
__global__ void k_flux(CView<T> q, int64_t rows, int64_t cols, T gamma, T* out) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (row >= rows || col >= cols) return;
  T s[4], f[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) s[k] = q.at(row, col, k);
  euler_flux<T, FAST, Y>(s, gamma, f);
#pragma unroll
  for (int k = 0; k < 4; ++k) out[(row * cols + col) * 4 + k] = f[k];
}

template <class T, bool FAST>
__global__ void k_con2primi(CView<T> q, int64_t rows, int64_t cols, T gamma, T* p, T* a, T* rho, T* u, T* v, T* h) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (row >= rows || col >= cols) return;
  const int64_t e = row * cols + col;
  con2prim<T, FAST>(q.at(row, col, 0), q.at(row, col, 1), q.at(row, col, 2), q.at(row, col, 3), gamma, p[e], a[e],
                    rho[e], u[e], v[e], h[e]);
}

// Solver planes -> the driver's (M, N, 8) array: conserved channels 0..3 and
// the primitive sync of Rie_prob_2d_rs.py:157-163 (rho_safe, u, v, p).
template <class T, bool FAST>
__global__ void k_export_aos8(Planes<T> Q, int64_t M, int64_t N, T gamma, double* out) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= M || j >= N) return;
  const T q0 = Q.at(0, i, j), q1 = Q.at(1, i, j), q2 = Q.at(2, i, j), q3 = Q.at(3, i, j);
  T p, a, rho, u, v, h;
  con2prim<T, FAST>(q0, q1, q2, q3, gamma, p, a, rho, u, v, h);
  double* o = out + (i * N + j) * 8;
  o[0] = (double)q0; o[1] = (double)q1; o[2] = (double)q2; o[3] = (double)q3;
  o[4] = (double)rho; o[5] = (double)u; o[6] = (double)v; o[7] = (double)p;
}

// Caller's strided array (channels 0..3) -> solver planes.
template <class T>
__global__ void k_import_planes(CView<double> q, int64_t M, int64_t N, Planes<T> Q) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= M || j >= N) return;
#pragma unroll
  for (int k = 0; k < 4; ++k) Q.at(k, i, j) = (T)q.at(i, j, k);
}

}  // inline namespace WENO_TU_NS
}  // namespace weno
