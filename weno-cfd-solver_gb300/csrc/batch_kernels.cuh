// Batched solver: many independent 2-D problems of uneven size stepped together.
//
// Pool layout.  Every solve stores only its interior cells, as four conserved
// planes of nx rows (row pitch `ld` = ny rounded up to 16 bytes, plane stride
// `ps`) at element offset `off` of a packed pool; the pool exists three times
// (current state, stage 1, stage 2) in one allocation, with identical offsets,
// so one 4-D tensor map per solve (column, row, plane, pool) addresses all of
// it.  Ghost cells are never stored: after the tile is staged, each ghost cell
// of the tile is filled from the interior cell (or inflow constant) the
// boundary fill would have copied there (Rie_prob_2d_rs.py:123-152,
// unitest.py:207-227), so the fill costs no pass of its own.
//
// Work.  The unit is a tile of TX x TY interior cells of one solve.  A packed
// tile list (solve, i0, j0) covers every active solve; one persistent kernel
// per RK stage walks it.  A CTA stages the tile plus its halo into shared
// memory with one TMA box load (cp.async.bulk.tensor, completion on an
// mbarrier), runs pass 1 (normal WENO5), pass 2 (Gauss-quadrature WENO, fluxes,
// Riemann solver), the sensor blend and the flux difference fused with the
// SSP-RK3 stage combination, and writes the tile of the next stage state.
// Stage 3 also reduces the new state's wave speed per solve for the next dt.
#pragma once

#include "euler_math.cuh"
#include "step_ctl.h"
#include "tma.cuh"

namespace weno {

struct SolveDesc {
  long long off;  // element offset of plane 0 in each pool
  long long ps;   // plane stride (elements)
  int nx, ny;
  int ld;         // row pitch (elements): ny rounded up to a multiple of 16 bytes
  int bc;         // 0 transmissive (mirror), 1 oblique-shock / DMR segments
  int bound;      // DMR: last row of the inflow segment on the lower boundary
  double dx;      // cell size (dx = dy)
  double post[8]; // DMR inflow state: conserved channels 0..3, primitive channels 4..7
  // Staged tile configuration only: this solve's face workspace, element offsets
  // in the workspace pool (see k_staged_pass1).
  long long w_p1x, w_p1y, w_fx, w_fy;  // plane 0 of each array
  long long s_p1x, s_p1y, s_fx, s_fy;  // plane strides
  int l_p1x, l_p1y;                    // row pitches of P1x and of P1y / Fy (Fx uses ld)
};

struct SolveCtl {
  double t, t_end, dt, cfl_dx;
  unsigned long long cmax_bits;
  int active;      // 0: finished (t >= t_end - 1e-12 or step cap) or not admitted
  int status;      // 1: non-finite wave speed; 4: a tile's staging copy did not land
  long long steps, max_steps;
};

inline namespace WENO_TU_NS {

// Where the boundary fill would take ghost cell (I, J) (padded coordinates)
// from: an interior cell (i, j) with a sign on the normal momentum, or the
// inflow constant.
__device__ __forceinline__ double nan_max_b(double a, double b) {
  return (a != a || b != b) ? __longlong_as_double(0x7ff8000000000000ll) : fmax(a, b);
}

struct GhostSrc {
  int i, j;
  bool post;
  bool flip2;
};

__device__ __forceinline__ GhostSrc resolve_cell(const SolveDesc& d, int I, int J) {
  GhostSrc g{0, 0, false, false};
  const int nx = d.nx, ny = d.ny;
  if (d.bc == 0) {
    const int M = nx + 6, N = ny + 6;
    const int si = I < 3 ? 5 - I : (I >= M - 3 ? 2 * M - 7 - I : I);
    const int sj = J < 3 ? 5 - J : (J >= N - 3 ? 2 * N - 7 - J : J);
    g.i = si - 3;
    g.j = sj - 3;
    return g;
  }
  if (I < 3) {
    g.post = true;
  } else if (J >= ny + 3) {
    g.i = (I < nx + 3 ? I : nx + 2) - 3;
    g.j = ny - 1;
  } else if (J < 3) {
    const int s = I < nx + 3 ? I : nx + 2;
    const int band_row = (I >= nx + 3 && J < I - nx - 3) ? nx + 2 : I;
    if (band_row <= d.bound) {
      g.post = true;
    } else if (band_row <= d.bound + 9) {
      g.i = s - 3;
      g.j = 0;
    } else {
      g.i = s - 3;
      g.j = 2 - J;
      g.flip2 = true;
    }
  } else if (I >= nx + 3) {
    g.i = nx - 1;
    g.j = J - 3;
  } else {
    g.i = I - 3;
    g.j = J - 3;
  }
  return g;
}

template <int TX, int TY, bool BLEND>
struct TileGeom {
  static constexpr int HF = BLEND ? 1 : 0;     // extra face halo for the sensor stencil
  static constexpr int UR = TX + 6 + 2 * HF;   // tile rows incl. halo
  static constexpr int UCV = TY + 6 + 2 * HF;  // tile columns incl. halo
  // The staged box starts at column j0 - 4 (a 16-byte boundary, j0 being a
  // multiple of TY): halo column c of the tile sits at box column c + CO, and
  // the box is TY + 8 columns wide, which is also the shared-memory row pitch.
  static constexpr int CO = 1 - HF;
  static constexpr int UC = TY + 8;
  static constexpr int P1XR = TX + 1 + 2 * HF, P1XC = TY + 4 + 2 * HF;  // pass-1 x faces x columns
  static constexpr int P1YR = TX + 4 + 2 * HF, P1YC = TY + 1 + 2 * HF;  // pass-1 rows x y faces
  static constexpr int P1 = (P1XR * P1XC > P1YR * P1YC) ? P1XR * P1XC : P1YR * P1YC;
  static constexpr int FXR = TX + 1 + 2 * HF, FXC = TY + 2 * HF;  // x faces for the residual (+sensor halo)
  static constexpr int FYR = TX + 2 * HF, FYC = TY + 1 + 2 * HF;
  static constexpr int NF = BLEND ? 9 : 4;    // HLLC[4], HLLE[4], pbar  |  F[4]
  static constexpr int U_ELEMS = 4 * UR * UC;
  static constexpr int P1_ELEMS = 8 * P1;
  static constexpr int FX_ELEMS = NF * FXR * FXC;
  static constexpr int FY_ELEMS = NF * FYR * FYC;
  // x and y face fluxes share one buffer: the x flux difference of every cell
  // is kept in DX (4 x TX x TY) before the y sweep overwrites the faces.
  static constexpr int F_ELEMS = FX_ELEMS > FY_ELEMS ? FX_ELEMS : FY_ELEMS;
  static constexpr int DX_ELEMS = 4 * TX * TY;
  static constexpr int TOTAL = U_ELEMS + P1_ELEMS + F_ELEMS + DX_ELEMS;
};

// Sensor weight at face (fr, fc) of a local face array of R x C entries whose
// global origin is (gr0, gc0) in a global face array of GR x GC entries
// (riemann.rs:352-410: central differences, one-sided on the global edges).
template <class T, bool FAST>
__device__ __forceinline__ T tile_sensor(const T* pbar, int R, int C, int fr, int fc, int gr, int gc, int GR, int GC,
                                         T jp_lo, T jp_hi) {
  const int min_dim = GR < GC ? GR : GC;
  const T dx = T(1.0) / T((double)min_dim);
  const T two_dx = T(2.0) * dx;
  const int ra = gr == 0 ? 0 : (gr == GR - 1 ? -1 : -1);
  const int rb = gr == 0 ? 1 : (gr == GR - 1 ? 0 : 1);
  const int ca = gc == 0 ? 0 : (gc == GC - 1 ? -1 : -1);
  const int cb = gc == 0 ? 1 : (gc == GC - 1 ? 0 : 1);
  (void)R;
  const T p = pbar[fr * C + fc];
  const T dpdx = qdiv<T, FAST>(pbar[(fr + rb) * C + fc] - pbar[(fr + ra) * C + fc], two_dx);
  const T dpdy = qdiv<T, FAST>(pbar[fr * C + fc + cb] - pbar[fr * C + fc + ca], two_dx);
  return sensor_weight<T, FAST>(dpdx, dpdy, p, jp_lo, jp_hi);
}

// Both Gauss-point values of the four components of one face side: `p`
// points at the first of five transverse values of component 0, `ks` is the
// component stride and `ts` the transverse stride.  FAST float runs the
// components as two packed pairs on the FP32x2 instructions.
template <class T, bool FAST>
__device__ __forceinline__ void tile_gq_side(const T* p, int ks, int ts, T weps, T a1[4], T a2[4]) {
  if constexpr (FAST && is_f32<T>) {
#pragma unroll
    for (int k = 0; k < 4; k += 2) {
      const T* u = p + k * ks;
      const T* w = u + ks;
      f32x2 ra, rb;
      weno5_gq_pair<f32x2, true>(f32x2(u[0], w[0]), f32x2(u[ts], w[ts]), f32x2(u[2 * ts], w[2 * ts]),
                                 f32x2(u[3 * ts], w[3 * ts]), f32x2(u[4 * ts], w[4 * ts]), ra, rb, f32x2(weps));
      a1[k] = ra.v.x, a1[k + 1] = ra.v.y, a2[k] = rb.v.x, a2[k + 1] = rb.v.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const T* u = p + k * ks;
      weno5_gq_pair<T, FAST>(u[0], u[ts], u[2 * ts], u[3 * ts], u[4 * ts], a1[k], a2[k], weps);
    }
  }
}

// Riemann solver of one tile face and its store into the face buffer F
// (HLLE flux planes, or HLLC + HLLE + mean pressure for the sensor blend).
// S = 2 (HLLE only): states and fluxes are twice the face averages.
template <class T, bool FAST, bool Y, bool BLEND, int S = 1>
__device__ __forceinline__ void tile_face_flux(const T ql[4], const T fl[4], const T qr[4], const T fr[4], T gamma,
                                               T* F, int FN, int e) {
  static_assert(S == 1 || !BLEND, "doubled states feed the HLLE flux only");
  const RiemannPre<T, FAST, Y> rp = riemann_pre<T, FAST, Y, S>(ql, qr, gamma);
  T H[4];
  hlle_flux<T, FAST, Y, S>(rp, ql, fl, qr, fr, H);
  if constexpr (BLEND) {
    T Gc[4];
    hllc_flux<T, FAST, Y>(rp, ql, fl, qr, fr, Gc);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      F[k * FN + e] = Gc[k];
      F[(4 + k) * FN + e] = H[k];
    }
    F[8 * FN + e] = T(0.5) * (rp.p_l + rp.p_r);
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) F[k * FN + e] = H[k];
  }
}

// One SSP-RK3 stage (1..3) for every tile of the list.  The stage input (pool
// stage-1 of q, q1, q2) is read through each solve's tensor map `tmaps[solve]`;
// Qn is the step's initial state, Qo the output pool.
template <class T, bool FAST, bool CHAR, bool BLEND, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) k_stage_tiles(const SolveDesc* __restrict__ solves, SolveCtl* ctl,
                                                     const int4* __restrict__ tiles, int ntiles,
                                                     const CUtensorMap* tmaps, const T* Qn, T* Qo, int stage,
                                                     T gamma, T jp_lo, T jp_hi, T weps, int skip_tile,
                                                     unsigned long long wait_ns) {
  using G = TileGeom<TX, TY, BLEND>;
  static_assert(G::UC * sizeof(T) % 16 == 0, "box rows must be whole 16-byte units");
  constexpr uint32_t kBoxBytes = (uint32_t)(sizeof(T) * G::U_ELEMS);
  constexpr int S = FAST && !BLEND ? 2 : 1;  // FAST HLLE takes the Gauss-point sums
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* U = reinterpret_cast<T*>(smem_raw);
  T* P1 = U + G::U_ELEMS;
  T* FX = P1 + G::P1_ELEMS;
  T* FY = FX;  // the y faces reuse the x faces' buffer
  T* DXF = FX + G::F_ELEMS;
  __shared__ double red[NT / 32];
  __shared__ uint64_t bar;
  const int tid = threadIdx.x;
  if (tid == 0) {
    tma::mbar_init(&bar, 1);
    tma::fence_mbar_init();
  }
  __syncthreads();
  uint32_t phase = 0;

  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int4 tl = tiles[t];
    const SolveDesc d = solves[tl.x];
    if (!ctl[tl.x].active) continue;  // uniform across the CTA
    const int i0 = tl.y, j0 = tl.z;
    const int nx = d.nx, ny = d.ny;
    const long long ps = d.ps;
    const int HF = G::HF;

    // ---- stage the tile and its halo: one TMA box of (TY+8) x UR x 4 planes
    // from the stage-input pool (stage-1); cells outside the solve read 0 ----
    {
      const CUtensorMap* tm = tmaps + tl.x;
      if (tid == 0) {
        tma::tensormap_acquire(tm);
        if (t != skip_tile) {  // skip_tile >= 0 only under the test hook weno_batch_debug_skip_copy
          tma::mbar_arrive_expect_tx(&bar, kBoxBytes);
          tma::load_4d(U, tm, j0 - 4, i0 - HF - 3, 0, stage - 1, &bar);
        }
      }
      const uint32_t par = phase;
      phase ^= 1u;
      const bool landed = tma::mbar_wait_bounded(&bar, par, wait_ns);
      if (!__syncthreads_and(landed)) {
        // This CTA leaves: flag the solve of this tile and of every later tile
        // it would have walked, so no solve keeps stale tiles with a clean status.
        if (tid == 0)
          for (int t2 = t; t2 < ntiles; t2 += gridDim.x) atomicOr(&ctl[tiles[t2].x].status, 4);
        tma::mbar_wait_bounded(&bar, par, wait_ns);  // let a late copy land before the CTA leaves
        return;
      }
    }
    // ---- ghost cells of the tile from the staged interior ----
    for (int e = tid; e < G::UR * G::UCV; e += NT) {
      const int r = e / G::UCV, c = e % G::UCV;
      const int I = i0 - HF + r, J = j0 - HF + c;  // padded coordinates
      if (I < 0 || I >= nx + 6 || J < 0 || J >= ny + 6) continue;
      if (I >= 3 && I < nx + 3 && J >= 3 && J < ny + 3) continue;
      const GhostSrc g = resolve_cell(d, I, J);
      T v[4];
      if (g.post) {
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = T(d.post[k]);
      } else {
        const int sr = g.i + 3 - (i0 - HF), sc = g.j + 3 - (j0 - HF);
        if (sr < 0 || sr >= G::UR || sc < 0 || sc >= G::UCV) {
          // not reachable for tiles that start inside their solve; kept as a checked fallback
#pragma unroll
          for (int k = 0; k < 4; ++k) v[k] = T(__longlong_as_double(0x7ff8000000000000ll));
          atomicOr(&ctl[tl.x].status, 4);
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) v[k] = U[k * G::UR * G::UC + sr * G::UC + sc + G::CO];
          if (g.flip2) v[2] = -v[2];
        }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) U[k * G::UR * G::UC + r * G::UC + c + G::CO] = v[k];
    }
    __syncthreads();

    // ---- x sweep: pass 1 on faces fi = i0-HF+fr (global face rows 0..nx) ----
    for (int e = tid; e < G::P1XR * G::P1XC; e += NT) {
      const int fr = e / G::P1XC, c = e % G::P1XC;
      const int fi = i0 - HF + fr;
      if (fi < 0 || fi > nx) continue;
      // pass-1 column J = j0+1-HF+c <-> tile column c+1
      T cells[6][4];
#pragma unroll
      for (int s = 0; s < 6; ++s)
#pragma unroll
        for (int k = 0; k < 4; ++k) cells[s][k] = U[k * G::UR * G::UC + (fr + s) * G::UC + c + 1 + G::CO];
      T ql[4], qr[4];
      pass1_face<T, FAST, false, CHAR>(cells, gamma, ql, qr, weps);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        P1[k * G::P1 + e] = ql[k];
        P1[(4 + k) * G::P1 + e] = qr[k];
      }
    }
    __syncthreads();
    // ---- x sweep: pass 2 on faces (fi, jj), jj = j0-HF+fc ----
    for (int e = tid; e < G::FXR * G::FXC; e += NT) {
      const int fr = e / G::FXC, fc = e % G::FXC;
      const int fi = i0 - HF + fr, jj = j0 - HF + fc;
      if (fi < 0 || fi > nx || jj < 0 || jj >= ny) continue;
      T ql[4], qr[4], fl[4], fr_[4];
      {
        T a1[4], a2[4], f1[4], f2[4];
        tile_gq_side<T, FAST>(P1 + fr * G::P1XC + fc, G::P1, 1, weps, a1, a2);
        euler_flux_pair<T, FAST, false>(a1, a2, gamma, f1, f2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          fl[k] = S == 1 ? T(0.5) * (f1[k] + f2[k]) : f1[k] + f2[k];
          ql[k] = S == 1 ? T(0.5) * (a1[k] + a2[k]) : a1[k] + a2[k];
        }
        tile_gq_side<T, FAST>(P1 + 4 * G::P1 + fr * G::P1XC + fc, G::P1, 1, weps, a1, a2);
        euler_flux_pair<T, FAST, false>(a1, a2, gamma, f1, f2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          fr_[k] = S == 1 ? T(0.5) * (f2[k] + f1[k]) : f2[k] + f1[k];
          qr[k] = S == 1 ? T(0.5) * (a1[k] + a2[k]) : a1[k] + a2[k];
        }
      }
      tile_face_flux<T, FAST, false, BLEND, S>(ql, fl, qr, fr_, gamma, FX, G::FXR * G::FXC, e);
    }
    __syncthreads();
    // ---- x flux difference of every cell of the tile (sensor blend of the x faces) ----
    for (int e = tid; e < TX * TY; e += NT) {
      const int il = e / TY, jl = e % TY;
      const int i = i0 + il, j = j0 + jl;
      if (i >= nx || j >= ny) continue;
      const int fxr = il + HF, fxc = jl + HF;  // Fx rows fi = i, i+1
      const int FN = G::FXR * G::FXC;
      T wa = T(1.0), wb = T(1.0);
      if constexpr (BLEND) {
        wa = tile_sensor<T, FAST>(FX + 8 * FN, G::FXR, G::FXC, fxr, fxc, i, j, nx + 1, ny, jp_lo, jp_hi);
        wb = tile_sensor<T, FAST>(FX + 8 * FN, G::FXR, G::FXC, fxr + 1, fxc, i + 1, j, nx + 1, ny, jp_lo, jp_hi);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        T fxa, fxb;
        if constexpr (BLEND) {
          fxa = wa * FX[k * FN + fxr * G::FXC + fxc] + (T(1.0) - wa) * FX[(4 + k) * FN + fxr * G::FXC + fxc];
          fxb = wb * FX[k * FN + (fxr + 1) * G::FXC + fxc] + (T(1.0) - wb) * FX[(4 + k) * FN + (fxr + 1) * G::FXC + fxc];
        } else {
          fxa = FX[k * FN + fxr * G::FXC + fxc];
          fxb = FX[k * FN + (fxr + 1) * G::FXC + fxc];
        }
        if constexpr (FAST) DXF[k * TX * TY + e] = (fxb - fxa) * qrcp<T, FAST>(T(d.dx));
        else DXF[k * TX * TY + e] = (fxb - fxa) / T(d.dx);
      }
    }
    __syncthreads();

    // ---- y sweep: pass 1 on rows I = i0+1-HF+r, faces fj = j0-HF+fc ----
    for (int e = tid; e < G::P1YR * G::P1YC; e += NT) {
      const int r = e / G::P1YC, fc = e % G::P1YC;
      const int I = i0 + 1 - HF + r, fj = j0 - HF + fc;
      if (I < 0 || I >= nx + 6 || fj < 0 || fj > ny) continue;
      T cells[6][4];
#pragma unroll
      for (int s = 0; s < 6; ++s)
#pragma unroll
        for (int k = 0; k < 4; ++k) cells[s][k] = U[k * G::UR * G::UC + (r + 1) * G::UC + fc + s + G::CO];
      T ql[4], qr[4];
      pass1_face<T, FAST, true, CHAR>(cells, gamma, ql, qr, weps);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        P1[k * G::P1 + e] = ql[k];
        P1[(4 + k) * G::P1 + e] = qr[k];
      }
    }
    __syncthreads();
    // ---- y sweep: pass 2 on faces (ii, fj), ii = i0-HF+fr ----
    for (int e = tid; e < G::FYR * G::FYC; e += NT) {
      const int fr = e / G::FYC, fc = e % G::FYC;
      const int ii = i0 - HF + fr, fj = j0 - HF + fc;
      if (ii < 0 || ii >= nx || fj < 0 || fj > ny) continue;
      T ql[4], qr[4], fl[4], fr_[4];
      {
        T a1[4], a2[4], f1[4], f2[4];
        tile_gq_side<T, FAST>(P1 + fr * G::P1YC + fc, G::P1, G::P1YC, weps, a1, a2);
        euler_flux_pair<T, FAST, true>(a1, a2, gamma, f1, f2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          fl[k] = S == 1 ? T(0.5) * (f1[k] + f2[k]) : f1[k] + f2[k];
          ql[k] = S == 1 ? T(0.5) * (a1[k] + a2[k]) : a1[k] + a2[k];
        }
        tile_gq_side<T, FAST>(P1 + 4 * G::P1 + fr * G::P1YC + fc, G::P1, G::P1YC, weps, a1, a2);
        euler_flux_pair<T, FAST, true>(a1, a2, gamma, f1, f2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          fr_[k] = S == 1 ? T(0.5) * (f2[k] + f1[k]) : f2[k] + f1[k];
          qr[k] = S == 1 ? T(0.5) * (a1[k] + a2[k]) : a1[k] + a2[k];
        }
      }
      tile_face_flux<T, FAST, true, BLEND, S>(ql, fl, qr, fr_, gamma, FY, G::FYR * G::FYC, e);
    }
    __syncthreads();

    // ---- residual + SSP-RK3 combination (+ wave speed for the next dt) ----
    const double dt = ctl[tl.x].dt;
    const T* qn = Qn + d.off;
    T* qo = Qo + d.off;
    double best = 0.0;
    for (int e = tid; e < TX * TY; e += NT) {
      const int il = e / TY, jl = e % TY;
      const int i = i0 + il, j = j0 + jl;
      if (i >= nx || j >= ny) continue;
      T L[4];
      const int fyr = il + HF, fyc = jl + HF;  // Fy cols fj = j, j+1
      const int FM = G::FYR * G::FYC;
      T va = T(1.0), vb = T(1.0);
      if constexpr (BLEND) {
        va = tile_sensor<T, FAST>(FY + 8 * FM, G::FYR, G::FYC, fyr, fyc, i, j, nx, ny + 1, jp_lo, jp_hi);
        vb = tile_sensor<T, FAST>(FY + 8 * FM, G::FYR, G::FYC, fyr, fyc + 1, i, j + 1, nx, ny + 1, jp_lo, jp_hi);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        T fya, fyb;
        if constexpr (BLEND) {
          fya = va * FY[k * FM + fyr * G::FYC + fyc] + (T(1.0) - va) * FY[(4 + k) * FM + fyr * G::FYC + fyc];
          fyb = vb * FY[k * FM + fyr * G::FYC + fyc + 1] + (T(1.0) - vb) * FY[(4 + k) * FM + fyr * G::FYC + fyc + 1];
        } else {
          fya = FY[k * FM + fyr * G::FYC + fyc];
          fyb = FY[k * FM + fyr * G::FYC + fyc + 1];
        }
        const T dfdx = DXF[k * TX * TY + e];
        T dgdy;
        if constexpr (FAST) dgdy = (fyb - fya) * qrcp<T, FAST>(T(d.dx));
        else dgdy = (fyb - fya) / T(d.dx);
        L[k] = -(dfdx + dgdy);
      }
      const long long o = (long long)i * d.ld + j;
      // stage input of this cell, from the tile (padded (i+3, j+3) -> tile (i+3-i0+HF, ...))
      const int ur = i + 3 - i0 + HF, uc = j + 3 - j0 + HF;
      T v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const T qs = U[k * G::UR * G::UC + ur * G::UC + uc + G::CO];
        if (stage == 1) {
          v[k] = qs + T(dt) * L[k];
        } else if (stage == 2) {
          v[k] = T(0.75) * qn[k * ps + o] + T(0.25) * qs + T(0.25 * dt) * L[k];
        } else {
          v[k] = T(1.0 / 3.0) * qn[k * ps + o] + T(2.0 / 3.0) * qs + T((2.0 / 3.0) * dt) * L[k];
        }
        qo[k * ps + o] = v[k];
      }
      if (stage == 3) {
        // Rie_prob_2d_rs.py:312-315 on the new state (primitives as con2primi
        // writes them), in the state's precision; the maximum and dt are FP64
        const T r0 = v[0];
        const T rho = fmax(r0, T(kEps));
        T uu, vv;
        if constexpr (FAST) {
          const T ir = qrcp<T, FAST>(rho);
          uu = v[1] * ir;
          vv = v[2] * ir;
        } else {
          uu = v[1] / rho;
          vv = v[2] / rho;
        }
        const T pp = fmax((gamma - T(1.0)) * (v[3] - T(0.5) * rho * (uu * uu + vv * vv)), T(kEps));
        const T rden = r0 != r0 ? r0 : fmax(r0, T(1e-14));  // np.maximum: a NaN density stays NaN
        const T x = sqrt(qdiv<T, FAST>(gamma * pp, rden)) + sqrt(uu * uu + vv * vv);
        best = nan_max_b(best, (double)x);
      }
    }
    if (stage == 3) {
      for (int off = 16; off > 0; off >>= 1) best = nan_max_b(best, __shfl_xor_sync(0xffffffffu, best, off));
      if ((tid & 31) == 0) red[tid >> 5] = best;
      __syncthreads();
      if (tid == 0) {
        double b = 0.0;
        for (int w = 0; w < NT / 32; ++w) b = nan_max_b(b, red[w]);
        atomicMax(&ctl[tl.x].cmax_bits, (unsigned long long)__double_as_longlong(b));
        if (!(b < INFINITY)) atomicOr(&ctl[tl.x].status, 1);
      }
    }
    // the next tile's TMA load overwrites U: order this tile's shared-memory
    // accesses before it
    tma::fence_proxy_async_smem();
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Staged variant: the arithmetic of k_stage_tiles in three launches per stage,
// with the pass-1 face states and the face fluxes of every solve in a global
// workspace instead of shared memory, so each face is reconstructed once (the
// fused kernel recomputes the halo faces of every tile, 1.2-1.5x the pass-1
// work at 16 x 32).  In FP64 the kernels are bound by the FP64 pipe and HBM is
// nearly idle, so moving the faces through HBM and L2 costs less than that
// recompute.  Per solve (interior nx x ny):
//   P1x  8 planes (q_l, q_r) of (nx+1) x (ny+4): face row fi, column c <-> J = c-2
//   P1y  8 planes of (nx+4) x (ny+1): row r <-> I = r-2, face column fj
//   Fx   NF planes of (nx+1) x ny (pitch ld), Fy NF planes of nx x (ny+1)
//        (NF = 4: HLLE; 9: HLLC, HLLE and the mean pressure of the sensor blend)
// The work of a launch is the packed cell-tile list: a tile (i0, j0) owns its
// own faces, and the tiles on a solve's edges also own the faces beyond it.
// ---------------------------------------------------------------------------

// The four conserved values of padded cell (I, J) of a solve: from the pool
// (interior cells only) or, for a ghost cell, from the cell (or inflow state)
// the boundary fill would copy there.
template <class T>
__device__ __forceinline__ void staged_cell(const SolveDesc& d, const T* q, int I, int J, T v[4]) {
  int i = I - 3, j = J - 3;
  bool flip = false;
  if (i < 0 || i >= d.nx || j < 0 || j >= d.ny) {
    const GhostSrc g = resolve_cell(d, I, J);
    if (g.post) {
#pragma unroll
      for (int k = 0; k < 4; ++k) v[k] = T(d.post[k]);
      return;
    }
    i = g.i;
    j = g.j;
    flip = g.flip2;
  }
  const long long o = (long long)i * d.ld + j;
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = q[k * d.ps + o];
  if (flip) v[2] = -v[2];
}

// Pass 1 of both directions for every tile: q_l, q_r of each face into P1x / P1y.
// Qin is the pool of the stage input.
template <class T, bool FAST, bool CHAR, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) k_staged_pass1(const SolveDesc* __restrict__ solves,
                                                      const SolveCtl* __restrict__ ctl,
                                                      const int4* __restrict__ tiles, int ntiles, const T* Qin, T* W,
                                                      T gamma, T weps) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int4 tl = tiles[t];
    if (!ctl[tl.x].active) continue;
    const SolveDesc& d = solves[tl.x];
    const int nx = d.nx, ny = d.ny, i0 = tl.y, j0 = tl.z;
    const bool last_r = i0 + TX >= nx, last_c = j0 + TY >= ny;
    const int xr0 = i0, xr1 = last_r ? nx + 1 : i0 + TX;
    const int xc0 = j0 == 0 ? -2 : j0, xc1 = last_c ? ny + 2 : j0 + TY;
    const int yr0 = i0 == 0 ? -2 : i0, yr1 = last_r ? nx + 2 : i0 + TX;
    const int yc0 = j0, yc1 = last_c ? ny + 1 : j0 + TY;
    const int nxc = xc1 - xc0, nxf = (xr1 - xr0) * nxc;
    const int nyc = yc1 - yc0, nyf = (yr1 - yr0) * nyc;
    const T* q = Qin + d.off;
    for (int e = threadIdx.x; e < nxf + nyf; e += NT) {
      T cells[6][4], ql[4], qr[4];
      if (e < nxf) {
        const int fi = xr0 + e / nxc, J = xc0 + e % nxc;  // face between padded rows fi+2 and fi+3
#pragma unroll
        for (int s = 0; s < 6; ++s) staged_cell(d, q, fi + s, J + 3, cells[s]);
        pass1_face<T, FAST, false, CHAR>(cells, gamma, ql, qr, weps);
        T* w = W + d.w_p1x + (long long)fi * d.l_p1x + (J + 2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          w[k * d.s_p1x] = ql[k];
          w[(4 + k) * d.s_p1x] = qr[k];
        }
      } else {
        const int e2 = e - nxf;
        const int I = yr0 + e2 / nyc, fj = yc0 + e2 % nyc;  // face between padded columns fj+2 and fj+3
#pragma unroll
        for (int s = 0; s < 6; ++s) staged_cell(d, q, I + 3, fj + s, cells[s]);
        pass1_face<T, FAST, true, CHAR>(cells, gamma, ql, qr, weps);
        T* w = W + d.w_p1y + (long long)(I + 2) * d.l_p1y + fj;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          w[k * d.s_p1y] = ql[k];
          w[(4 + k) * d.s_p1y] = qr[k];
        }
      }
    }
  }
}

// FAST double: face-averaged states and fluxes of two neighbouring faces (along
// the transverse direction) from one side's pass-1 planes: p points at the
// first of the six transverse values of component 0, ks is the plane stride
// and ts the transverse stride.  The two faces' Gauss-point reconstructions
// share their first and second differences (weno5_gq_two).  With `two` false
// only face A is wanted and the sixth value is not read.  SUM: twice the
// averages (the Gauss-point sums), for the doubled-state HLLE.
template <bool Y, bool SUM>
__device__ __forceinline__ void staged_gq_two(const double* p, long long ks, long long ts, bool two, double gamma,
                                              double weps, double qA[4], double fA[4], double qB[4], double fB[4]) {
  double a1A[4], a2A[4], a1B[4], a2B[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double* u = p + k * ks;
    const double v4 = u[4 * ts];
    weno5_gq_two<double>(u[0], u[ts], u[2 * ts], u[3 * ts], v4, two ? u[5 * ts] : v4, weps, a1A[k], a2A[k], a1B[k],
                         a2B[k]);
  }
  double f1[4], f2[4];
  euler_flux_pair<double, true, Y>(a1A, a2A, gamma, f1, f2);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    fA[k] = SUM ? f1[k] + f2[k] : 0.5 * (f1[k] + f2[k]);
    qA[k] = SUM ? a1A[k] + a2A[k] : 0.5 * (a1A[k] + a2A[k]);
  }
  if (!two) return;
  euler_flux_pair<double, true, Y>(a1B, a2B, gamma, f1, f2);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    fB[k] = SUM ? f1[k] + f2[k] : 0.5 * (f1[k] + f2[k]);
    qB[k] = SUM ? a1B[k] + a2B[k] : 0.5 * (a1B[k] + a2B[k]);
  }
}

// Pass 2 (Gauss-point WENO of the pass-1 states, Euler fluxes, face averages)
// and the Riemann solver of every face a tile owns, into Fx / Fy.  FAST double
// takes two transverse neighbours per thread (as the single-grid k_pass2_two).
template <class T, bool FAST, bool BLEND, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) k_staged_pass2(const SolveDesc* __restrict__ solves,
                                                      const SolveCtl* __restrict__ ctl,
                                                      const int4* __restrict__ tiles, int ntiles, T* W, T gamma,
                                                      T weps) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int4 tl = tiles[t];
    if (!ctl[tl.x].active) continue;
    const SolveDesc& d = solves[tl.x];
    const int nx = d.nx, ny = d.ny, i0 = tl.y, j0 = tl.z;
    const bool last_r = i0 + TX >= nx, last_c = j0 + TY >= ny;
    const int xr1 = last_r ? nx + 1 : i0 + TX, xc1 = last_c ? ny : j0 + TY;
    const int yr1 = last_r ? nx : i0 + TX, yc1 = last_c ? ny + 1 : j0 + TY;
    const int nxc = xc1 - j0, nxf = (xr1 - i0) * nxc;
    const int nyc = yc1 - j0, nyf = (yr1 - i0) * nyc;
    if constexpr (FAST && is_native_f64<T>) {
      constexpr bool SUM = !BLEND;  // the HLLE flux takes the Gauss-point sums
      constexpr int S = SUM ? 2 : 1;
      const int nxp = (nxc + 1) / 2, nxi = (xr1 - i0) * nxp;  // x-face pairs (jj, jj+1)
      const int nyi = ((yr1 - i0 + 1) / 2) * nyc;              // y-face pairs (ii, ii+1)
      for (int e = threadIdx.x; e < nxi + nyi; e += NT) {
        double qlA[4], flA[4], qlB[4], flB[4], qrA[4], frA[4], qrB[4], frB[4];
        if (e < nxi) {
          const int fi = i0 + e / nxp, jj = j0 + 2 * (e % nxp);
          const bool two = jj + 1 < xc1;
          const double* p = W + d.w_p1x + (long long)fi * d.l_p1x + jj;
          staged_gq_two<false, SUM>(p, d.s_p1x, 1, two, gamma, weps, qlA, flA, qlB, flB);
          staged_gq_two<false, SUM>(p + 4 * d.s_p1x, d.s_p1x, 1, two, gamma, weps, qrA, frA, qrB, frB);
          tile_face_flux<T, FAST, false, BLEND, S>(qlA, flA, qrA, frA, gamma, W + d.w_fx, (int)d.s_fx,
                                                   fi * d.ld + jj);
          if (two)
            tile_face_flux<T, FAST, false, BLEND, S>(qlB, flB, qrB, frB, gamma, W + d.w_fx, (int)d.s_fx,
                                                     fi * d.ld + jj + 1);
        } else {
          const int e2 = e - nxi;
          const int ii = i0 + 2 * (e2 / nyc), fj = j0 + e2 % nyc;
          const bool two = ii + 1 < yr1;
          const double* p = W + d.w_p1y + (long long)ii * d.l_p1y + fj;
          staged_gq_two<true, SUM>(p, d.s_p1y, d.l_p1y, two, gamma, weps, qlA, flA, qlB, flB);
          staged_gq_two<true, SUM>(p + 4 * d.s_p1y, d.s_p1y, d.l_p1y, two, gamma, weps, qrA, frA, qrB, frB);
          tile_face_flux<T, FAST, true, BLEND, S>(qlA, flA, qrA, frA, gamma, W + d.w_fy, (int)d.s_fy,
                                                  ii * d.l_p1y + fj);
          if (two)
            tile_face_flux<T, FAST, true, BLEND, S>(qlB, flB, qrB, frB, gamma, W + d.w_fy, (int)d.s_fy,
                                                    (ii + 1) * d.l_p1y + fj);
        }
      }
    } else {
      // FAST HLLE takes the Gauss-point sums (twice the face averages)
      constexpr int S = FAST && !BLEND ? 2 : 1;
      for (int e = threadIdx.x; e < nxf + nyf; e += NT) {
        T ql[4], qr[4], fl[4], fr_[4], a1[4], a2[4], f1[4], f2[4];
        if (e < nxf) {
          const int fi = i0 + e / nxc, jj = j0 + e % nxc;
          // the five transverse pass-1 states J = jj-2 .. jj+2 (columns jj .. jj+4)
          const T* p = W + d.w_p1x + (long long)fi * d.l_p1x + jj;
          tile_gq_side<T, FAST>(p, (int)d.s_p1x, 1, weps, a1, a2);
          euler_flux_pair<T, FAST, false>(a1, a2, gamma, f1, f2);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            fl[k] = S == 1 ? T(0.5) * (f1[k] + f2[k]) : f1[k] + f2[k];
            ql[k] = S == 1 ? T(0.5) * (a1[k] + a2[k]) : a1[k] + a2[k];
          }
          tile_gq_side<T, FAST>(p + 4 * d.s_p1x, (int)d.s_p1x, 1, weps, a1, a2);
          euler_flux_pair<T, FAST, false>(a1, a2, gamma, f1, f2);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            fr_[k] = S == 1 ? T(0.5) * (f2[k] + f1[k]) : f2[k] + f1[k];
            qr[k] = S == 1 ? T(0.5) * (a1[k] + a2[k]) : a1[k] + a2[k];
          }
          tile_face_flux<T, FAST, false, BLEND, S>(ql, fl, qr, fr_, gamma, W + d.w_fx, (int)d.s_fx, fi * d.ld + jj);
        } else {
          const int e2 = e - nxf;
          const int ii = i0 + e2 / nyc, fj = j0 + e2 % nyc;
          // the five transverse pass-1 states I = ii-2 .. ii+2 (rows ii .. ii+4)
          const T* p = W + d.w_p1y + (long long)ii * d.l_p1y + fj;
          tile_gq_side<T, FAST>(p, (int)d.s_p1y, d.l_p1y, weps, a1, a2);
          euler_flux_pair<T, FAST, true>(a1, a2, gamma, f1, f2);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            fl[k] = S == 1 ? T(0.5) * (f1[k] + f2[k]) : f1[k] + f2[k];
            ql[k] = S == 1 ? T(0.5) * (a1[k] + a2[k]) : a1[k] + a2[k];
          }
          tile_gq_side<T, FAST>(p + 4 * d.s_p1y, (int)d.s_p1y, d.l_p1y, weps, a1, a2);
          euler_flux_pair<T, FAST, true>(a1, a2, gamma, f1, f2);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            fr_[k] = S == 1 ? T(0.5) * (f2[k] + f1[k]) : f2[k] + f1[k];
            qr[k] = S == 1 ? T(0.5) * (a1[k] + a2[k]) : a1[k] + a2[k];
          }
          tile_face_flux<T, FAST, true, BLEND, S>(ql, fl, qr, fr_, gamma, W + d.w_fy, (int)d.s_fy, ii * d.l_p1y + fj);
        }
      }
    }
  }
}

// Sensor blend, flux difference and SSP-RK3 stage combination of every cell
// (the last part of k_stage_tiles, on the workspace fluxes); stage 3 also
// reduces the new state's wave speed per solve.  Qs is the pool of the stage
// input, Qn the step's initial state, Qo the output pool.
template <class T, bool FAST, bool BLEND, int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) k_staged_residual(const SolveDesc* __restrict__ solves, SolveCtl* ctl,
                                                         const int4* __restrict__ tiles, int ntiles, const T* W,
                                                         const T* Qs, const T* Qn, T* Qo, int stage, T gamma,
                                                         T jp_lo, T jp_hi) {
  __shared__ double red[NT / 32];
  const int tid = threadIdx.x;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int4 tl = tiles[t];
    if (!ctl[tl.x].active) continue;  // uniform across the CTA
    const SolveDesc& d = solves[tl.x];
    const int nx = d.nx, ny = d.ny, i0 = tl.y, j0 = tl.z;
    const double dt = ctl[tl.x].dt;
    const T* Fx = W + d.w_fx;
    const T* Fy = W + d.w_fy;
    const long long fxs = d.s_fx, fys = d.s_fy;
    const int lx = d.ld, ly = d.l_p1y;
    double best = 0.0;
    for (int e = tid; e < TX * TY; e += NT) {
      const int i = i0 + e / TY, j = j0 + e % TY;
      if (i >= nx || j >= ny) continue;
      T wa = T(1.0), wb = T(1.0), va = T(1.0), vb = T(1.0);
      if constexpr (BLEND) {
        wa = tile_sensor<T, FAST>(Fx + 8 * fxs, 0, lx, i, j, i, j, nx + 1, ny, jp_lo, jp_hi);
        wb = tile_sensor<T, FAST>(Fx + 8 * fxs, 0, lx, i + 1, j, i + 1, j, nx + 1, ny, jp_lo, jp_hi);
        va = tile_sensor<T, FAST>(Fy + 8 * fys, 0, ly, i, j, i, j, nx, ny + 1, jp_lo, jp_hi);
        vb = tile_sensor<T, FAST>(Fy + 8 * fys, 0, ly, i, j + 1, i, j + 1, nx, ny + 1, jp_lo, jp_hi);
      }
      const long long xa = (long long)i * lx + j, xb = xa + lx;
      const long long ya = (long long)i * ly + j, yb = ya + 1;
      T L[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        T fxa, fxb, fya, fyb;
        if constexpr (BLEND) {
          fxa = wa * Fx[k * fxs + xa] + (T(1.0) - wa) * Fx[(4 + k) * fxs + xa];
          fxb = wb * Fx[k * fxs + xb] + (T(1.0) - wb) * Fx[(4 + k) * fxs + xb];
          fya = va * Fy[k * fys + ya] + (T(1.0) - va) * Fy[(4 + k) * fys + ya];
          fyb = vb * Fy[k * fys + yb] + (T(1.0) - vb) * Fy[(4 + k) * fys + yb];
        } else {
          fxa = Fx[k * fxs + xa];
          fxb = Fx[k * fxs + xb];
          fya = Fy[k * fys + ya];
          fyb = Fy[k * fys + yb];
        }
        T dfdx, dgdy;
        if constexpr (FAST) {
          dfdx = (fxb - fxa) * qrcp<T, FAST>(T(d.dx));
          dgdy = (fyb - fya) * qrcp<T, FAST>(T(d.dx));
        } else {
          dfdx = (fxb - fxa) / T(d.dx);
          dgdy = (fyb - fya) / T(d.dx);
        }
        L[k] = -(dfdx + dgdy);
      }
      const long long o = d.off + (long long)i * d.ld + j;
      T v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const T qs = Qs[k * d.ps + o];
        if (stage == 1) {
          v[k] = qs + T(dt) * L[k];
        } else if (stage == 2) {
          v[k] = T(0.75) * Qn[k * d.ps + o] + T(0.25) * qs + T(0.25 * dt) * L[k];
        } else {
          v[k] = T(1.0 / 3.0) * Qn[k * d.ps + o] + T(2.0 / 3.0) * qs + T((2.0 / 3.0) * dt) * L[k];
        }
        Qo[k * d.ps + o] = v[k];
      }
      if (stage == 3) {
        const T r0 = v[0];
        const T rho = fmax(r0, T(kEps));
        T uu, vv;
        if constexpr (FAST) {
          const T ir = qrcp<T, FAST>(rho);
          uu = v[1] * ir;
          vv = v[2] * ir;
        } else {
          uu = v[1] / rho;
          vv = v[2] / rho;
        }
        const T pp = fmax((gamma - T(1.0)) * (v[3] - T(0.5) * rho * (uu * uu + vv * vv)), T(kEps));
        const T rden = r0 != r0 ? r0 : fmax(r0, T(1e-14));  // np.maximum: a NaN density stays NaN
        const T x = sqrt(qdiv<T, FAST>(gamma * pp, rden)) + sqrt(uu * uu + vv * vv);
        best = nan_max_b(best, (double)x);
      }
    }
    if (stage == 3) {
      for (int off = 16; off > 0; off >>= 1) best = nan_max_b(best, __shfl_xor_sync(0xffffffffu, best, off));
      if ((tid & 31) == 0) red[tid >> 5] = best;
      __syncthreads();
      if (tid == 0) {
        double b = 0.0;
        for (int w = 0; w < NT / 32; ++w) b = nan_max_b(b, red[w]);
        atomicMax(&ctl[tl.x].cmax_bits, (unsigned long long)__double_as_longlong(b));
        if (!(b < INFINITY)) atomicOr(&ctl[tl.x].status, 1);
      }
      __syncthreads();
    }
  }
}

// Wave-speed maximum of the current state per solve (the first dt of a run).
template <class T, int NT>
__global__ void __launch_bounds__(NT) k_cfl_tiles(const SolveDesc* __restrict__ solves, SolveCtl* ctl,
                                                   const int4* __restrict__ tiles, int ntiles, int TX, int TY,
                                                   const T* Q, T gamma) {
  __shared__ double red[NT / 32];
  const int tid = threadIdx.x;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int4 tl = tiles[t];
    if (!ctl[tl.x].active) continue;
    const SolveDesc d = solves[tl.x];
    double best = 0.0;
    for (int e = tid; e < TX * TY; e += NT) {
      const int i = tl.y + e / TY, j = tl.z + e % TY;
      if (i >= d.nx || j >= d.ny) continue;
      const long long o = d.off + (long long)i * d.ld + j;
      const double r0 = (double)Q[o];
      const double rho = fmax(r0, kEps);
      const double uu = (double)Q[o + d.ps] / rho, vv = (double)Q[o + 2 * d.ps] / rho;
      const double pp = fmax(((double)gamma - 1.0) * ((double)Q[o + 3 * d.ps] - 0.5 * rho * (uu * uu + vv * vv)), kEps);
      const double x = sqrt((double)gamma * pp / (r0 != r0 ? r0 : fmax(r0, 1e-14))) + sqrt(uu * uu + vv * vv);
      best = nan_max_b(best, x);
    }
    for (int off = 16; off > 0; off >>= 1) best = nan_max_b(best, __shfl_xor_sync(0xffffffffu, best, off));
    if ((tid & 31) == 0) red[tid >> 5] = best;
    __syncthreads();
    if (tid == 0) {
      double b = 0.0;
      for (int w = 0; w < NT / 32; ++w) b = nan_max_b(b, red[w]);
      atomicMax(&ctl[tl.x].cmax_bits, (unsigned long long)__double_as_longlong(b));
      if (!(b < INFINITY)) atomicOr(&ctl[tl.x].status, 1);
    }
    __syncthreads();
  }
}

// Per-solve clock.  phase 0 (start of a step): dt from the reduced wave speed,
// clipped to t_end.  phase 1 (end of a step): advance the clock, test the loop
// condition, clear the reduction for the next step's dt.
__global__ void k_solve_clock(SolveCtl* ctl, int nsolves, int phase) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsolves) return;
  SolveCtl& c = ctl[s];
  if (!c.active) return;
  if (c.status & 4) {
    // a tile of this solve was not staged in some stage: its state is incomplete
    c.active = 0;
    return;
  }
  if (phase == 0) {
    const double cmax = __longlong_as_double((long long)c.cmax_bits) + 1e-16;
    if (!(cmax < INFINITY)) {
      // a non-finite wave speed (NaN, or an overflow to infinity that would give
      // dt = 0 for ever): the solve stops here with its status set
      c.status |= 1;
      c.active = 0;
      return;
    }
    double dt = c.cfl_dx / cmax;
    if (c.t_end >= 0.0) {
      const double remaining = c.t_end - c.t;
      if (remaining < dt) dt = remaining;
    }
    c.dt = dt;
    c.cmax_bits = 0ull;
  } else {
    c.t += c.dt;
    c.steps += 1;
    bool more = c.steps < c.max_steps;
    if (c.t_end >= 0.0) more = more && (c.t < c.t_end - 1e-12);
    c.active = more ? 1 : 0;
  }
}

}  // inline namespace WENO_TU_NS
}  // namespace weno
