// Launcher definitions (see launch_api.h).  Included only by tu_exact.cu and
// tu_fast.cu.
#pragma once

#include "kernels.cuh"
#include "launch_api.h"

namespace weno {

inline namespace WENO_TU_NS {
namespace detail {

inline dim3 grid2d(int64_t rows, int64_t cols, dim3 blk) {
  return dim3((unsigned)((cols + blk.x - 1) / blk.x), (unsigned)((rows + blk.y - 1) / blk.y), 1);
}

template <class T>
inline CView<T> cview(HostView v) {
  return CView<T>{static_cast<const T*>(v.p), v.s0, v.s1, v.s2};
}
template <class T>
inline Planes<T> planes(HostPlanes v) {
  return Planes<T>{static_cast<T*>(v.p), v.ps, v.ld};
}
template <class T>
inline S3<T> s3(HostView v) {
  return S3<T>{static_cast<T*>(const_cast<void*>(v.p)), v.s0, v.s1, v.s2};
}

const dim3 kBlk(32, 4, 1);

}  // namespace detail
}  // inline namespace WENO_TU_NS

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::pass1(HostView u, int64_t rows, int64_t cols, double gamma, bool ydir, bool chr,
                                   HostPlanes PL, HostPlanes PR, double weps, cudaStream_t st) {
  using namespace detail;
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const dim3 g = grid2d(rows, cols, kBlk);
  auto U = cview<T>(u);
  auto L = planes<T>(PL), R = planes<T>(PR);
  if constexpr (FAST && std::is_same<T, double>::value) {
    if (!chr) {  // component-wise: two faces per thread along the sweep
      const dim3 g2 = ydir ? grid2d(rows, (cols + 1) / 2, kBlk) : grid2d((rows + 1) / 2, cols, kBlk);
      if (!ydir) k_pass1_cons2<false><<<g2, kBlk, 0, st>>>(U, rows, cols, L, R, weps);
      else k_pass1_cons2<true><<<g2, kBlk, 0, st>>>(U, rows, cols, L, R, weps);
      return cudaGetLastError();
    }
  }
  if (!ydir && chr) k_pass1<T, FAST, false, true><<<g, kBlk, 0, st>>>(U, rows, cols, (T)gamma, L, R, (T)weps);
  else if (!ydir) k_pass1<T, FAST, false, false><<<g, kBlk, 0, st>>>(U, rows, cols, (T)gamma, L, R, (T)weps);
  else if (chr) k_pass1<T, FAST, true, true><<<g, kBlk, 0, st>>>(U, rows, cols, (T)gamma, L, R, (T)weps);
  else k_pass1<T, FAST, true, false><<<g, kBlk, 0, st>>>(U, rows, cols, (T)gamma, L, R, (T)weps);
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::pass2(HostPlanes PL, HostPlanes PR, int64_t rows, int64_t cols, double gamma, bool ydir,
                                   int kind, void* a, void* b, void* c, void* d, int64_t ps, int64_t ld, double weps,
                                   cudaStream_t st) {
  using namespace detail;
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const dim3 g = grid2d(rows, cols, kBlk);
  auto L = planes<T>(PL), R = planes<T>(PR);
  Pass2Dst dst{a, b, c, d, ps, ld};
  const T gm = (T)gamma;
  if constexpr (FAST && !std::is_same<T, df64>::value) {
    // two faces per thread along the transverse direction (df64 keeps one:
    // its larger per-face register footprint outweighs the shared differences)
    const dim3 g2 = ydir ? grid2d((rows + 1) / 2, cols, kBlk) : grid2d(rows, (cols + 1) / 2, kBlk);
#define WENO_P2T(Y, K) k_pass2_two<T, Y, K><<<g2, kBlk, 0, st>>>(L, R, rows, cols, gm, dst, (T)weps)
    if (!ydir) {
      if (kind == 0) WENO_P2T(false, P2_STATES);
      else if (kind == 1) WENO_P2T(false, P2_HLLE);
      else WENO_P2T(false, P2_BLEND);
    } else {
      if (kind == 0) WENO_P2T(true, P2_STATES);
      else if (kind == 1) WENO_P2T(true, P2_HLLE);
      else WENO_P2T(true, P2_BLEND);
    }
#undef WENO_P2T
    return cudaGetLastError();
  }
#define WENO_P2(Y, K) k_pass2<T, FAST, Y, K><<<g, kBlk, 0, st>>>(L, R, rows, cols, gm, dst, (T)weps)
  if (!ydir) {
    if (kind == 0) WENO_P2(false, P2_STATES);
    else if (kind == 1) WENO_P2(false, P2_HLLE);
    else WENO_P2(false, P2_BLEND);
  } else {
    if (kind == 0) WENO_P2(true, P2_STATES);
    else if (kind == 1) WENO_P2(true, P2_HLLE);
    else WENO_P2(true, P2_BLEND);
  }
#undef WENO_P2
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::riemann(const void* ql, const void* fl, const void* qr, const void* fr, int64_t rows,
                                     int64_t cols, double gamma, bool ydir, int kind, void* out, void* a, void* b,
                                     void* c, int64_t ps, int64_t ld, cudaStream_t st) {
  using namespace detail;
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const dim3 g = grid2d(rows, cols, kBlk);
  const T *QL = static_cast<const T*>(ql), *FL = static_cast<const T*>(fl);
  const T *QR = static_cast<const T*>(qr), *FR = static_cast<const T*>(fr);
  Planes<T> A{static_cast<T*>(a), ps, ld}, B{static_cast<T*>(b), ps, ld}, C{static_cast<T*>(c), ps, ld};
  T* o = static_cast<T*>(out);
  const T gm = (T)gamma;
#define WENO_RS(Y, K) k_riemann<T, FAST, Y, K><<<g, kBlk, 0, st>>>(QL, FL, QR, FR, rows, cols, gm, o, A, B, C)
  if (!ydir) {
    if (kind == 0) WENO_RS(false, 0);
    else if (kind == 1) WENO_RS(false, 1);
    else WENO_RS(false, 2);
  } else {
    if (kind == 0) WENO_RS(true, 0);
    else if (kind == 1) WENO_RS(true, 1);
    else WENO_RS(true, 2);
  }
#undef WENO_RS
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::blend(HostPlanes Fc, HostPlanes Fe, HostPlanes Pbar, int64_t rows, int64_t cols,
                                   double jp_lo, double jp_hi, void* out, cudaStream_t st) {
  using namespace detail;
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const dim3 g = grid2d(rows, cols, kBlk);
  auto C = planes<T>(Fc), E = planes<T>(Fe), P = planes<T>(Pbar);
  if (out) k_blend<T, FAST, true><<<g, kBlk, 0, st>>>(C, E, P, rows, cols, (T)jp_lo, (T)jp_hi, static_cast<T*>(out), C);
  else k_blend<T, FAST, false><<<g, kBlk, 0, st>>>(C, E, P, rows, cols, (T)jp_lo, (T)jp_hi, nullptr, C);
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::residual(HostPlanes Fx, HostPlanes Fy, int64_t rows, int64_t cols, double dx, int stage,
                                      void* out, HostPlanes Qn, HostPlanes Qs, HostPlanes Qo, const StepCtl* ctl,
                                      cudaStream_t st) {
  using namespace detail;
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const dim3 g = grid2d(rows, cols, kBlk);
  auto X = planes<T>(Fx), Yp = planes<T>(Fy), N = planes<T>(Qn), S = planes<T>(Qs), O = planes<T>(Qo);
  T* o = static_cast<T*>(out);
  switch (stage) {
    case 0: k_residual<T, FAST, 0><<<g, kBlk, 0, st>>>(X, Yp, rows, cols, (T)dx, o, N, S, O, ctl); break;
    case 1: k_residual<T, FAST, 1><<<g, kBlk, 0, st>>>(X, Yp, rows, cols, (T)dx, o, N, S, O, ctl); break;
    case 2: k_residual<T, FAST, 2><<<g, kBlk, 0, st>>>(X, Yp, rows, cols, (T)dx, o, N, S, O, ctl); break;
    default: k_residual<T, FAST, 3><<<g, kBlk, 0, st>>>(X, Yp, rows, cols, (T)dx, o, N, S, O, ctl); break;
  }
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::flux(HostView q, int64_t rows, int64_t cols, double gamma, bool ydir, void* out,
                                  cudaStream_t st) {
  using namespace detail;
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const dim3 g = grid2d(rows, cols, kBlk);
  if (ydir) k_flux<T, FAST, true><<<g, kBlk, 0, st>>>(cview<T>(q), rows, cols, (T)gamma, static_cast<T*>(out));
  else k_flux<T, FAST, false><<<g, kBlk, 0, st>>>(cview<T>(q), rows, cols, (T)gamma, static_cast<T*>(out));
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::con2primi(HostView q, int64_t rows, int64_t cols, double gamma, void* p, void* a,
                                       void* rho, void* u, void* v, void* h, cudaStream_t st) {
  using namespace detail;
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const dim3 g = grid2d(rows, cols, kBlk);
  k_con2primi<T, FAST><<<g, kBlk, 0, st>>>(cview<T>(q), rows, cols, (T)gamma, static_cast<T*>(p),
                                           static_cast<T*>(a), static_cast<T*>(rho), static_cast<T*>(u),
                                           static_cast<T*>(v), static_cast<T*>(h));
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::bc_transmissive(HostView q, int nc, int64_t M, int64_t N, const StepCtl* ctl,
                                             cudaStream_t st) {
  using namespace detail;
  const dim3 g = grid2d(M, N, kBlk);
  if (nc == 8) k_bc_transmissive<T, 8><<<g, kBlk, 0, st>>>(s3<T>(q), M, N, ctl);
  else k_bc_transmissive<T, 4><<<g, kBlk, 0, st>>>(s3<T>(q), M, N, ctl);
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::bc_dmr(HostView q, int nc, int64_t nx, int64_t ny, int64_t bound, const double* post8,
                                    const StepCtl* ctl, cudaStream_t st) {
  using namespace detail;
  const dim3 g = grid2d(nx + 6, ny + 6, kBlk);
  Post8<T> post;
  for (int k = 0; k < 8; ++k) post.v[k] = (T)post8[k];
  if (nc == 8) k_bc_dmr<T, 8><<<g, kBlk, 0, st>>>(s3<T>(q), nx, ny, bound, post, ctl);
  else k_bc_dmr<T, 4><<<g, kBlk, 0, st>>>(s3<T>(q), nx, ny, bound, post, ctl);
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::cfl_max(HostView q, bool aos, int64_t nx, int64_t ny, double gamma, StepCtl* ctl,
                                     int sm_count, cudaStream_t st) {
  const int64_t total = nx * ny;
  int64_t blocks = (total + 255) / 256;
  const int64_t cap = (int64_t)sm_count * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (aos) k_cfl_max<T, true><<<(unsigned)blocks, 256, 0, st>>>(detail::cview<T>(q), nx, ny, (T)gamma, ctl);
  else k_cfl_max<T, false><<<(unsigned)blocks, 256, 0, st>>>(detail::cview<T>(q), nx, ny, (T)gamma, ctl);
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::export_aos8(HostPlanes Q, int64_t M, int64_t N, double gamma, double* out,
                                         cudaStream_t st) {
  using namespace detail;
  const dim3 g = grid2d(M, N, kBlk);
  k_export_aos8<T, FAST><<<g, kBlk, 0, st>>>(planes<T>(Q), M, N, (T)gamma, out);
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::totals(HostView q, int64_t nx, int64_t ny, double* out4, int sm_count, cudaStream_t st) {
  int64_t blocks = (nx * ny + 255) / 256;
  if (blocks > (int64_t)sm_count * 4) blocks = (int64_t)sm_count * 4;
  if (blocks < 1) blocks = 1;
  cudaError_t e = cudaMemsetAsync(out4, 0, 4 * sizeof(double), st);
  if (e) return e;
  k_totals<T><<<(unsigned)blocks, 256, 0, st>>>(detail::cview<T>(q), nx, ny, out4);
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t Launch<T, FAST>::import_planes(HostView q, int64_t M, int64_t N, HostPlanes Q, cudaStream_t st) {
  using namespace detail;
  const dim3 g = grid2d(M, N, kBlk);
  k_import_planes<T><<<g, kBlk, 0, st>>>(cview<double>(q), M, N, planes<T>(Q));
  return cudaGetLastError();
}

}  // namespace weno
