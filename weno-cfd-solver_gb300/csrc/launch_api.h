// Host-side launchers of the residual kernels, one set per (arithmetic type,
// arithmetic policy).  The definitions live in launch_impl.cuh and are compiled
// only in tu_exact.cu (--fmad=false: reference-identical IEEE doubles) and
// tu_fast.cu (--fmad=true: the FAST forms), so the policy of a kernel is fixed
// by the translation unit it was built in.  This header only declares them.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace weno {

// Strided read-only view of a caller array (elements, not bytes).
struct HostView {
  const void* p;
  int64_t s0, s1, s2;
};

// Plane set: component k, element (r, c) at p[k*ps + r*ld + c].
struct HostPlanes {
  void* p;
  int64_t ps, ld;
};

struct StepCtl;
namespace dfm {
struct df64;
}

template <class T, bool FAST>
struct Launch {
  // Pass 1 over `rows x cols` faces (x: rows = m-5, cols = n; y: rows = m, cols = n-5).
  static cudaError_t pass1(HostView u, int64_t rows, int64_t cols, double gamma, bool ydir, bool chr,
                           HostPlanes PL, HostPlanes PR, double weps, cudaStream_t st);
  // Pass 2 over the final face array.  kind 0: dense q_l, f_l, q_r, f_r into
  // a..d; kind 1: HLLE flux planes into a; kind 2: HLLC planes into a, HLLE
  // planes into b, mean pressure plane into c.  ps/ld describe a, b, c.
  static cudaError_t pass2(HostPlanes PL, HostPlanes PR, int64_t rows, int64_t cols, double gamma, bool ydir,
                           int kind, void* a, void* b, void* c, void* d, int64_t ps, int64_t ld, double weps,
                           cudaStream_t st);
  // Riemann solver on dense (rows, cols, 4) face arrays.  kind 0 HLLC / 1 HLLE
  // -> dense out; kind 2 -> planes Fc (a), Fe (b), pbar (c).
  static cudaError_t riemann(const void* ql, const void* fl, const void* qr, const void* fr, int64_t rows,
                             int64_t cols, double gamma, bool ydir, int kind, void* out, void* a, void* b, void* c,
                             int64_t ps, int64_t ld, cudaStream_t st);
  // Sensor blend; writes dense `out` if non-null, else in place into Fc.
  static cudaError_t blend(HostPlanes Fc, HostPlanes Fe, HostPlanes Pbar, int64_t rows, int64_t cols, double jp_lo,
                           double jp_hi, void* out, cudaStream_t st);
  // Flux difference over (rows, cols) = (m-6, n-6) cells.  stage 0: dense out;
  // stages 1..3: SSP-RK3 combination into Qo planes (interior offset 3).
  static cudaError_t residual(HostPlanes Fx, HostPlanes Fy, int64_t rows, int64_t cols, double dx, int stage,
                              void* out, HostPlanes Qn, HostPlanes Qs, HostPlanes Qo, const StepCtl* ctl,
                              cudaStream_t st);
  static cudaError_t flux(HostView q, int64_t rows, int64_t cols, double gamma, bool ydir, void* out, cudaStream_t st);
  static cudaError_t con2primi(HostView q, int64_t rows, int64_t cols, double gamma, void* p, void* a, void* rho,
                               void* u, void* v, void* h, cudaStream_t st);
  // Boundary fills on nc (4 or 8) channels of a strided array, in place.
  static cudaError_t bc_transmissive(HostView q, int nc, int64_t M, int64_t N, const StepCtl* ctl, cudaStream_t st);
  static cudaError_t bc_dmr(HostView q, int nc, int64_t nx, int64_t ny, int64_t bound, const double* post8,
                            const StepCtl* ctl, cudaStream_t st);
  // CFL reduction into ctl->cmax_bits; aos = read primitives from channels 5..7.
  static cudaError_t cfl_max(HostView q, bool aos, int64_t nx, int64_t ny, double gamma, StepCtl* ctl,
                             int sm_count, cudaStream_t st);
  static cudaError_t export_aos8(HostPlanes Q, int64_t M, int64_t N, double gamma, double* out, cudaStream_t st);
  static cudaError_t totals(HostView q, int64_t nx, int64_t ny, double* out4, int sm_count, cudaStream_t st);
  static cudaError_t import_planes(HostView q, int64_t M, int64_t N, HostPlanes Q, cudaStream_t st);
};

// Control-block kernels (precision independent).
cudaError_t launch_dt(StepCtl* ctl, cudaStream_t st);
cudaError_t launch_step_end(StepCtl* ctl, cudaStream_t st);
cudaError_t launch_run_begin(StepCtl* ctl, double t_final, long long add, cudaStream_t st);

extern template struct Launch<double, false>;
extern template struct Launch<double, true>;
extern template struct Launch<float, true>;
extern template struct Launch<dfm::df64, true>;

}  // namespace weno
