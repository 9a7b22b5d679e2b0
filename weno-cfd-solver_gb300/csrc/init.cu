// Device generators of the benchmark initial data in the drivers' (nx+6, ny+6, 8)
// layout (conserved channels, then rho, u, v, p), ghost cells included, as
// Rie_prob_2d_rs.py:213-263 and unitest.py:169-205 build them on the host.
// Compiled with --fmad=false: the conserved energy p/(gamma-1) + 0.5*rho*(u^2+v^2)
// is evaluated in numpy's order and matches weno_ext.problems bit for bit.
#include <cuda_runtime.h>

#include <cmath>

#define WENO_TU_NS init_tu
#include "../../include/weno_gb300.h"
#include "errors.h"
#include "launch_api.h"
#include "step_ctl.h"

namespace {

struct Prim4 {
  double rho, u, v, p;
};

__device__ __forceinline__ void store_cell(double* o, const Prim4& s, double gamma) {
  o[0] = s.rho;
  o[1] = s.rho * s.u;
  o[2] = s.rho * s.v;
  o[3] = s.p / (gamma - 1.0) + 0.5 * s.rho * (s.u * s.u + s.v * s.v);
  o[4] = s.rho;
  o[5] = s.u;
  o[6] = s.v;
  o[7] = s.p;
}

// Four quadrants split at padded indices si (axis 0) and sj (axis 1); states in
// the order (i < si, j < sj), (i >= si, j < sj), (i < si, j >= sj), (i >= si, j >= sj).
__global__ void k_init_quadrant(double* out, int M, int N, int si, int sj, Prim4 s0, Prim4 s1, Prim4 s2, Prim4 s3,
                                double gamma) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= M || j >= N) return;
  const Prim4& s = (j < sj) ? (i < si ? s0 : s1) : (i < si ? s2 : s3);
  store_cell(out + ((long long)i * N + j) * 8, s, gamma);
}

// Planar shock through (x0, 0) at angle theta (tan_t = tan(theta)): cells with
// y - tan_t * (x - x0) >= 0 get the post-shock state, cell centres
// x = ((i - 3) + 0.5) / nx * lx, y = ((j - 3) + 0.5) / ny * ly.
__global__ void k_init_shock(double* out, int nx, int ny, double lx, double ly, double x0, double tan_t, Prim4 pre,
                             Prim4 post, double gamma) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int M = nx + 6, N = ny + 6;
  if (i >= M || j >= N) return;
  const double x = ((double)(i - 3) + 0.5) / nx * lx;
  const double y = ((double)(j - 3) + 0.5) / ny * ly;
  store_cell(out + ((long long)i * N + j) * 8, (y - tan_t * (x - x0) >= 0.0) ? post : pre, gamma);
}

// Rie_prob_2d_rs.py:42-120 apply_bc_reflecting on a square (n, n, 8) array,
// pointwise.  Edge ghosts (one index a ghost, the other interior) mirror the
// interior about the wall: low side g <- 5-g, high side g <- 2n-7-g, with the
// normal momentum and velocity negated (channels 2, 6 across the axis-0 walls,
// 1, 5 across the axis-1 walls).  The reference fills the four 3x3 corner
// blocks afterwards from interior blocks with both pairs negated: the low
// corner index g takes 5-g, the high one g-3 (a shift, not a mirror:
// gh = n-3+g <- n-6+g, Rie_prob_2d_rs.py:105-117).  Every source is an
// interior cell, so the cells are independent.
__global__ void k_bc_reflecting(double* q, int64_t n, int64_t s0, int64_t s1, int64_t s2) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= n || j >= n) return;
  const bool gi = i < 3 || i >= n - 3, gj = j < 3 || j >= n - 3;
  if (!gi && !gj) return;
  int64_t si = i, sj = j;
  double sgn[8] = {1, 1, 1, 1, 1, 1, 1, 1};
  if (gi && gj) {
    si = i < 3 ? 5 - i : i - 3;
    sj = j < 3 ? 5 - j : j - 3;
    sgn[1] = sgn[2] = sgn[5] = sgn[6] = -1;
  } else if (gi) {
    si = i < 3 ? 5 - i : 2 * n - 7 - i;
    sgn[2] = sgn[6] = -1;
  } else {
    sj = j < 3 ? 5 - j : 2 * n - 7 - j;
    sgn[1] = sgn[5] = -1;
  }
  const double* src = q + si * s0 + sj * s1;
  double* dst = q + i * s0 + j * s1;
#pragma unroll
  for (int k = 0; k < 8; ++k) dst[k * s2] = src[k * s2] * sgn[k];
}

// unitest.py:169-204 init_refac before its boundary fill: primitive channels
// (rho, u, v, p) = (1.4, 0, 0, 1) everywhere, the post-shock state
// (8, 4.125, -7.1447, 116.5) in interior row i from column jrow(i) + 3 on
// (ghost columns included), jrow(i) = max(rint(y_s(x_i) / ly * ny), 0) with the
// shock line y_s(x) = sqrt(3) x - sqrt(3)/6 and x_i = (i - 3 + 0.5) / nx * lx
// (np.round rounds half to even, as rint does); conserved channels on the
// interior only, zero in the ghost cells.
__device__ __host__ inline int64_t refac_row(int64_t i, int64_t nx, int64_t ny, double lx, double ly) {
  const double x = ((double)(i - 3) + 0.5) / (double)nx * lx;
  const double y = sqrt(3.0) * x - sqrt(3.0) / 6.0;
  return (int64_t)rint(y / ly * (double)ny);
}

__global__ void k_init_refac(double* out, int64_t nx, int64_t ny, double lx, double ly, double gamma) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  const int64_t M = nx + 6, N = ny + 6;
  if (i >= M || j >= N) return;
  Prim4 s{1.4, 0.0, 0.0, 1.0};
  if (i >= 3 && i < nx + 3) {
    int64_t jr = refac_row(i, nx, ny, lx, ly);
    if (jr < 0) jr = 0;
    if (j >= jr + 3) s = Prim4{8.0, 4.125, -7.1447, 116.5};
  }
  double* o = out + (i * N + j) * 8;
  if (i >= 3 && i < nx + 3 && j >= 3 && j < ny + 3) {
    store_cell(o, s, gamma);
  } else {
    o[0] = o[1] = o[2] = o[3] = 0.0;
    o[4] = s.rho;
    o[5] = s.u;
    o[6] = s.v;
    o[7] = s.p;
  }
}

}  // namespace

extern "C" int weno_bc_reflecting(double* q, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2,
                                  void* stream) {
  if (!q) return weno::set_last_error(WENO_ERR_ARG, "bc_reflecting: null array");
  if (m != n || c != 8 || m < 9)
    return weno::set_last_error(WENO_ERR_SHAPE, "bc_reflecting: needs a square (n, n, 8) array with n >= 9 "
                                                "(the reference indexes axis 0 with the axis-1 extent)");
  const dim3 blk(32, 4), grd((unsigned)((n + 31) / 32), (unsigned)((m + 3) / 4));
  k_bc_reflecting<<<grd, blk, 0, static_cast<cudaStream_t>(stream)>>>(q, n, s0, s1, s2);
  cudaError_t e = cudaGetLastError();
  return e ? weno::set_last_error(WENO_ERR_CUDA, cudaGetErrorString(e)) : WENO_OK;
}

extern "C" int weno_init_refac(double* out, int64_t nx, int64_t ny, double lx, double ly, double gamma,
                               int64_t* bound_out, void* stream) {
  if (!out || nx < 10 || ny < 3 || !(lx > 0) || !(ly > 0))
    return weno::set_last_error(WENO_ERR_ARG, "init_refac: bad argument");
  // bound: the last interior row whose shock-line height rounds to the wall (unitest.py:186-190)
  int64_t bound = 0;
  for (int64_t i = 3; i < nx + 3; ++i)
    if (refac_row(i, nx, ny, lx, ly) == 0) bound = i;
  const int M = (int)nx + 6, N = (int)ny + 6;
  const dim3 blk(32, 4), grd((N + 31) / 32, (M + 3) / 4);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_init_refac<<<grd, blk, 0, st>>>(out, nx, ny, lx, ly, gamma);
  cudaError_t e = cudaGetLastError();
  if (e) return weno::set_last_error(WENO_ERR_CUDA, cudaGetErrorString(e));
  if (bound_out) *bound_out = bound;
  // unitest.py:205 apply_bc_refac with the driver's literal inflow vector (unitest.py:215)
  static const double post8[8] = {8, 33, -57.1576, 563.499, 8, 4.125, -7.1447, 116.5};
  weno::HostView v{out, N * 8, 8, 1};
  e = weno::Launch<double, false>::bc_dmr(v, 8, nx, ny, bound, post8, nullptr, st);
  return e ? weno::set_last_error(WENO_ERR_CUDA, cudaGetErrorString(e)) : WENO_OK;
}

extern "C" int weno_init_quadrant(double* out, int64_t nx, int64_t ny, int64_t si, int64_t sj, const double* prim16,
                                  double gamma, void* stream) {
  if (!out || !prim16 || nx < 1 || ny < 1) return weno::set_last_error(WENO_ERR_ARG, "init_quadrant: bad argument");
  Prim4 s[4];
  for (int k = 0; k < 4; ++k) s[k] = Prim4{prim16[4 * k], prim16[4 * k + 1], prim16[4 * k + 2], prim16[4 * k + 3]};
  const int M = (int)nx + 6, N = (int)ny + 6;
  const dim3 blk(32, 4), grd((N + 31) / 32, (M + 3) / 4);
  k_init_quadrant<<<grd, blk, 0, static_cast<cudaStream_t>(stream)>>>(out, M, N, (int)si, (int)sj, s[0], s[1], s[2],
                                                                      s[3], gamma);
  cudaError_t e = cudaGetLastError();
  return e ? weno::set_last_error(WENO_ERR_CUDA, cudaGetErrorString(e)) : WENO_OK;
}

extern "C" int weno_init_oblique_shock(double* out, int64_t nx, int64_t ny, double lx, double ly, double x0,
                                       double mach, double theta, double rho1, double p1, double gamma,
                                       int64_t* bound_out, double* post8_out, void* stream) {
  if (!out || nx < 3 || ny < 3 || !(mach > 1.0)) return weno::set_last_error(WENO_ERR_ARG, "init_oblique_shock: bad argument");
  // Normal-shock Rankine-Hugoniot relations; the gas behind moves along the
  // shock normal (sin theta, -cos theta).
  const double m2 = mach * mach;
  const double rho2 = rho1 * (gamma + 1.0) * m2 / ((gamma - 1.0) * m2 + 2.0);
  const double p2 = p1 * (2.0 * gamma * m2 - (gamma - 1.0)) / (gamma + 1.0);
  const double w = mach * std::sqrt(gamma * p1 / rho1);
  const double un = w * (1.0 - rho1 / rho2);
  const Prim4 post{rho2, un * std::sin(theta), -un * std::cos(theta), p2};
  const Prim4 pre{rho1, 0.0, 0.0, p1};
  const int M = (int)nx + 6, N = (int)ny + 6;
  const dim3 blk(32, 4), grd((N + 31) / 32, (M + 3) / 4);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_init_shock<<<grd, blk, 0, st>>>(out, (int)nx, (int)ny, lx, ly, x0, std::tan(theta), pre, post, gamma);
  cudaError_t e = cudaGetLastError();
  if (e) return weno::set_last_error(WENO_ERR_CUDA, cudaGetErrorString(e));
  double post8[8];
  post8[0] = post.rho;
  post8[1] = post.rho * post.u;
  post8[2] = post.rho * post.v;
  post8[3] = post.p / (gamma - 1.0) + 0.5 * post.rho * (post.u * post.u + post.v * post.v);
  post8[4] = post.rho;
  post8[5] = post.u;
  post8[6] = post.v;
  post8[7] = post.p;
  const int64_t bound = (int64_t)(3 + std::floor(x0 / (lx / nx) - 0.5));
  if (bound_out) *bound_out = bound;
  if (post8_out)
    for (int k = 0; k < 8; ++k) post8_out[k] = post8[k];
  // the oblique-shock boundary once, on all eight channels (unitest.py:205)
  weno::HostView v{out, N * 8, 8, 1};
  e = weno::Launch<double, false>::bc_dmr(v, 8, nx, ny, bound, post8, nullptr, st);
  return e ? weno::set_last_error(WENO_ERR_CUDA, cudaGetErrorString(e)) : WENO_OK;
}
