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

}  // namespace

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
