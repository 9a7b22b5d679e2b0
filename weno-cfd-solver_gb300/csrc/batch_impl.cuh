// Batched launcher definitions (see batch_api.h).
#pragma once

#include "batch_api.h"
#include "batch_kernels.cuh"

namespace weno {

inline namespace WENO_TU_NS {
namespace bdetail {

constexpr int kNT = 256;

template <class T, int TX, int TY, bool BLEND>
constexpr size_t tile_smem() {
  return sizeof(T) * (size_t)TileGeom<TX, TY, BLEND>::TOTAL;
}

template <class T, bool FAST, bool CHAR, bool BLEND, int TX, int TY>
cudaError_t launch_stage(const SolveDesc* solves, SolveCtl* ctl, const int4* tiles, int ntiles, int grid,
                         const CUtensorMap* tmaps, const T* qn, T* qo, int stage, T gamma, T jp_lo, T jp_hi, T weps,
                         int skip_tile, unsigned long long wait_ns, cudaStream_t st) {
  constexpr size_t sm = tile_smem<T, TX, TY, BLEND>();
  if constexpr (sm > 227 * 1024) {
    return cudaErrorInvalidConfiguration;
  } else {
    auto k = k_stage_tiles<T, FAST, CHAR, BLEND, TX, TY, kNT>;
    // The attribute is per device and cheap to set: set it on every launch (also
    // keeps host threads from racing on a cached flag).
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k<<<grid, kNT, sm, st>>>(solves, ctl, tiles, ntiles, tmaps, qn, qo, stage, gamma, jp_lo, jp_hi, weps, skip_tile,
                             wait_ns);
    return cudaGetLastError();
  }
}

template <class T, bool FAST, bool CHAR, bool BLEND, int TX, int TY>
int occupancy() {
  constexpr size_t sm = tile_smem<T, TX, TY, BLEND>();
  if constexpr (sm > 227 * 1024) {
    return 0;
  } else {
    auto k = k_stage_tiles<T, FAST, CHAR, BLEND, TX, TY, kNT>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kNT, sm) != cudaSuccess) return 0;
    return n;
  }
}

}  // namespace bdetail
}  // inline namespace WENO_TU_NS

// Fused configurations only (0-3); the staged configuration has its own launcher.
#define WENO_TILE_SWITCH(cfg, MACRO) \
  switch (cfg) {                     \
    case 0: MACRO(8, 32); break;     \
    case 1: MACRO(16, 32); break;    \
    case 2: MACRO(16, 16); break;    \
    default: MACRO(8, 64); break;    \
  }

template <class T, bool FAST>
void BatchLaunch<T, FAST>::box(int cfg, bool blend, unsigned* cols, unsigned* rows) {
#define WENO_BOX(TX, TY)                                      \
  *cols = (unsigned)TileGeom<TX, TY, false>::UC;              \
  *rows = blend ? (unsigned)TileGeom<TX, TY, true>::UR : (unsigned)TileGeom<TX, TY, false>::UR;
  WENO_TILE_SWITCH(cfg, WENO_BOX)
#undef WENO_BOX
}

template <class T, bool FAST>
size_t BatchLaunch<T, FAST>::smem_bytes(int cfg, bool blend) {
  size_t r = 0;
#define WENO_SM(TX, TY) \
  r = blend ? bdetail::tile_smem<T, TX, TY, true>() : bdetail::tile_smem<T, TX, TY, false>()
  WENO_TILE_SWITCH(cfg, WENO_SM)
#undef WENO_SM
  return r > 227 * 1024 ? 0 : r;
}

template <class T, bool FAST>
int BatchLaunch<T, FAST>::ctas_per_sm(int cfg, bool chr, bool blend) {
  int r = 0;
#define WENO_OCC(TX, TY)                                                                   \
  if (chr && blend) r = bdetail::occupancy<T, FAST, true, true, TX, TY>();                 \
  else if (chr) r = bdetail::occupancy<T, FAST, true, false, TX, TY>();                    \
  else if (blend) r = bdetail::occupancy<T, FAST, false, true, TX, TY>();                  \
  else r = bdetail::occupancy<T, FAST, false, false, TX, TY>();
  WENO_TILE_SWITCH(cfg, WENO_OCC)
#undef WENO_OCC
  return r;
}

template <class T, bool FAST>
cudaError_t BatchLaunch<T, FAST>::stage(int cfg, bool chr, bool blend, const SolveDesc* solves, SolveCtl* ctl,
                                        const void* tiles, int ntiles, int grid, const void* tmaps, const void* qn,
                                        void* qo, int stage, double gamma, double jp_lo, double jp_hi,
                                        double weps, int skip_tile, unsigned long long wait_ns, cudaStream_t st) {
  if (ntiles <= 0 || grid <= 0) return cudaSuccess;
  const int4* tl = static_cast<const int4*>(tiles);
  const CUtensorMap* a = static_cast<const CUtensorMap*>(tmaps);
  const T* b = static_cast<const T*>(qn);
  T* o = static_cast<T*>(qo);
  cudaError_t e = cudaSuccess;
#define WENO_ST(TX, TY)                                                                                           \
  if (chr && blend)                                                                                               \
    e = bdetail::launch_stage<T, FAST, true, true, TX, TY>(solves, ctl, tl, ntiles, grid, a, b, o, stage, (T)gamma, \
                                                           (T)jp_lo, (T)jp_hi, (T)weps, skip_tile, wait_ns, st);                               \
  else if (chr)                                                                                                   \
    e = bdetail::launch_stage<T, FAST, true, false, TX, TY>(solves, ctl, tl, ntiles, grid, a, b, o, stage,         \
                                                            (T)gamma, (T)jp_lo, (T)jp_hi, (T)weps, skip_tile, wait_ns, st);                    \
  else if (blend)                                                                                                 \
    e = bdetail::launch_stage<T, FAST, false, true, TX, TY>(solves, ctl, tl, ntiles, grid, a, b, o, stage,         \
                                                            (T)gamma, (T)jp_lo, (T)jp_hi, (T)weps, skip_tile, wait_ns, st);                    \
  else                                                                                                            \
    e = bdetail::launch_stage<T, FAST, false, false, TX, TY>(solves, ctl, tl, ntiles, grid, a, b, o, stage,        \
                                                             (T)gamma, (T)jp_lo, (T)jp_hi, (T)weps, skip_tile, wait_ns, st);
  WENO_TILE_SWITCH(cfg, WENO_ST)
#undef WENO_ST
  return e;
}

template <class T, bool FAST>
cudaError_t BatchLaunch<T, FAST>::staged(bool chr, bool blend, const SolveDesc* solves, SolveCtl* ctl,
                                         const void* tiles, int ntiles, int grid, const void* qs, const void* qn,
                                         void* qo, void* ws, int stage, double gamma, double jp_lo, double jp_hi,
                                         double weps, cudaStream_t st) {
  if (ntiles <= 0 || grid <= 0) return cudaSuccess;
  constexpr int TX = kTileTX[kStagedConfig], TY = kTileTY[kStagedConfig], NT = bdetail::kNT;
  const int4* tl = static_cast<const int4*>(tiles);
  T* W = static_cast<T*>(ws);
  const T* Qs = static_cast<const T*>(qs);
  if (chr)
    k_staged_pass1<T, FAST, true, TX, TY, NT><<<grid, NT, 0, st>>>(solves, ctl, tl, ntiles, Qs, W, (T)gamma, (T)weps);
  else
    k_staged_pass1<T, FAST, false, TX, TY, NT><<<grid, NT, 0, st>>>(solves, ctl, tl, ntiles, Qs, W, (T)gamma,
                                                                     (T)weps);
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  if (blend)
    k_staged_pass2<T, FAST, true, TX, TY, NT><<<grid, NT, 0, st>>>(solves, ctl, tl, ntiles, W, (T)gamma, (T)weps);
  else
    k_staged_pass2<T, FAST, false, TX, TY, NT><<<grid, NT, 0, st>>>(solves, ctl, tl, ntiles, W, (T)gamma, (T)weps);
  if ((e = cudaGetLastError())) return e;
  const T* Qn = static_cast<const T*>(qn);
  T* Qo = static_cast<T*>(qo);
  if (blend)
    k_staged_residual<T, FAST, true, TX, TY, NT><<<grid, NT, 0, st>>>(solves, ctl, tl, ntiles, W, Qs, Qn, Qo, stage,
                                                                       (T)gamma, (T)jp_lo, (T)jp_hi);
  else
    k_staged_residual<T, FAST, false, TX, TY, NT><<<grid, NT, 0, st>>>(solves, ctl, tl, ntiles, W, Qs, Qn, Qo,
                                                                        stage, (T)gamma, (T)jp_lo, (T)jp_hi);
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t BatchLaunch<T, FAST>::cfl(int cfg, const SolveDesc* solves, SolveCtl* ctl, const void* tiles, int ntiles,
                                      int grid, const void* q, double gamma, cudaStream_t st) {
  if (ntiles <= 0 || grid <= 0) return cudaSuccess;
  const int tx = kTileTX[cfg < kNumTileConfigs ? cfg : 0], ty = kTileTY[cfg < kNumTileConfigs ? cfg : 0];
  k_cfl_tiles<T, bdetail::kNT><<<grid, bdetail::kNT, 0, st>>>(solves, ctl, static_cast<const int4*>(tiles), ntiles,
                                                              tx, ty, static_cast<const T*>(q), (T)gamma);
  return cudaGetLastError();
}

template <class T, bool FAST>
cudaError_t BatchLaunch<T, FAST>::clock(SolveCtl* ctl, int nsolves, int phase, cudaStream_t st) {
  if (nsolves <= 0) return cudaSuccess;
  k_solve_clock<<<(nsolves + 127) / 128, 128, 0, st>>>(ctl, nsolves, phase);
  return cudaGetLastError();
}

#undef WENO_TILE_SWITCH

}  // namespace weno
