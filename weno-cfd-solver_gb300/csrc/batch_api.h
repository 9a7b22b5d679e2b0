// Host-side launchers of the batched (tiled, fused) stage kernels.  Defined in
// batch_impl.cuh and compiled in batch_exact.cu (double, --fmad=false),
// batch_f64.cu (double, FAST) and batch_f32.cu (float, FAST).
#pragma once

#include <cuda_runtime.h>

namespace weno {

struct SolveDesc;
struct SolveCtl;

// Tile shapes (TX x TY interior cells per CTA) the autotuner chooses from.
constexpr int kNumTileConfigs = 4;
constexpr int kTileTX[kNumTileConfigs] = {8, 16, 16, 8};
constexpr int kTileTY[kNumTileConfigs] = {32, 32, 16, 64};

template <class T, bool FAST>
struct BatchLaunch {
  // TMA box of one tile: columns (innermost, also the shared-memory row pitch) and rows.
  static void box(int cfg, bool blend, unsigned* cols, unsigned* rows);
  // Shared memory bytes of one CTA, or 0 if the configuration does not fit.
  static size_t smem_bytes(int cfg, bool blend);
  // Resident CTAs per SM for the configuration (0 if it cannot launch).
  static int ctas_per_sm(int cfg, bool chr, bool blend);
  static cudaError_t stage(int cfg, bool chr, bool blend, const SolveDesc* solves, SolveCtl* ctl, const void* tiles,
                           int ntiles, int grid, const void* tmaps, const void* qn, void* qo, int stage, double gamma,
                           double jp_lo, double jp_hi, double weps, int skip_tile, unsigned long long wait_ns,
                           cudaStream_t st);
  static cudaError_t cfl(int cfg, const SolveDesc* solves, SolveCtl* ctl, const void* tiles, int ntiles, int grid,
                         const void* q, double gamma, cudaStream_t st);
  static cudaError_t clock(SolveCtl* ctl, int nsolves, int phase, cudaStream_t st);
};

extern template struct BatchLaunch<double, false>;
extern template struct BatchLaunch<double, true>;
extern template struct BatchLaunch<float, true>;

}  // namespace weno
