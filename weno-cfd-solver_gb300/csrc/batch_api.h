// Host-side launchers of the batched (tiled, fused) stage kernels.  Defined in
// batch_impl.cuh and compiled in batch_exact.cu (double, --fmad=false),
// batch_f64.cu (double, FAST) and batch_f32.cu (float, FAST).
#pragma once

#include <cuda_runtime.h>

namespace weno {

struct SolveDesc;
struct SolveCtl;

// Tile shapes (TX x TY interior cells per CTA) the autotuner chooses from:
// configurations 0-3 run the fused stage kernel k_stage_tiles; configuration 4
// (kStagedConfig) runs the staged kernels (pass 1, pass 2, residual in three
// launches per stage, faces in a global workspace) over 16 x 32 tiles.
constexpr int kNumTileConfigs = 5;
constexpr int kStagedConfig = 4;
constexpr int kTileTX[kNumTileConfigs] = {8, 16, 16, 8, 16};
constexpr int kTileTY[kNumTileConfigs] = {32, 32, 16, 64, 32};

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
  // One stage of the staged configuration: three launches (pass 1 of Qs into
  // the workspace, pass 2 and the Riemann solvers, residual and combination).
  static cudaError_t staged(bool chr, bool blend, const SolveDesc* solves, SolveCtl* ctl, const void* tiles,
                            int ntiles, int grid, const void* qs, const void* qn, void* qo, void* ws, int stage,
                            double gamma, double jp_lo, double jp_hi, double weps, cudaStream_t st);
  static cudaError_t cfl(int cfg, const SolveDesc* solves, SolveCtl* ctl, const void* tiles, int ntiles, int grid,
                         const void* q, double gamma, cudaStream_t st);
  static cudaError_t clock(SolveCtl* ctl, int nsolves, int phase, cudaStream_t st);
};

extern template struct BatchLaunch<double, false>;
extern template struct BatchLaunch<double, true>;
extern template struct BatchLaunch<float, true>;

}  // namespace weno
