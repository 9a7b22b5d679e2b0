// Exact translation unit: compiled with --fmad=false so that every a*b+c is
// two IEEE-754 operations, as in the reference's Rust core.  With the
// reference's operation order (FAST = false) the doubles produced here are
// bit-identical to the Rust ones.
#define WENO_TU_NS tu_exact
#include "launch_impl.cuh"

namespace weno {

template struct Launch<double, false>;

cudaError_t launch_dt(StepCtl* ctl, cudaStream_t st) {
  k_dt<<<1, 1, 0, st>>>(ctl);
  return cudaGetLastError();
}

cudaError_t launch_step_end(StepCtl* ctl, cudaStream_t st) {
  k_step_end<<<1, 1, 0, st>>>(ctl);
  return cudaGetLastError();
}

cudaError_t launch_run_begin(StepCtl* ctl, double t_final, long long add, cudaStream_t st) {
  k_run_begin<<<1, 1, 0, st>>>(ctl, t_final, add);
  return cudaGetLastError();
}

}  // namespace weno
