// Batched stage kernels, double, reference operation order, --fmad=false:
// bit-identical to the oracle (used to prove the fused tile pipeline).
#define WENO_TU_NS batch_exact
#include "batch_impl.cuh"

namespace weno {
template struct BatchLaunch<double, false>;
}
