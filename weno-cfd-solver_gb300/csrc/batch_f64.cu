// Batched stage kernels, double, FAST forms with FMA.
#define WENO_TU_NS batch_f64
#include "batch_impl.cuh"

namespace weno {
template struct BatchLaunch<double, true>;
}
