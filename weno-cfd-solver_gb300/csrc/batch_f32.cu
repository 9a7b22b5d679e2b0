// Batched stage kernels, float (the FP32 bulk precision), FAST forms.
#define WENO_TU_NS batch_f32
#include "batch_impl.cuh"

namespace weno {
template struct BatchLaunch<float, true>;
}
