// Fast translation unit: FMA contraction on, FAST arithmetic forms.  FP64
// results agree with the reference to rounding (checked by tolerance against
// the oracle); FP32 is the bulk-precision variant.
#define WENO_TU_NS tu_fast
#include "launch_impl.cuh"

namespace weno {

template struct Launch<double, true>;
template struct Launch<float, true>;

}  // namespace weno
