// df64 translation unit: the FAST forms evaluated in double-float arithmetic
// (about 48 significant bits) on the FP32 pipes -- the FP64-class solver mode
// that GB300's FP64:FP32 rate ratio of 1:64 favours.
#define WENO_TU_NS tu_df64
#include "launch_impl.cuh"

namespace weno {

template struct Launch<df64, true>;

}  // namespace weno
