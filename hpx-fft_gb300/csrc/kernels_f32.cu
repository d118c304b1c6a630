// Kernel instantiations for the ArithF32 compute type.
#define HPXFFT_DEFINE_LAUNCHERS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct Launch<ArithF32>;
}
