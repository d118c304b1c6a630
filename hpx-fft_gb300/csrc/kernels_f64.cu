// Kernel instantiations for the ArithF64 compute type.
#define HPXFFT_DEFINE_LAUNCHERS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct Launch<ArithF64>;
}
