// Kernel instantiations for the ArithFF compute type.
#define HPXFFT_DEFINE_LAUNCHERS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct Launch<ArithFF>;
}
