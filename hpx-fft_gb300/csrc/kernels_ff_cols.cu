// cols kernels for the ArithFF compute type.
#define HPXFFT_DEFINE_COLS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct ColLaunch<ArithFF>;
template struct ColStepLaunch<ArithFF>;
}
