// cols kernels for the ArithF32 compute type.
#define HPXFFT_DEFINE_COLS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct ColLaunch<ArithF32>;
template struct ColStepLaunch<ArithF32>;
}
