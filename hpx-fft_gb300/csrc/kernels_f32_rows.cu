// rows kernels for the ArithF32 compute type.
#define HPXFFT_DEFINE_ROWS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct RowLaunch<ArithF32>;
}
