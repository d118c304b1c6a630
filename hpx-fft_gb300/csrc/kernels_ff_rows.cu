// rows kernels for the ArithFF compute type.
#define HPXFFT_DEFINE_ROWS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct RowLaunch<ArithFF>;
}
