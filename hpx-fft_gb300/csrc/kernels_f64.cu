// Row and column kernels for native FP64 (DFMA) arithmetic: runtime radix
// plans only (a cross-check path; GB300's FP64 rate is 1/58 of FP32).
#define HPXFFT_DEFINE_ROWS
#define HPXFFT_DEFINE_COLS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct RowLaunch<ArithF64>;
template struct ColLaunch<ArithF64>;
template struct ColStepLaunch<ArithF64>;
}
