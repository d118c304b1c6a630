// Twiddle-table generators (FP64 sincospi, rounded to each compute type).
#define HPXFFT_DEFINE_TWIDDLES
#include "launch.cuh"

namespace hpxfft_gpu {
template struct TwiddleLaunch<ArithF32>;
template struct TwiddleLaunch<ArithF64>;
template struct TwiddleLaunch<ArithFF>;
}
