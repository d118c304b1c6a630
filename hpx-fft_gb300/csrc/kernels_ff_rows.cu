// rows kernels for the ArithFF compute type.
#define HPXFFT_DEFINE_ROWS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct RowLaunch<ArithFF>;

cudaError_t RowLaunchFF16::prepare() { return set_attrs(row_r2c_kernel<ArithFF16, 1, 8192, 0>, false); }

cudaError_t RowLaunchFF16::r2c(const RowArgs &a, const LaunchShape &s, cudaStream_t st)
{
    return launch_rows_ahead(row_r2c_kernel<ArithFF16, 1, 8192, 0>, a, s, 1, st);
}
}
