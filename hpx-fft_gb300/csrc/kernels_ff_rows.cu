// rows kernels for the ArithFF compute type.
#define HPXFFT_DEFINE_ROWS
#include "launch.cuh"

namespace hpxfft_gpu {
template struct RowLaunch<ArithFF>;

cudaError_t RowLaunchFF16::prepare()
{
    cudaError_t e = set_attrs(row_r2c_kernel<ArithFF16, 1, 8192, 0>, false);
    return e == cudaSuccess ? set_attrs(row_r2c_kernel<ArithFF16D, 1, 8192, 0>, false) : e;
}

cudaError_t RowLaunchFF16::r2c(const RowArgs &a, const LaunchShape &s, cudaStream_t st)
{
    return launch_rows_ahead(row_r2c_kernel<ArithFF16, 1, 8192, 0>, a, s, 1, st);
}

cudaError_t RowLaunchFF16::halves(const RowArgs &a, const LaunchShape &s, cudaStream_t st)
{
    RowArgs b = a;
    b.prefetch = 0;  // the prefetch's row arithmetic is for whole rows
    return launch_rows_ahead(row_r2c_kernel<ArithFF16D, 1, 8192, 0>, b, s, 1, st);
}
}
