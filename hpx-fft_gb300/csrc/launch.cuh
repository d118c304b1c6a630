// Launchers for the transform kernels of one compute type.  Each
// kernels_<type>.cu instantiates them for its type, so the three compute
// types compile in parallel.
#pragma once
#include <cuda_runtime.h>

#include "fft_kernels.cuh"

namespace hpxfft_gpu {

struct LaunchShape {
    dim3 grid;
    int threads;
    size_t smem;
    int cluster;
};

template <class A>
struct Launch {
    // Raise the dynamic shared memory limit and allow 16-CTA clusters.
    static cudaError_t prepare();
    static cudaError_t row_r2c(const RowArgs &a, const LaunchShape &s, cudaStream_t st);
    static cudaError_t row_c2r(const RowArgs &a, const LaunchShape &s, cudaStream_t st);
    static cudaError_t col(const ColArgs &a, int dir, const LaunchShape &s, cudaStream_t st);
    static cudaError_t twiddles(void *tab, int n, cudaStream_t st);
};

#ifdef HPXFFT_DEFINE_LAUNCHERS
template <class K, class Args>
static cudaError_t launch_cluster(K kernel, const Args &a, const LaunchShape &s, cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = s.grid;
    cfg.blockDim = dim3((unsigned)s.threads, 1, 1);
    cfg.dynamicSmemBytes = s.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)s.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, a);
}

template <class K>
static cudaError_t set_attrs(K kernel, bool nonportable)
{
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    if (nonportable) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}

template <class A>
cudaError_t Launch<A>::prepare()
{
    cudaError_t e = cudaSuccess;
#define HPXFFT_TRY(x)                 \
    do {                              \
        e = (x);                      \
        if (e != cudaSuccess) return e; \
    } while (0)
    HPXFFT_TRY(set_attrs(row_r2c_kernel<A, 1>, false));
    HPXFFT_TRY(set_attrs(row_r2c_kernel<A, 2>, false));
    HPXFFT_TRY(set_attrs(row_r2c_kernel<A, 4>, false));
    HPXFFT_TRY(set_attrs(row_c2r_kernel<A, 1>, false));
    HPXFFT_TRY(set_attrs(row_c2r_kernel<A, 2>, false));
    HPXFFT_TRY(set_attrs(row_c2r_kernel<A, 4>, false));
    HPXFFT_TRY(set_attrs(col_kernel<A, 1, -1>, false));
    HPXFFT_TRY(set_attrs(col_kernel<A, 2, -1>, false));
    HPXFFT_TRY(set_attrs(col_kernel<A, 4, -1>, false));
    HPXFFT_TRY(set_attrs(col_kernel<A, 8, -1>, false));
    HPXFFT_TRY(set_attrs(col_kernel<A, 16, -1>, true));
    HPXFFT_TRY(set_attrs(col_kernel<A, 1, +1>, false));
    HPXFFT_TRY(set_attrs(col_kernel<A, 2, +1>, false));
    HPXFFT_TRY(set_attrs(col_kernel<A, 4, +1>, false));
    HPXFFT_TRY(set_attrs(col_kernel<A, 8, +1>, false));
    HPXFFT_TRY(set_attrs(col_kernel<A, 16, +1>, true));
#undef HPXFFT_TRY
    return e;
}

template <class A>
cudaError_t Launch<A>::row_r2c(const RowArgs &a, const LaunchShape &s, cudaStream_t st)
{
    switch (s.cluster) {
    case 1: return launch_cluster(row_r2c_kernel<A, 1>, a, s, st);
    case 2: return launch_cluster(row_r2c_kernel<A, 2>, a, s, st);
    case 4: return launch_cluster(row_r2c_kernel<A, 4>, a, s, st);
    default: return cudaErrorInvalidValue;
    }
}

template <class A>
cudaError_t Launch<A>::row_c2r(const RowArgs &a, const LaunchShape &s, cudaStream_t st)
{
    switch (s.cluster) {
    case 1: return launch_cluster(row_c2r_kernel<A, 1>, a, s, st);
    case 2: return launch_cluster(row_c2r_kernel<A, 2>, a, s, st);
    case 4: return launch_cluster(row_c2r_kernel<A, 4>, a, s, st);
    default: return cudaErrorInvalidValue;
    }
}

template <class A>
cudaError_t Launch<A>::col(const ColArgs &a, int dir, const LaunchShape &s, cudaStream_t st)
{
    if (dir < 0) {
        switch (s.cluster) {
        case 1: return launch_cluster(col_kernel<A, 1, -1>, a, s, st);
        case 2: return launch_cluster(col_kernel<A, 2, -1>, a, s, st);
        case 4: return launch_cluster(col_kernel<A, 4, -1>, a, s, st);
        case 8: return launch_cluster(col_kernel<A, 8, -1>, a, s, st);
        case 16: return launch_cluster(col_kernel<A, 16, -1>, a, s, st);
        default: return cudaErrorInvalidValue;
        }
    }
    switch (s.cluster) {
    case 1: return launch_cluster(col_kernel<A, 1, +1>, a, s, st);
    case 2: return launch_cluster(col_kernel<A, 2, +1>, a, s, st);
    case 4: return launch_cluster(col_kernel<A, 4, +1>, a, s, st);
    case 8: return launch_cluster(col_kernel<A, 8, +1>, a, s, st);
    case 16: return launch_cluster(col_kernel<A, 16, +1>, a, s, st);
    default: return cudaErrorInvalidValue;
    }
}

template <class A>
cudaError_t Launch<A>::twiddles(void *tab, int n, cudaStream_t st)
{
    using T = typename A::T;
    const int threads = 256;
    twiddle_kernel<T><<<(n + threads - 1) / threads, threads, 0, st>>>(reinterpret_cast<cpx<T> *>(tab), n);
    return cudaGetLastError();
}
#endif

}  // namespace hpxfft_gpu
