// Arithmetic-pipe throughput of the current device: FP32 FMA and FP64 FMA
// (hpxfft_measure_pipe_peaks).  The FP64 drop-in computes in float-float on
// the FP32 pipe because the FP64 pipe of this part retires far fewer FMAs;
// this measures both rates on the device the library runs on, so the ratio
// behind that choice is a number, not an assumption.
#include <cuda_runtime.h>

#include <string>

#include "../../include/hpxfft_gb300.h"

namespace hpxfft_gpu {

int set_error(int status, const std::string &msg);

// Eight independent FMA chains per thread (enough to cover the FMA latency
// with every warp slot of the SM occupied).  The final sum is compared with
// a value it cannot take, so the compiler keeps every chain.
template <class T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T *sink, int iters, T seed)
{
    const T m = (T)0.9999999, c = (T)1e-7;
    T a0 = seed + (T)threadIdx.x, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
    T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
#pragma unroll 4
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, m, c);
        a1 = fma(a1, m, c);
        a2 = fma(a2, m, c);
        a3 = fma(a3, m, c);
        a4 = fma(a4, m, c);
        a5 = fma(a5, m, c);
        a6 = fma(a6, m, c);
        a7 = fma(a7, m, c);
    }
    const T s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == (T)-1) sink[blockIdx.x] = s;
}

template <class T>
static cudaError_t time_chains(int blocks, int iters, void *sink, double *tflops)
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        fma_chain_kernel<T><<<blocks, 256>>>((T *)sink, iters / 8, (T)1);  // warm-up
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e0);
    if (e == cudaSuccess) {
        fma_chain_kernel<T><<<blocks, 256>>>((T *)sink, iters, (T)1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) *tflops = 2.0 * 8.0 * (double)iters * blocks * 256.0 / (1e-3 * ms) / 1e12;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return e;
}

}  // namespace hpxfft_gpu

extern "C" int hpxfft_measure_pipe_peaks(double *fp32_tflops, double *fp64_tflops)
{
    using namespace hpxfft_gpu;
    if (!fp32_tflops || !fp64_tflops) return set_error(HPXFFT_ERR_INVALID_ARG, "null argument");
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return set_error(HPXFFT_ERR_CUDA, std::string("device query: ") + cudaGetErrorString(e));
    const int blocks = 8 * sms;  // 2048 threads per SM
    void *sink = nullptr;
    if (cudaMalloc(&sink, sizeof(double) * blocks) != cudaSuccess) {
        cudaGetLastError();
        return set_error(HPXFFT_ERR_ALLOC, "pipe probe buffer");
    }
    // about 20 ms each at the rates of a GB300 (FP32 ~70, FP64 ~1.2 TFLOP/s)
    e = time_chains<float>(blocks, 1 << 18, sink, fp32_tflops);
    if (e == cudaSuccess) e = time_chains<double>(blocks, 1 << 12, sink, fp64_tflops);
    cudaFree(sink);
    if (e != cudaSuccess) return set_error(HPXFFT_ERR_CUDA, std::string("pipe probe: ") + cudaGetErrorString(e));
    return HPXFFT_OK;
}
