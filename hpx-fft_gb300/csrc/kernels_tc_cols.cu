// Split-BF16 tensor-core column steps and their DFT-matrix table.
#include "launch.cuh"
#include "tc_colstep.cuh"

namespace hpxfft_gpu {

#define HPXFFT_TC_LENGTHS(X) X(32) X(64) X(128) X(256)

// polls of the MMA completion barrier before a CTA reports a timeout
constexpr long long kTcSpinLimit = 1LL << 22;

cudaError_t TcColStepLaunch::prepare()
{
    cudaError_t e = cudaSuccess;
#define HPXFFT_X(L)                                                                                              \
    if ((e = cudaFuncSetAttribute(colstep_tc_kernel<-1, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,         \
                                  (int)kTcSmem)) != cudaSuccess)                                                  \
        return e;                                                                                                \
    if ((e = cudaFuncSetAttribute(colstep_tc_kernel<+1, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,         \
                                  (int)kTcSmem)) != cudaSuccess)                                                  \
        return e;
    HPXFFT_TC_LENGTHS(HPXFFT_X)
#undef HPXFFT_X
    return e;
}

bool TcColStepLaunch::supports(int L)
{
#define HPXFFT_X(L_) \
    if (L == L_) return true;
    HPXFFT_TC_LENGTHS(HPXFFT_X)
#undef HPXFFT_X
    return false;
}

int TcColStepLaunch::log2W(int L) { return ilog2c(kTcVectors / (L / 16)); }
int TcColStepLaunch::threads() { return kTcThreads; }
size_t TcColStepLaunch::smem() { return kTcSmem; }
size_t TcColStepLaunch::table_bytes() { return 2 * (size_t)kTcBBytes; }

cudaError_t TcColStepLaunch::table(void *dft, cudaStream_t st)
{
    tc_dft16_table_kernel<<<8, 256, 0, st>>>(reinterpret_cast<__nv_bfloat16 *>(dft));
    return cudaGetLastError();
}

cudaError_t TcColStepLaunch::run(const ColStepArgs &a, const void *dft, int *error, int dir, dim3 grid,
                                 cudaStream_t st)
{
    TcColStepArgs ta;
    ta.c = a;
    ta.dft = dft;
    ta.error = error;
    ta.spin_limit = kTcSpinLimit;
#define HPXFFT_X(L_)                                                                                   \
    if (a.L == L_) {                                                                                   \
        if (a.log2W != log2W(L_)) return cudaErrorInvalidValue;                                        \
        if (dir < 0)                                                                                   \
            colstep_tc_kernel<-1, L_><<<grid, kTcThreads, kTcSmem, st>>>(ta);                          \
        else                                                                                           \
            colstep_tc_kernel<+1, L_><<<grid, kTcThreads, kTcSmem, st>>>(ta);                          \
        return cudaGetLastError();                                                                     \
    }
    HPXFFT_TC_LENGTHS(HPXFFT_X)
#undef HPXFFT_X
    return cudaErrorInvalidValue;
}

}  // namespace hpxfft_gpu
