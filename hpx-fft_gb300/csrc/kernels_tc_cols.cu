// Split-BF16 tensor-core column steps, rows and their DFT-matrix table.
#include "launch.cuh"
#include "tc_colstep.cuh"

namespace hpxfft_gpu {

#define HPXFFT_TC_LENGTHS(X) X(32) X(64) X(128) X(256)
#define HPXFFT_TC_SHAPES(X) X(32, 512) X(64, 512) X(128, 512) X(256, 512) X(32, 256) X(64, 256) X(128, 256) X(256, 256)

// polls of the MMA completion barrier before a CTA reports a timeout
constexpr long long kTcSpinLimit = 1LL << 22;

cudaError_t TcColStepLaunch::prepare()
{
    cudaError_t e = cudaSuccess;
#define HPXFFT_X(L, NV)                                                                                          \
    if ((e = cudaFuncSetAttribute(colstep_tc_kernel<-1, L, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                  (int)tc_smem(NV))) != cudaSuccess)                                              \
        return e;                                                                                                \
    if ((e = cudaFuncSetAttribute(colstep_tc_kernel<+1, L, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                  (int)tc_smem(NV))) != cudaSuccess)                                              \
        return e;
    HPXFFT_TC_SHAPES(HPXFFT_X)
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

int TcColStepLaunch::log2W(int L, int nv) { return ilog2c(nv / (L / 16)); }
int TcColStepLaunch::threads(int nv) { return nv; }
size_t TcColStepLaunch::smem(int nv) { return tc_smem(nv); }
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
#define HPXFFT_X(L_, NV)                                                                               \
    if (a.L == L_ && a.log2W == log2W(L_, NV)) {                                                       \
        if (dir < 0)                                                                                   \
            colstep_tc_kernel<-1, L_, NV><<<grid, NV, tc_smem(NV), st>>>(ta);                          \
        else                                                                                           \
            colstep_tc_kernel<+1, L_, NV><<<grid, NV, tc_smem(NV), st>>>(ta);                          \
        return cudaGetLastError();                                                                     \
    }
    HPXFFT_TC_SHAPES(HPXFFT_X)
#undef HPXFFT_X
    return cudaErrorInvalidValue;
}

#define HPXFFT_TC_ROWS(X) X(8192, 0) X(4096, 1) X(2048, 2) X(1024, 3) X(512, 4) X(256, 4) X(128, 4)

cudaError_t TcRowLaunch::prepare()
{
    cudaError_t e = cudaSuccess;
#define HPXFFT_X(L, W)                                                                                           \
    if ((e = cudaFuncSetAttribute(row_r2c_tc_kernel<L, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,          \
                                  (int)tc_smem(L * (1 << W) / 16))) != cudaSuccess)                               \
        return e;
    HPXFFT_TC_ROWS(HPXFFT_X)
#undef HPXFFT_X
    return e;
}

bool TcRowLaunch::supports(int M, int log2W, int C)
{
    if (C != 1) return false;
#define HPXFFT_X(L_, W_) \
    if (M == L_ && log2W == W_) return true;
    HPXFFT_TC_ROWS(HPXFFT_X)
#undef HPXFFT_X
    return false;
}

int TcRowLaunch::threads(int M, int log2W) { return (M << log2W) / 16; }
size_t TcRowLaunch::smem(int M, int log2W) { return tc_smem((M << log2W) / 16); }

cudaError_t TcRowLaunch::run(const RowArgs &a, const void *dft, int *error, dim3 grid, cudaStream_t st)
{
    TcRowArgs ta;
    ta.r = a;
    ta.dft = dft;
    ta.error = error;
    ta.spin_limit = kTcSpinLimit;
#define HPXFFT_X(L_, W_)                                                                                \
    if (a.M == L_ && a.log2W == W_) {                                                                   \
        row_r2c_tc_kernel<L_, W_><<<grid, (L_ << W_) / 16, tc_smem((L_ << W_) / 16), st>>>(ta);         \
        return cudaGetLastError();                                                                      \
    }
    HPXFFT_TC_ROWS(HPXFFT_X)
#undef HPXFFT_X
    return cudaErrorInvalidValue;
}

}  // namespace hpxfft_gpu
