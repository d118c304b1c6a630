// Launchers for the transform kernels of one compute type.  Row kernels,
// column kernels and twiddle generators are defined in separate translation
// units (kernels_<type>_{rows,cols}.cu) so they compile in parallel.
#pragma once
#include <cuda_runtime.h>

#include <mutex>

#include "fft_kernels.cuh"

namespace hpxfft_gpu {

struct LaunchShape {
    dim3 grid;
    int threads;
    size_t smem;
    int cluster;
};

// Compile-time configurations (local length L, log2 interleave, cluster size)
// for power-of-two sizes: at most 4096 float-float or 8192 FP32 elements per
// CTA (64 KB of data), the shapes the planner picks.
// Rows: one row per CTA up to that size (shorter rows packed), longer rows
// split over a cluster; float-float rows of 8192 pairs also run as one
// 1024-thread CTA (no cluster exchange), which the planner prefers.
#define HPXFFT_ROW_FIXED_FF(X) X(8192, 0, 1) X(8192, 0, 2) X(4096, 0, 1) X(4096, 0, 2) X(4096, 0, 4) X(2048, 1, 1) X(1024, 2, 1) X(512, 3, 1) X(256, 4, 1) X(128, 4, 1)
#define HPXFFT_ROW_FIXED_F32(X) X(8192, 0, 1) X(8192, 0, 2) X(4096, 1, 1) X(2048, 2, 1) X(1024, 3, 1) X(512, 4, 1) X(256, 4, 1) X(128, 4, 1)
// Columns: strips of 4 (float-float) or 8 (FP32) columns, 64-byte row
// segments; nx >= 2048 splits into local length 1024 over 2..16 CTAs.
#define HPXFFT_COL_FIXED_FF(X) X(256, 2, 1) X(512, 2, 1) X(1024, 2, 1) X(1024, 2, 2) X(1024, 2, 4) X(1024, 2, 8) X(1024, 2, 16) X(2048, 1, 16)
#define HPXFFT_COL_FIXED_F32(X) X(256, 3, 1) X(512, 3, 1) X(1024, 3, 1) X(1024, 3, 2) X(1024, 3, 4) X(1024, 3, 8) X(1024, 3, 16) X(2048, 2, 16)

template <class A>
struct RowLaunch {
    static cudaError_t prepare();
    static bool has_fixed(int L, int log2W, int C);
    // FL = 0 selects the runtime radix plan
    static cudaError_t r2c(const RowArgs &a, const LaunchShape &s, int FL, cudaStream_t st);
    static cudaError_t c2r(const RowArgs &a, const LaunchShape &s, int FL, cudaStream_t st);
};

// The float-float 8192-pair row with radix-16 passes (ArithFF16).
struct RowLaunchFF16 {
    static cudaError_t prepare();
    static cudaError_t r2c(const RowArgs &a, const LaunchShape &s, cudaStream_t st);
    // the two halves of rows of 16384 pairs as rows of their own (ArithFF16D)
    static cudaError_t halves(const RowArgs &a, const LaunchShape &s, cudaStream_t st);
};

template <class A>
struct ColLaunch {
    static constexpr int kLog2W = sizeof(typename A::S) == 4 ? 3 : 2;  // 64-byte row segments
    static cudaError_t prepare();
    static bool has_fixed(int L, int log2W, int C);
    static cudaError_t run(const ColArgs &a, int dir, const LaunchShape &s, int FL, cudaStream_t st);
};

// Two-kernel column steps: (DFT length, log2 strip width), strips of up to 64
// columns (512-byte float-float / FP32 segments of 32 / 64 columns).
#define HPXFFT_COLSTEP_FIXED_FF(X) X(32, 6) X(64, 6) X(128, 5) X(256, 4)
#define HPXFFT_COLSTEP_FIXED_F32(X) X(32, 6) X(64, 6) X(128, 6) X(256, 5)

template <class A>
struct ColStepLaunch {
    static cudaError_t prepare();
    static bool has_fixed(int L, int log2W);
    static cudaError_t run(const ColStepArgs &a, int dir, const LaunchShape &s, int FL, cudaStream_t st);
};

// Split-BF16 tensor-core column steps (kernels_tc_cols.cu): lengths 16 * L2,
// L2 in {2, 4, 8, 16}, nv = 512 or 256 length-16 vectors per CTA.
struct TcColStepLaunch {
    static cudaError_t prepare();
    static bool supports(int L);
    static int log2W(int L, int nv);  // columns per CTA: 16 nv / L
    static int threads(int nv);
    static size_t smem(int nv);
    static size_t table_bytes();
    static cudaError_t table(void *dft, cudaStream_t st);
    static cudaError_t run(const ColStepArgs &a, const void *dft, int *error, int dir, dim3 grid, cudaStream_t st);
};

// Split-BF16 row r2c (kernels_tc_cols.cu): compiled (M, log2 rows per CTA)
// shapes of the FP32 row plan with 128, 256 or 512 length-16 vectors per CTA.
struct TcRowLaunch {
    static cudaError_t prepare();
    static bool supports(int M, int log2W, int C);
    static int threads(int M, int log2W);
    static size_t smem(int M, int log2W);
    static cudaError_t run(const RowArgs &a, const void *dft, int *error, dim3 grid, cudaStream_t st);
};

template <class A>
struct TwiddleLaunch {
    static cudaError_t full(void *tab, int n, cudaStream_t st);
    static cudaError_t pass(void *tab, int Ls, int R, cudaStream_t st);
};

#if defined(HPXFFT_DEFINE_ROWS) || defined(HPXFFT_DEFINE_COLS) || defined(HPXFFT_DEFINE_TWIDDLES)
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

// CTAs of `kernel` with shape s resident on the device at once, cached per
// kernel, device and shape in a fixed table (no heap use: the allocation-free
// entry point launches these kernels too); 0 if the query fails.
struct ResidentEntry {
    const void *kernel;
    int dev, threads;
    size_t smem;
    int n;
};
template <class K>
static int resident_ctas(K kernel, const LaunchShape &s)
{
    static std::mutex mu;
    static ResidentEntry table[128];
    static int used = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::lock_guard<std::mutex> lock(mu);
    for (int i = 0; i < used; ++i)
        if (table[i].kernel == (const void *)kernel && table[i].dev == dev && table[i].threads == s.threads &&
            table[i].smem == s.smem)
            return table[i].n;
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, s.threads, s.smem) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (used < 128) table[used++] = ResidentEntry{(const void *)kernel, dev, s.threads, s.smem, per_sm * sms};
    return per_sm * sms;
}

// A grid of at most one wave for a kernel that loops over its blocks' work.
template <class K, class Args>
static cudaError_t launch_persistent(K kernel, const Args &a, const LaunchShape &s, cudaStream_t st)
{
    LaunchShape p = s;
    const int n = resident_ctas(kernel, s);
    if (n > 0 && (int)p.grid.x > n) p.grid.x = (unsigned)n;
    return launch_cluster(kernel, a, p, st);
}

// One row group per CTA: each CTA prefetches into L2 the group of the CTA
// that will take its place (block + resident CTAs), so that CTA's
// first-pass loads hit L2 (single-CTA shapes, device input only).
template <class K>
static cudaError_t launch_rows_ahead(K kernel, const RowArgs &a, const LaunchShape &s, int C, cudaStream_t st)
{
    RowArgs b = a;
    b.prefetch_ahead = C == 1 && a.prefetch ? resident_ctas(kernel, s) : 0;
    return launch_cluster(kernel, b, s, st);
}

template <class K>
static cudaError_t set_attrs(K kernel, bool nonportable)
{
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    if (e != cudaSuccess) return e;
    if (nonportable) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
}
#define HPXFFT_TRY(x)                   \
    do {                                \
        cudaError_t e_ = (x);           \
        if (e_ != cudaSuccess) return e_; \
    } while (0)
#endif

#ifdef HPXFFT_DEFINE_ROWS
template <class A>
cudaError_t RowLaunch<A>::prepare()
{
    HPXFFT_TRY(set_attrs(row_r2c_kernel<A, 1, 0, 0>, false));
    HPXFFT_TRY(set_attrs(row_r2c_kernel<A, 2, 0, 0>, false));
    HPXFFT_TRY(set_attrs(row_r2c_kernel<A, 4, 0, 0>, false));
    HPXFFT_TRY(set_attrs(row_c2r_kernel<A, 1, 0, 0>, false));
    HPXFFT_TRY(set_attrs(row_c2r_kernel<A, 2, 0, 0>, false));
    HPXFFT_TRY(set_attrs(row_c2r_kernel<A, 4, 0, 0>, false));
    if constexpr (A::kFixedChains) {
#define HPXFFT_X(L, W, C)                                                  \
    HPXFFT_TRY(set_attrs(row_r2c_kernel<A, C, L, W>, false));              \
    HPXFFT_TRY(set_attrs(row_c2r_kernel<A, C, L, W>, false));
        if constexpr (sizeof(typename A::S) == 4) {
            HPXFFT_ROW_FIXED_F32(HPXFFT_X)
        } else {
            HPXFFT_ROW_FIXED_FF(HPXFFT_X)
        }
#undef HPXFFT_X
    }
    return cudaSuccess;
}

template <class A>
bool RowLaunch<A>::has_fixed(int L, int log2W, int C)
{
    if constexpr (!A::kFixedChains) return false;
#define HPXFFT_X(L_, W_, C_) \
    if (L == L_ && log2W == W_ && C == C_) return true;
    if constexpr (sizeof(typename A::S) == 4) {
        HPXFFT_ROW_FIXED_F32(HPXFFT_X)
    } else {
        HPXFFT_ROW_FIXED_FF(HPXFFT_X)
    }
#undef HPXFFT_X
    return false;
}

template <class A>
cudaError_t RowLaunch<A>::r2c(const RowArgs &a, const LaunchShape &s, int FL, cudaStream_t st)
{
    if constexpr (A::kFixedChains) {
        if (FL) {
#define HPXFFT_X(L_, W_, C_)                                                                            \
    if (FL == L_ && a.log2W == W_ && s.cluster == C_)                                                   \
        return row_persistent<A>(C_, L_, W_) ? launch_persistent(row_r2c_kernel<A, C_, L_, W_>, a, s, st) \
                                             : launch_rows_ahead(row_r2c_kernel<A, C_, L_, W_>, a, s, C_, st);
            if constexpr (sizeof(typename A::S) == 4) {
                HPXFFT_ROW_FIXED_F32(HPXFFT_X)
            } else {
                HPXFFT_ROW_FIXED_FF(HPXFFT_X)
            }
#undef HPXFFT_X
            return cudaErrorInvalidValue;
        }
    }
    switch (s.cluster) {
    case 1: return launch_cluster(row_r2c_kernel<A, 1, 0, 0>, a, s, st);
    case 2: return launch_cluster(row_r2c_kernel<A, 2, 0, 0>, a, s, st);
    case 4: return launch_cluster(row_r2c_kernel<A, 4, 0, 0>, a, s, st);
    default: return cudaErrorInvalidValue;
    }
}

template <class A>
cudaError_t RowLaunch<A>::c2r(const RowArgs &a, const LaunchShape &s, int FL, cudaStream_t st)
{
    if constexpr (A::kFixedChains) {
        if (FL) {
#define HPXFFT_X(L_, W_, C_) \
    if (FL == L_ && a.log2W == W_ && s.cluster == C_) return launch_cluster(row_c2r_kernel<A, C_, L_, W_>, a, s, st);
            if constexpr (sizeof(typename A::S) == 4) {
                HPXFFT_ROW_FIXED_F32(HPXFFT_X)
            } else {
                HPXFFT_ROW_FIXED_FF(HPXFFT_X)
            }
#undef HPXFFT_X
            return cudaErrorInvalidValue;
        }
    }
    switch (s.cluster) {
    case 1: return launch_cluster(row_c2r_kernel<A, 1, 0, 0>, a, s, st);
    case 2: return launch_cluster(row_c2r_kernel<A, 2, 0, 0>, a, s, st);
    case 4: return launch_cluster(row_c2r_kernel<A, 4, 0, 0>, a, s, st);
    default: return cudaErrorInvalidValue;
    }
}
#endif

#ifdef HPXFFT_DEFINE_COLS
template <class A>
cudaError_t ColLaunch<A>::prepare()
{
#define HPXFFT_G(C, NP)                                           \
    HPXFFT_TRY(set_attrs(col_kernel<A, C, -1, 0, 0>, NP));        \
    HPXFFT_TRY(set_attrs(col_kernel<A, C, +1, 0, 0>, NP));
    HPXFFT_G(1, false) HPXFFT_G(2, false) HPXFFT_G(4, false) HPXFFT_G(8, false) HPXFFT_G(16, true)
#undef HPXFFT_G
    if constexpr (A::kFixedChains) {
#define HPXFFT_X(L, W, C)                                                 \
    HPXFFT_TRY(set_attrs(col_kernel<A, C, -1, L, W>, C > 8));             \
    HPXFFT_TRY(set_attrs(col_kernel<A, C, +1, L, W>, C > 8));
        if constexpr (sizeof(typename A::S) == 4) {
        HPXFFT_COL_FIXED_F32(HPXFFT_X)
    } else {
        HPXFFT_COL_FIXED_FF(HPXFFT_X)
    }
#undef HPXFFT_X
    }
    return cudaSuccess;
}

template <class A>
bool ColLaunch<A>::has_fixed(int L, int log2W, int C)
{
    if constexpr (!A::kFixedChains) return false;
#define HPXFFT_X(L_, W_, C_) \
    if (L == L_ && log2W == W_ && C == C_) return true;
    if constexpr (sizeof(typename A::S) == 4) {
        HPXFFT_COL_FIXED_F32(HPXFFT_X)
    } else {
        HPXFFT_COL_FIXED_FF(HPXFFT_X)
    }
#undef HPXFFT_X
    return false;
}

template <class A>
cudaError_t ColLaunch<A>::run(const ColArgs &a, int dir, const LaunchShape &s, int FL, cudaStream_t st)
{
    if constexpr (A::kFixedChains) {
        if (FL) {
#define HPXFFT_X(L_, W_, C_)                                                              \
    if (FL == L_ && a.log2W == W_ && s.cluster == C_)                                     \
        return dir < 0 ? launch_cluster(col_kernel<A, C_, -1, L_, W_>, a, s, st)          \
                       : launch_cluster(col_kernel<A, C_, +1, L_, W_>, a, s, st);
            if constexpr (sizeof(typename A::S) == 4) {
        HPXFFT_COL_FIXED_F32(HPXFFT_X)
    } else {
        HPXFFT_COL_FIXED_FF(HPXFFT_X)
    }
#undef HPXFFT_X
            return cudaErrorInvalidValue;
        }
    }
#define HPXFFT_G(C_)                                                                       \
    case C_:                                                                               \
        return dir < 0 ? launch_cluster(col_kernel<A, C_, -1, 0, 0>, a, s, st)            \
                       : launch_cluster(col_kernel<A, C_, +1, 0, 0>, a, s, st);
    switch (s.cluster) {
        HPXFFT_G(1) HPXFFT_G(2) HPXFFT_G(4) HPXFFT_G(8) HPXFFT_G(16)
    default: return cudaErrorInvalidValue;
    }
#undef HPXFFT_G
}
#endif

#ifdef HPXFFT_DEFINE_COLS
template <class A>
cudaError_t ColStepLaunch<A>::prepare()
{
    HPXFFT_TRY(set_attrs(colstep_kernel<A, -1, 0, 0>, false));
    HPXFFT_TRY(set_attrs(colstep_kernel<A, +1, 0, 0>, false));
    if constexpr (A::kFixedChains) {
#define HPXFFT_X(L, W)                                                 \
    HPXFFT_TRY(set_attrs(colstep_kernel<A, -1, L, W>, false));         \
    HPXFFT_TRY(set_attrs(colstep_kernel<A, +1, L, W>, false));         \
    if constexpr (sizeof(typename A::S) == 4) {                        \
        HPXFFT_TRY(set_attrs(colstep_direct_kernel<A, -1, L, W>, false));  \
        HPXFFT_TRY(set_attrs(colstep_direct_kernel<A, +1, L, W>, false));  \
    } else {                                                           \
        HPXFFT_TRY(set_attrs(colstep_warp_kernel<A, -1, L, W>, false));    \
        HPXFFT_TRY(set_attrs(colstep_warp_kernel<A, -1, L, W, true>, false));  \
    }
        if constexpr (sizeof(typename A::S) == 4) {
            HPXFFT_COLSTEP_FIXED_F32(HPXFFT_X)
        } else {
            HPXFFT_COLSTEP_FIXED_FF(HPXFFT_X)
        }
#undef HPXFFT_X
    }
    return cudaSuccess;
}

template <class A>
bool ColStepLaunch<A>::has_fixed(int L, int log2W)
{
    if constexpr (!A::kFixedChains) return false;
#define HPXFFT_X(L_, W_) \
    if (L == L_ && log2W == W_) return true;
    if constexpr (sizeof(typename A::S) == 4) {
        HPXFFT_COLSTEP_FIXED_F32(HPXFFT_X)
    } else {
        HPXFFT_COLSTEP_FIXED_FF(HPXFFT_X)
    }
#undef HPXFFT_X
    return false;
}

template <class A>
cudaError_t ColStepLaunch<A>::run(const ColStepArgs &a, int dir, const LaunchShape &s, int FL, cudaStream_t st)
{
    if constexpr (A::kFixedChains) {
        // FP32: register-fed first and last passes (16384^2 steps 0.58 / 0.53
        // -> 0.46 / 0.40 ms); float-float is arithmetic-bound and measured no
        // faster that way, so it keeps the staged kernel
        // per-row factors (Bluestein): the staged kernel, whose registers
        // hold them without spilling (the warp-local one takes output factors)
        const bool row_factors = a.pre_tab || a.post_tab;
        if constexpr (sizeof(typename A::S) == 4) {
            if (FL && !row_factors) {
#define HPXFFT_X(L_, W_)                                                                   \
    if (FL == L_ && a.log2W == W_)                                                         \
        return dir < 0 ? launch_cluster(colstep_direct_kernel<A, -1, L_, W_>, a, s, st)     \
                       : launch_cluster(colstep_direct_kernel<A, +1, L_, W_>, a, s, st);
                HPXFFT_COLSTEP_FIXED_F32(HPXFFT_X)
#undef HPXFFT_X
                return cudaErrorInvalidValue;
            }
        }
        if constexpr (sizeof(typename A::S) == 8) {
            // float-float forward steps with pair input: warp-local passes
            if (FL && a.pairs_in && a.warp_local && dir < 0 && !a.pre_tab) {
#define HPXFFT_X(L_, W_)                                                                              \
    if (FL == L_ && a.log2W == W_) {                                                                  \
        LaunchShape ws = s;                                                                           \
        ws.smem = (size_t)(1 << W_) * wl_col_stride(L_) * sizeof(cpx<typename A::T>);                 \
        return a.post_tab ? launch_cluster(colstep_warp_kernel<A, -1, L_, W_, true>, a, ws, st)       \
                          : launch_cluster(colstep_warp_kernel<A, -1, L_, W_>, a, ws, st);            \
    }
                HPXFFT_COLSTEP_FIXED_FF(HPXFFT_X)
#undef HPXFFT_X
            }
        }
        if (FL) {
#define HPXFFT_X(L_, W_)                                                              \
    if (FL == L_ && a.log2W == W_)                                                    \
        return dir < 0 ? launch_cluster(colstep_kernel<A, -1, L_, W_>, a, s, st)      \
                       : launch_cluster(colstep_kernel<A, +1, L_, W_>, a, s, st);
            if constexpr (sizeof(typename A::S) == 4) {
                HPXFFT_COLSTEP_FIXED_F32(HPXFFT_X)
            } else {
                HPXFFT_COLSTEP_FIXED_FF(HPXFFT_X)
            }
#undef HPXFFT_X
            return cudaErrorInvalidValue;
        }
    }
    return dir < 0 ? launch_cluster(colstep_kernel<A, -1, 0, 0>, a, s, st)
                   : launch_cluster(colstep_kernel<A, +1, 0, 0>, a, s, st);
}
#endif

#ifdef HPXFFT_DEFINE_TWIDDLES
template <class A>
cudaError_t TwiddleLaunch<A>::full(void *tab, int n, cudaStream_t st)
{
    using T = typename A::T;
    const int threads = 256;
    twiddle_kernel<T><<<(n + threads - 1) / threads, threads, 0, st>>>(reinterpret_cast<cpx<T> *>(tab), n);
    return cudaGetLastError();
}

template <class A>
cudaError_t TwiddleLaunch<A>::pass(void *tab, int Ls, int R, cudaStream_t st)
{
    using T = typename A::T;
    const int n = Ls * (R - 1), threads = 256;
    if (n <= 0) return cudaSuccess;
    pass_twiddle_kernel<T><<<(n + threads - 1) / threads, threads, 0, st>>>(reinterpret_cast<cpx<T> *>(tab), Ls, R);
    return cudaGetLastError();
}
#endif

}  // namespace hpxfft_gpu
