// Device side of the 2D real-to-complex transform.
//
// The reference (core/src/shared/loop.cpp:56-113) runs four phases over host
// memory: row r2c (FFTW), transpose, column c2c (FFTW), transpose back.  Here
// the two transposes disappear: the column kernels work on strips of W
// adjacent ky columns directly in the [kx][ky] layout, so the whole 2D
// transform is two HBM passes (row pass: read S, write S; column pass: read S,
// write S) over the caller's padded in-place buffer, or three when long
// columns take the two-kernel four-step split through a scratch array.
//
// One 1D transform of length N is held in shared memory.  When it does not
// fit one CTA it is split over a thread-block cluster of C CTAs: CTA c owns
// the inputs n = c + C*m, runs a length-N/C Stockham FFT on them, multiplies
// by W_N^(c*k2), and the length-C DFTs across the cluster read the peers'
// shared memory (DSMEM).  The result index is k = k2 + (N/C)*k1.
#pragma once
#include <cooperative_groups.h>

#include "cplx.cuh"

namespace hpxfft_gpu {
namespace cg = cooperative_groups;

constexpr int kMaxPasses = 24;
// Radix sequence of one local Stockham transform (radices 2,3,4,5,7,8,11,13,16).
struct PassPlan {
    int n;
    int radix[kMaxPasses];
};

// Radix sequence of a runtime-planned local length L: radix-16 passes, then
// the power-of-two remainder, then the odd primes 3, 5, 7, 11, 13.  False
// when L has a prime factor above 13 or needs more than kMaxPasses passes.
// Uses no heap (the allocation-free entry point plans with it too).
inline bool factorize_radices(int L, PassPlan &pp)
{
    pp.n = 0;
    if (L < 1) return false;
    int odd[kMaxPasses], nodd = 0, rest = L;
    for (int q : {3, 5, 7, 11, 13})
        while (rest % q == 0) {
            if (nodd == kMaxPasses) return false;
            rest /= q;
            odd[nodd++] = q;
        }
    if (rest & (rest - 1)) return false;  // a prime factor above 13
    int p2 = 0;
    while ((1 << p2) < rest) ++p2;
    if (p2 / 4 + (p2 % 4 ? 1 : 0) + nodd > kMaxPasses) return false;
    for (; p2 >= 4; p2 -= 4) pp.radix[pp.n++] = 16;
    if (p2 > 0) pp.radix[pp.n++] = 1 << p2;
    for (int i = 0; i < nodd; ++i) pp.radix[pp.n++] = odd[i];
    return true;
}

// Compute-type traits: T = arithmetic type, S = storage (HBM) real type.
// kFixedChains: compile-time pass chains are instantiated for this type.
// kEPTFixed: elements per thread of the compile-time chains (also their
// largest radix); they run 1024-thread CTAs.  Runtime-plan kernels keep 16
// elements per thread and kMaxThreads threads.
// Compile-time chains run at most 512 threads with a 64-register budget, so
// two CTAs (and their <= 64 KB of data) share an SM: one streams its strip
// in or out while the other computes.
constexpr int kFixedThreadsMax = 512;
constexpr int kFixedMinBlocks = 2;

struct ArithF32 {
    using T = float;
    using S = float;
    static constexpr bool kScaled = false;
    static constexpr bool kFixedChains = true;
    static constexpr int kMaxThreads = 1024;
    static constexpr int kEPTFixed = 16;
    static constexpr int kMinBlocks = kFixedMinBlocks;  // CTAs per SM the compile-time chains keep
    static constexpr int kDecim = 1;  // sub-rows per row (ArithFF16D)
};
struct ArithF64 {
    using T = double;
    using S = double;
    static constexpr bool kScaled = false;
    static constexpr bool kFixedChains = false;
    static constexpr int kMaxThreads = 512;
    static constexpr int kEPTFixed = 8;
    static constexpr int kMinBlocks = kFixedMinBlocks;
    static constexpr int kDecim = 1;  // sub-rows per row (ArithFF16D)
};
struct ArithFF {
    using T = ff;
    using S = double;
    static constexpr bool kScaled = true;  // per-transform power-of-two scale
    static constexpr bool kFixedChains = true;
    static constexpr int kMaxThreads = 512;
    static constexpr int kEPTFixed = 8;  // 32 data registers within the 64-register budget
    static constexpr int kMinBlocks = kFixedMinBlocks;
    static constexpr int kDecim = 1;  // sub-rows per row (ArithFF16D)
};
// Float-float rows of 8192 pairs with radix-16 passes (16 x 16 x 16 x 2):
// 512 threads at up to 128 registers; the row's 139 KB of shared memory
// keeps one CTA per SM either way.
struct ArithFF16 : ArithFF {
    static constexpr int kEPTFixed = 16;
    static constexpr int kMinBlocks = 1;
};
// The halves of float-float rows of 16384 pairs, transformed as rows of
// their own: virtual row v is sub-row c = v % 2 of row v / 2 (its pairs
// z[2m + c]); its DFT, without the packed-real split, is stored as raw
// pairs (one exponent per virtual row) for the combining kernel.
struct ArithFF16D : ArithFF16 {
    static constexpr int kDecim = 2;
};

// Elements held per thread in every pass (16 complex values).
constexpr int kElemsPerThread = 16;

// ----------------------------------------------------------------- storage
// Data loads bypass L1 (.cg), stores stream (.cs): each element is read and
// written once per pass, L1 stays with the twiddles, and a kernel that reads
// data another SM wrote in the same launch (the batched work queue) sees it
// at L2.  (Default-policy stores measured slower on 16384^2 FP32 and no
// faster on the batch.)
__device__ __forceinline__ double2 ld_stream(const double *p) { return __ldcg(reinterpret_cast<const double2 *>(p)); }
__device__ __forceinline__ float2 ld_stream(const float *p) { return __ldcg(reinterpret_cast<const float2 *>(p)); }

template <class A>
__device__ __forceinline__ cpx<typename A::T> load_c(const typename A::S *p, int E)
{
    using S = typename A::S;
    if constexpr (A::kScaled) {
        const double2 v = ld_stream(p);
        return cpx<ff>{ff_from_double(v.x, E), ff_from_double(v.y, E)};
    } else if constexpr (sizeof(S) == 8) {
        const double2 v = ld_stream(p);
        return cpx<double>{v.x, v.y};
    } else {
        const float2 v = ld_stream(p);
        return cpx<float>{v.x, v.y};
    }
}

template <class A>
__device__ __forceinline__ void store_c(typename A::S *p, cpx<typename A::T> v, int E)
{
    if constexpr (A::kScaled) {
        double2 o;
        o.x = ff_to_double(renorm(v.re), E);
        o.y = ff_to_double(renorm(v.im), E);
        __stcs(reinterpret_cast<double2 *>(p), o);
    } else if constexpr (sizeof(typename A::S) == 8) {
        __stcs(reinterpret_cast<double2 *>(p), make_double2(v.re, v.im));
    } else {
        __stcs(reinterpret_cast<float2 *>(p), make_float2(v.re, v.im));
    }
}

__device__ __forceinline__ int scale_exp(int emax) { return (emax == 0 || emax == 0x7ff) ? 0 : emax - 1023; }

// Float-float intermediates between kernels of one transform travel as raw
// renormalised (hi, lo) pairs (16 bytes per complex, like a double2) in units
// of 2^E, with E stored per producing block; no double conversion on either
// side.  Blocks whose inputs are all zero carry kExpNone, which never wins a
// maximum.
constexpr int kExpNone = -(1 << 20);
__device__ __forceinline__ int block_exp(int emax) { return emax == 0 ? kExpNone : scale_exp(emax); }

template <class A>
__device__ __forceinline__ void store_pair(typename A::S *p, cpx<typename A::T> v)
{
    if constexpr (A::kScaled) {
        const ff re = renorm(v.re), im = renorm(v.im);
        __stcs(reinterpret_cast<float4 *>(p), make_float4(re.hi, re.lo, im.hi, im.lo));
    }
}

// 2^d as a float for d <= 0, flushed below the normal range
__device__ __forceinline__ float pow2_le0(int d) { return d >= -126 ? __int_as_float((127 + d) << 23) : 0.0f; }

// twiddle W_Ltab^e (table holds the forward sign); DIR > 0 conjugates
template <int DIR, class T>
__device__ __forceinline__ cpx<T> twid(const cpx<T> *__restrict__ tw, int e)
{
    cpx<T> w = tw[e];
    if constexpr (DIR > 0) w.im = -w.im;
    return w;
}

// Shared-memory slot of logical element i: one pad slot after every 16
// elements keeps the strided Stockham stores free of bank conflicts.
__device__ __forceinline__ int pidx(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_elems(int n) { return n + (n >> 4) + 1; }

// ----------------------------------------------------------- Stockham pass
// One radix-R pass of a self-sorting (Stockham, decimation in time) FFT on W
// interleaved transforms of length L held in shared memory as s[n*W + w].
// Ls = length of the sub-transforms already combined.  Every thread keeps its
// tasks in registers across the barrier, so the pass works in place.
template <class T, int R, int DIR>
__device__ __forceinline__ void fft_pass(cpx<T> *s, int L, int log2W, int Ls, const cpx<T> *__restrict__ tw,
                                         int Ltab)
{
    constexpr int TPT = (kElemsPerThread + R - 1) / R;
    const int LR = L / R;
    const int ntask = LR << log2W;
    const int wmask = (1 << log2W) - 1;
    const int step = Ltab / (Ls * R);
    cpx<T> v[TPT][R];
#pragma unroll
    for (int t = 0; t < TPT; ++t) {
        const int task = threadIdx.x + t * blockDim.x;
        if (task < ntask) {
            const int w = task & wmask, jj = task >> log2W;
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = s[pidx(((jj + r * LR) << log2W) + w)];
            if (Ls > 1) {
                const int k = jj % Ls;
#pragma unroll
                for (int r = 1; r < R; ++r) v[t][r] = cmul(v[t][r], twid<DIR>(tw, r * k * step));
            }
            DFT<R, DIR, T>::run(v[t]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < TPT; ++t) {
        const int task = threadIdx.x + t * blockDim.x;
        if (task < ntask) {
            const int w = task & wmask, jj = task >> log2W;
            const int k = jj % Ls;
            const int base = (jj - k) * R + k;  // (jj / Ls) * Ls * R + k
#pragma unroll
            for (int r = 0; r < R; ++r) s[pidx(((base + r * Ls) << log2W) + w)] = cnorm(v[t][r]);
        }
    }
    __syncthreads();
}

template <class T, int DIR>
__device__ void local_fft(cpx<T> *s, int L, int log2W, const PassPlan &pp, const cpx<T> *__restrict__ tw, int Ltab)
{
    int Ls = 1;
    for (int p = 0; p < pp.n; ++p) {
        const int R = pp.radix[p];
        switch (R) {
        case 16: fft_pass<T, 16, DIR>(s, L, log2W, Ls, tw, Ltab); break;
        case 8: fft_pass<T, 8, DIR>(s, L, log2W, Ls, tw, Ltab); break;
        case 4: fft_pass<T, 4, DIR>(s, L, log2W, Ls, tw, Ltab); break;
        case 2: fft_pass<T, 2, DIR>(s, L, log2W, Ls, tw, Ltab); break;
        case 3: fft_pass<T, 3, DIR>(s, L, log2W, Ls, tw, Ltab); break;
        case 5: fft_pass<T, 5, DIR>(s, L, log2W, Ls, tw, Ltab); break;
        case 7: fft_pass<T, 7, DIR>(s, L, log2W, Ls, tw, Ltab); break;
        case 11: fft_pass<T, 11, DIR>(s, L, log2W, Ls, tw, Ltab); break;
        case 13: fft_pass<T, 13, DIR>(s, L, log2W, Ls, tw, Ltab); break;
        default: break;
        }
        Ls *= R;
    }
}


// ------------------------------------------------ compile-time pass chains
// Power-of-two local lengths get a fixed radix chain (16, ..., 16, then the
// remainder 2/4/8) with all index arithmetic folded at compile time, so the
// register allocator sees straight-line code.  Twiddles come from per-pass
// tables laid out [r-1][k] (one coalesced load per r across a warp):
//   ptab_p[(r-1)*Ls + k] = W_{Ls*R}^{r*k},  r in [1,R), k in [0,Ls).
__host__ __device__ constexpr int ilog2c(int v)
{
    int r = 0;
    while ((1 << (r + 1)) <= v) ++r;
    return r;
}

// Float-float chains (radix 8 first) renormalise their pairs after every
// second pass only (Ls = 8, 512, ...): the error-free sums and products stay
// exact on unnormalised pairs, whose low word grows by a few units in the
// high word's last place in between; every store to global memory
// renormalises.  Other types: no-op.
template <class T, int Ls>
__host__ __device__ constexpr bool renorm_after_pass()
{
    return !std::is_same<T, ff>::value || (ilog2c(Ls) / 3) % 2 == 1;
}

template <class T, int R, int L, int W, int NT, int DIR, int Ls, bool RAW, bool POST>
__device__ __forceinline__ void fixed_pass(cpx<T> *s, const cpx<T> *__restrict__ tp, const int *sEc,
                                           const cpx<T> *__restrict__ post_tw, int post_mult)
{
    constexpr int LR = L / R;
    constexpr int NTASK = LR * W;
    constexpr int TPT = (NTASK + NT - 1) / NT;
    cpx<T> v[TPT][R];
    const bool active = threadIdx.x < NT;  // bodies may run in a larger CTA (batch kernel)
#pragma unroll
    for (int t = 0; t < TPT; ++t) {
        const int task = threadIdx.x + t * NT;
        if (active && (NTASK % NT == 0 || task < NTASK)) {
            const int w = task % W, jj = task / W;
            if (RAW && sEc) {
                // first pass of the float-float path: the slots still hold the
                // raw doubles; convert with the transform's scale exponent
                const int E = scale_exp(sEc[w]);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const double2 d = reinterpret_cast<const double2 *>(s)[pidx((jj + r * LR) * W + w)];
                    if constexpr (RAW) v[t][r] = cpx<T>{ff_from_double(d.x, E), ff_from_double(d.y, E)};
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) v[t][r] = s[pidx((jj + r * LR) * W + w)];
            }
            if constexpr (Ls > 1) {
                const int k = jj % Ls;
#pragma unroll
                for (int r = 1; r < R; ++r) v[t][r] = cmul(v[t][r], twid<DIR>(tp, (r - 1) * Ls + k));
            }
            DFT<R, DIR, T>::run(v[t]);
            if constexpr (POST) {
                // last pass of a cluster-split transform: W_N^(c k2) for output k2
                if (post_mult) {
                    const int k = jj % Ls;
                    const int base = (jj - k) * R + k;
#pragma unroll
                    for (int r = 0; r < R; ++r) v[t][r] = cmul(v[t][r], twid<DIR>(post_tw, post_mult * (base + r * Ls)));
                }
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < TPT; ++t) {
        const int task = threadIdx.x + t * NT;
        if (active && (NTASK % NT == 0 || task < NTASK)) {
            const int w = task % W, jj = task / W;
            const int k = jj % Ls;
            const int base = (jj - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if constexpr (renorm_after_pass<T, Ls>())
                    s[pidx((base + r * Ls) * W + w)] = cnorm(v[t][r]);
                else
                    s[pidx((base + r * Ls) * W + w)] = v[t][r];
            }
        }
    }
    __syncthreads();
}

// Radix of the pass after Ls: the largest power of two <= maxR dividing the
// rest, then the odd primes 3, 5, 7, 11, 13.
__host__ __device__ constexpr int fixed_radix(int L, int Ls, int maxR)
{
    const int rest = L / Ls;
    if (rest % 2 == 0) {
        int r = 2;
        while (r * 2 <= maxR && rest % (r * 2) == 0) r *= 2;
        return r;
    }
    if (rest % 3 == 0) return 3;
    if (rest % 5 == 0) return 5;
    if (rest % 7 == 0) return 7;
    if (rest % 11 == 0) return 11;
    if (rest % 13 == 0) return 13;
    return rest;
}

template <class T, int L, int W, int NT, int DIR, int MAXR, int Ls, int Off, bool RAW, bool POST>
struct FixedPasses {
    static __device__ __forceinline__ void run(cpx<T> *s, const cpx<T> *__restrict__ ptab, const int *sEc,
                                               const cpx<T> *__restrict__ post_tw, int post_mult)
    {
        if constexpr (Ls < L) {
            constexpr int R = fixed_radix(L, Ls, MAXR);
            constexpr bool last = Ls * R == L;
            fixed_pass<T, R, L, W, NT, DIR, Ls, RAW && Ls == 1, POST && last>(s, ptab + Off, sEc, post_tw, post_mult);
            FixedPasses<T, L, W, NT, DIR, MAXR, Ls * R, Off + (Ls > 1 ? Ls * (R - 1) : 0), RAW, POST>::run(
                s, ptab, sEc, post_tw, post_mult);
        }
    }
};

// Ls of the last pass of the compile-time chain for length L, and the
// per-pass table offset of the pass at Ls (the layout FixedPasses uses).
__host__ __device__ constexpr int last_pass_ls(int L, int maxR)
{
    int Ls = 1;
    while (Ls * fixed_radix(L, Ls, maxR) < L) Ls *= fixed_radix(L, Ls, maxR);
    return Ls;
}
__host__ __device__ constexpr int pass_table_offset(int L, int maxR, int upto)
{
    int Ls = 1, off = 0;
    while (Ls < upto) {
        const int R = fixed_radix(L, Ls, maxR);
        if (Ls > 1) off += Ls * (R - 1);
        Ls *= R;
    }
    return off;
}

// The compile-time chain's passes with Ls in [Ls, END), through shared memory.
template <class T, int L, int W, int NT, int DIR, int MAXR, int Ls, int Off, int END>
struct FixedPassRange {
    static __device__ __forceinline__ void run(cpx<T> *s, const cpx<T> *__restrict__ ptab)
    {
        if constexpr (Ls < END) {
            constexpr int R = fixed_radix(L, Ls, MAXR);
            fixed_pass<T, R, L, W, NT, DIR, Ls, false, false>(s, ptab + Off, nullptr, nullptr, 0);
            FixedPassRange<T, L, W, NT, DIR, MAXR, Ls * R, Off + Ls * (R - 1), END>::run(s, ptab);
        }
    }
};

// threads of a fixed-length CTA: EPT elements each, a multiple of 32
__host__ __device__ constexpr int fixed_threads(int L, int log2W, int EPT)
{
    return ((L << log2W) / EPT + 31) / 32 * 32 < 32 ? 32 : ((L << log2W) / EPT + 31) / 32 * 32;
}

// Loads of a thread are issued back to back before any is consumed, so a CTA
// keeps BATCH loads per thread in flight instead of waiting one DRAM latency
// per element.  ld(t) loads element t, use(t, v) consumes it.
template <int BATCH, class V, class LD, class USE>
__device__ __forceinline__ void batched_loop(int nel, int nth, LD ld, USE use)
{
    for (int base = (int)threadIdx.x < nth ? (int)threadIdx.x : nel; base < nel; base += BATCH * nth) {
        V v[BATCH];
#pragma unroll
        for (int i = 0; i < BATCH; ++i) {
            const int t = base + i * nth;
            if (t < nel) v[i] = ld(t);
        }
#pragma unroll
        for (int i = 0; i < BATCH; ++i) {
            const int t = base + i * nth;
            if (t < nel) use(t, v[i]);
        }
    }
}

// Largest input exponent per interleaved transform w, reduced over the CTA and
// (C > 1) over the cluster.  Every thread's elements share w = tid & (W-1).
template <int C>
__device__ __forceinline__ void reduce_exponents(int emax, int log2W, int *sE, int *sEc)
{
    const int W = 1 << log2W;
    for (int off = 16; off >= W; off >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, off));
    if ((threadIdx.x & 31) < W) atomicMax(&sE[threadIdx.x & (W - 1)], emax);
    if constexpr (C > 1) {
        cg::cluster_group cl = cg::this_cluster();
        cl.sync();
        if (threadIdx.x < (unsigned)W) {
            int e = 0;
            for (int r = 0; r < C; ++r) e = max(e, *cl.map_shared_rank(&sE[threadIdx.x], r));
            sEc[threadIdx.x] = e;
        }
    } else {
        __syncthreads();
        if (threadIdx.x < (unsigned)W) sEc[threadIdx.x] = sE[threadIdx.x];
    }
    __syncthreads();
}

// ---------------------------------------------------------------- arguments
struct RowArgs {
    const void *in;           // real rows (r2c) or complex rows (c2r)
    void *out;                // complex rows (r2c) or real rows (c2r)
    long long in_stride;      // reals per input row
    long long out_stride;     // reals per output row
    long long in_bstride;     // reals between batch items
    long long out_bstride;
    int nrows;
    int M;                    // ny / 2
    int log2W;                // rows per CTA = 1 << log2W (only with C == 1)
    int adjoint;              // c2r: half weights on the interior bins
    PassPlan pp;              // local transform of length M / C
    const void *tw;           // W_{2M}^e, e in [0, 2M)
    int Ltab;                 // 2M
    const void *ptab;         // per-pass twiddles of the compile-time chain
    int pairs_out;            // float-float r2c: store (hi, lo) pairs and one exponent per row
    int *exp_out;             // [batch][nrows] when pairs_out
    int prefetch;             // persistent r2c: prefetch the next row group into L2 (device input only)
    // non-persistent r2c with one row group per CTA: prefetch into L2 the
    // input of group blockIdx.x + prefetch_ahead (the CTA that takes this
    // CTA's place once it is done: prefetch_ahead = CTAs resident at once); 0: none
    int prefetch_ahead;
    // exponent slot of row r of batch item b (pairs_out): exp_out[b * exp_bstride + r]
    long long exp_bstride;
};

struct ColArgs {
    void *data;               // complex [nx][ncols] rows, in place
    long long row_stride;     // reals per row (2 * ncols for the padded layout)
    long long bstride;
    int nx;
    int ncols;
    int log2W;                // columns per strip
    PassPlan pp;              // local transform of length nx / C
    const void *tw;           // W_nx^e, e in [0, nx)
    int Ltab;                 // nx
    const void *ptab;         // per-pass twiddles of the compile-time chain
};

// The local transform of one CTA: the compile-time chain when FL > 0 (with
// the float-float conversion fused into its first pass when RAW, and the
// cluster twiddle W_N^(c k2) fused into its last pass when C > 1), else the
// runtime radix plan followed by a separate cluster-twiddle sweep.
// post_mult * k2 indexes the full table for W_N^(c k2).
template <class A, int DIR, int C, int FL, int FW, bool RAW>
__device__ __forceinline__ void local_stage(cpx<typename A::T> *s, int L, int log2W, const PassPlan &pp,
                                            const cpx<typename A::T> *__restrict__ tw, int Ltab,
                                            const cpx<typename A::T> *__restrict__ ptab, const int *sEc, int post_mult)
{
    using T = typename A::T;
    if constexpr (FL > 0) {
        constexpr int EPT = A::kEPTFixed;
        FixedPasses<T, FL, (1 << FW), fixed_threads(FL, FW, EPT), DIR, EPT, 1, 0, RAW, (C > 1)>::run(s, ptab, sEc, tw,
                                                                                                      post_mult);
    } else {
        local_fft<T, DIR>(s, L, log2W, pp, tw, Ltab);
        if constexpr (C > 1) {
            if (post_mult) {
                const int nel = L << log2W;
                for (int t = threadIdx.x; t < nel; t += blockDim.x)
                    s[pidx(t)] = cnorm(cmul(s[pidx(t)], twid<DIR>(tw, post_mult * (t >> log2W))));
            }
            __syncthreads();
        }
    }
}

// Kernel shape parameters: C = CTAs per cluster, FL = compile-time local
// length (0: runtime plan), FW = log2 of the interleave when FL > 0.
#define HPXFFT_SHAPE                                                                      \
    constexpr bool kFixed = FL > 0;                                                       \
    constexpr int EPT = kFixed ? A::kEPTFixed : kElemsPerThread;                          \
    const int log2W = kFixed ? FW : a.log2W;                                              \
    const int W = 1 << log2W, wmask = W - 1;                                              \
    const int tid = threadIdx.x;                                                          \
    const int nth = kFixed ? fixed_threads(FL, FW, EPT) : (int)blockDim.x;                \
    const int t0 = tid < nth ? tid : (1 << 30); /* threads past nth idle */               \
    unsigned crank = 0;                                                                   \
    if constexpr (C > 1) crank = cg::this_cluster().block_rank();                         \
    (void)kFixed;                                                                         \
    (void)t0;

// Compile-time chains: the CTA's own thread count, two CTAs per SM when it
// has at most 512 threads; runtime plans: the type's maximum, one CTA.
#define HPXFFT_BOUNDS(A, FL)                                                                     \
    __launch_bounds__((FL) > 0 ? fixed_threads(FL, FW, A::kEPTFixed) : A::kMaxThreads,           \
                      (FL) > 0 && fixed_threads(FL, FW, A::kEPTFixed) <= kFixedThreadsMax ? A::kMinBlocks : 1)

// ------------------------------------------------------------ row r2c kernel
// Packed-real row transform: z[m] = x[2m] + i x[2m+1], Z = DFT_M(z), then
//   X[k] = E - i W_2M^k O,  X[M-k] = conj(E + i W_2M^k O),
//   E = (Z[k] + conj Z[M-k]) / 2,  O = (Z[k] - conj Z[M-k]) / 2.
// Replaces the FFTW row pass core/src/shared/loop.cpp:61-69 (fft_1d_r2c_inplace,
// loop.cpp:6-9); output row kx holds X[kx][0..M] in place of the padded input.
// Body of the row r2c for row group `group` of batch item `bidx`.
// Packed-real split of the W transforms Z (length M) in shared memory into
// X[0..M] of rows row0 + w:  X[k] = E - i W_2M^k O,  X[M-k] = conj(E + i W_2M^k O).
// Threads t0, t0 + nth, ... take the tasks (t0 past the end: idle).
template <class A>
__device__ __forceinline__ void row_r2c_split(const cpx<typename A::T> *s, const RowArgs &a, int row0, int log2W,
                                              const cpx<typename A::T> *__restrict__ tw, typename A::S *out, int bidx,
                                              const int *sEc, int t0, int nth)
{
    using T = typename A::T;
    using S = typename A::S;
    const int M = a.M, wmask = (1 << log2W) - 1;
    const int ntask = (M / 2 + 1) << log2W;
    for (int t = t0; t < ntask; t += nth) {
        const int w = t & wmask, k = t >> log2W, row = row0 + w;
        if (row >= a.nrows) continue;
        const int E = A::kScaled ? scale_exp(sEc[w]) : 0;
        const cpx<T> za = s[pidx((k << log2W) + w)];
        const cpx<T> zb = cconj(s[pidx((((M - k) % M) << log2W) + w)]);
        const cpx<T> e = chalf(za + zb), o = chalf(za - zb);
        const cpx<T> tk = cmul(tw[k], o);
        S *orow = out + row * a.out_stride;
        if (A::kScaled && a.pairs_out) {
            store_pair<A>(orow + 2 * (long long)k, e + mul_i<-1>(tk));
            if (M - k != k) store_pair<A>(orow + 2 * (long long)(M - k), cconj(e + mul_i<+1>(tk)));
            if (k == 0) a.exp_out[(long long)bidx * a.exp_bstride + row] = block_exp(sEc[w]);
            continue;
        }
        store_c<A>(orow + 2 * (long long)k, e + mul_i<-1>(tk), E);
        if (M - k != k) store_c<A>(orow + 2 * (long long)(M - k), cconj(e + mul_i<+1>(tk)), E);
    }
}

// Last pass of a compile-time row chain fused with the packed-real split.
// Task jj of the last pass (Ls = LSL, radix RL) yields Z[jj + r LSL]; task
// LSL - jj yields their split partners Z[M - k], so a thread that runs both
// holds every (k, M - k) pair in registers and writes X[k], X[M - k] itself.
// Pair tasks: jj in [0, LSL/2] per row (jj = 0 and jj = LSL/2 pair with
// themselves).
template <class A, int FL, int FW, int NT>
__device__ __forceinline__ void row_last_pass_split(const cpx<typename A::T> *s,
                                                    const cpx<typename A::T> *__restrict__ ptab, const RowArgs &a,
                                                    int row0, const cpx<typename A::T> *__restrict__ tw,
                                                    typename A::S *out, int bidx, const int *sEc)
{
    using T = typename A::T;
    using S = typename A::S;
    constexpr int EPT = A::kEPTFixed, W = 1 << FW;
    constexpr int LSL = last_pass_ls(FL, EPT), RL = fixed_radix(FL, LSL, EPT), LRL = FL / RL;
    constexpr int Off = pass_table_offset(FL, EPT, LSL);
    constexpr int NPAIR = (LSL / 2 + 1) * W, TPT = (NPAIR + NT - 1) / NT;
    constexpr int M = FL;
    const cpx<T> *tp = ptab + Off;
    const int tid = threadIdx.x;
    if (tid >= NT) return;
    auto last_task = [&](int jj, int w, cpx<T> (&v)[RL]) {
#pragma unroll
        for (int r = 0; r < RL; ++r) v[r] = s[pidx(((jj + r * LRL) << FW) + w)];
#pragma unroll
        for (int r = 1; r < RL; ++r) v[r] = cmul(v[r], twid<-1>(tp, (r - 1) * LSL + jj));
        DFT<RL, -1, T>::run(v);
    };
#pragma unroll
    for (int t = 0; t < TPT; ++t) {
        const int task = tid + t * NT;
        if (!(NPAIR % NT == 0 || task < NPAIR)) continue;
        const int w = task % W, jj = task / W, row = row0 + w;
        if (row >= a.nrows) continue;
        const int jj2 = (LSL - jj) % LSL;
        cpx<T> va[RL], vb[RL];
        last_task(jj, w, va);
        if (jj2 != jj) last_task(jj2, w, vb);
        const int E = A::kScaled ? scale_exp(sEc[w]) : 0;
        S *orow = out + (long long)row * a.out_stride;
        auto emit = [&](int k, cpx<T> zk, cpx<T> zp) {  // k <= M/2, zp = Z[M - k]
            const cpx<T> zb = cconj(zp);
            const cpx<T> e = chalf(zk + zb), o = chalf(zk - zb);
            const cpx<T> tk = cmul(tw[k], o);
            if (A::kScaled && a.pairs_out) {
                store_pair<A>(orow + 2 * (long long)k, e + mul_i<-1>(tk));
                if (M - k != k) store_pair<A>(orow + 2 * (long long)(M - k), cconj(e + mul_i<+1>(tk)));
                if (k == 0) a.exp_out[(long long)bidx * a.exp_bstride + row] = block_exp(sEc[w]);
            } else {
                store_c<A>(orow + 2 * (long long)k, e + mul_i<-1>(tk), E);
                if (M - k != k) store_c<A>(orow + 2 * (long long)(M - k), cconj(e + mul_i<+1>(tk)), E);
            }
        };
#pragma unroll
        for (int r = 0; r < RL; ++r) {
            const int k = jj + r * LSL;  // an output of task jj
            if (jj2 != jj) {
                // partner M - k = jj2 + (RL - 1 - r) LSL, an output of task jj2
                const int kp = M - k;
                if (k <= kp)
                    emit(k, va[r], vb[RL - 1 - r]);
                else
                    emit(kp, vb[RL - 1 - r], va[r]);
            } else if (jj == 0) {
                // k = r LSL pairs with (RL - r) LSL in the same task (r = 0: k = 0 with itself)
                const int rp = (RL - r) % RL;
                if (r <= rp) emit(k, va[r], va[rp]);
            } else {
                // jj = LSL / 2: k pairs with LSL/2 + (RL - 1 - r) LSL
                const int rp = RL - 1 - r;
                if (r <= rp) emit(k, va[r], va[rp]);
            }
        }
    }
}

template <class A, int C, int FL, int FW>
__device__ __forceinline__ void row_r2c_body(const RowArgs &a, int group, int bidx)
{
    using T = typename A::T;
    using S = typename A::S;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T> *s = reinterpret_cast<cpx<T> *>(smem_raw);
    __shared__ int sE[64], sEc[64];
    HPXFFT_SHAPE
    const int M = a.M;
    const int L = kFixed ? FL : M / C;
    const int nel = L << log2W;
    const int row0 = group * W;
    const S *in = reinterpret_cast<const S *>(a.in) + (long long)bidx * a.in_bstride;
    S *out = reinterpret_cast<S *>(a.out) + (long long)bidx * a.out_bstride;
    const cpx<T> *tw = reinterpret_cast<const cpx<T> *>(a.tw);
    const cpx<T> *ptab = reinterpret_cast<const cpx<T> *>(a.ptab);

    auto ld_row = [&](int t) {
        using V2 = typename std::conditional<sizeof(S) == 8, double2, float2>::type;
        const int w = t & wmask, m = t >> log2W, row = row0 + w;
        V2 v{};
        if (row < a.nrows) v = ld_stream(in + row * a.in_stride + 2 * (crank + (long long)C * m));
        return v;
    };
    if constexpr (kFixed && C == 1) {
        // first pass fed from global memory: task (jj, w) takes elements
        // jj + LR1 r of row w into registers (float-float: the row's largest
        // exponent is reduced from the raw doubles before they are converted)
        using V2 = typename std::conditional<sizeof(S) == 8, double2, float2>::type;
        constexpr int NT = fixed_threads(FL, FW, EPT);
        constexpr int R1 = fixed_radix(FL, 1, EPT), LR1 = FL / R1;
        constexpr int NTASK = LR1 << FW, TPT = (NTASK + NT - 1) / NT;
        static_assert(NT % (1 << FW) == 0, "a thread's tasks share one row");
        const bool active = tid < NT;  // bodies may run in a larger CTA (batch kernel)
        V2 raw[TPT][R1];
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
            const int task = tid + t * NT;
            const int w = task & wmask, jj = task >> log2W, row = row0 + w;
#pragma unroll
            for (int r = 0; r < R1; ++r) {
                raw[t][r] = V2{};
                if (active && (NTASK % NT == 0 || task < NTASK) && row < a.nrows) {
                    if constexpr (A::kDecim > 1)  // pair D m + c of row row / D
                        raw[t][r] = ld_stream(in + (long long)(row / A::kDecim) * a.in_stride +
                                              2 * ((long long)(jj + r * LR1) * A::kDecim + row % A::kDecim));
                    else
                        raw[t][r] = ld_stream(in + row * a.in_stride + 2 * (long long)(jj + r * LR1));
                }
            }
        }
        if constexpr (A::kScaled) {
            if (tid < 64) sE[tid] = 0;
            __syncthreads();
            int emax = 0;
#pragma unroll
            for (int t = 0; t < TPT; ++t)
#pragma unroll
                for (int r = 0; r < R1; ++r)
                    emax = max(emax, max(dbl_biased_exp(raw[t][r].x), dbl_biased_exp(raw[t][r].y)));
            reduce_exponents<1>(emax, log2W, sE, sEc);
        }
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
            const int task = tid + t * NT;
            if (active && (NTASK % NT == 0 || task < NTASK)) {
                const int w = task & wmask, jj = task >> log2W;
                cpx<T> v[R1];
                if constexpr (A::kScaled) {
                    const int E = scale_exp(sEc[w]);
#pragma unroll
                    for (int r = 0; r < R1; ++r)
                        v[r] = cpx<T>{ff_from_double(raw[t][r].x, E), ff_from_double(raw[t][r].y, E)};
                } else {
#pragma unroll
                    for (int r = 0; r < R1; ++r) v[r] = cpx<T>{(T)raw[t][r].x, (T)raw[t][r].y};
                }
                DFT<R1, -1, T>::run(v);
#pragma unroll
                for (int r = 0; r < R1; ++r) s[pidx(((jj * R1 + r) << log2W) + w)] = v[r];  // pass 0: no renorm
            }
        }
        __syncthreads();
        constexpr int LSL = last_pass_ls(FL, EPT), RL = fixed_radix(FL, LSL, EPT);
        // FP32: the last pass fused with the packed-real split (16384^2 row
        // 0.61 -> 0.53 ms); float-float measured slower that way (2.84 ->
        // 2.94 ms, the 8192-pair CTA runs out of registers)
        if constexpr (LSL > 1 && !A::kScaled && RL <= 8) {
            FixedPassRange<T, FL, (1 << FW), NT, -1, EPT, R1, 0, LSL>::run(s, ptab);
            row_last_pass_split<A, FL, FW, NT>(s, ptab, a, row0, tw, out, bidx, sEc);
            return;
        }
        FixedPassRange<T, FL, (1 << FW), NT, -1, EPT, R1, 0, FL>::run(s, ptab);
    } else if constexpr (A::kScaled) {
        if (tid < 64) sE[tid] = 0;
        __syncthreads();
        int emax = 0;
        batched_loop<EPT, double2>(nel, nth, ld_row, [&](int t, double2 v) {
            reinterpret_cast<double2 *>(s)[pidx(t)] = v;
            emax = max(emax, max(dbl_biased_exp(v.x), dbl_biased_exp(v.y)));
        });
        reduce_exponents<C>(emax, log2W, sE, sEc);
        if constexpr (!kFixed) {
            for (int t = t0; t < nel; t += nth) {
                const double2 v = reinterpret_cast<double2 *>(s)[pidx(t)];
                const int E = scale_exp(sEc[t & wmask]);
                s[pidx(t)] = cpx<ff>{ff_from_double(v.x, E), ff_from_double(v.y, E)};
            }
        }
    } else {
        using V2 = typename std::conditional<sizeof(S) == 8, double2, float2>::type;
        batched_loop<EPT, V2>(nel, nth, ld_row, [&](int t, V2 v) { s[pidx(t)] = cpx<T>{(T)v.x, (T)v.y}; });
    }
    if constexpr (!(kFixed && C == 1)) {
        __syncthreads();
        // W_M^(c k2) = W_2M^(2 c k2)
        local_stage<A, -1, C, FL, FW, A::kScaled>(s, L, log2W, a.pp, tw, a.Ltab, ptab, sEc, 2 * (int)crank);
    }

    if constexpr (A::kDecim > 1) {
        // the sub-row's DFT as raw pairs, its exponent beside it
        if (row0 < a.nrows) {
            S *orow = out + (long long)row0 * a.out_stride;
            for (int k = t0; k < L; k += nth) store_pair<A>(orow + 2 * (long long)k, s[pidx(k)]);
            if (tid == 0) a.exp_out[(long long)bidx * a.exp_bstride + row0] = block_exp(sEc[0]);
        }
    } else if constexpr (C == 1) {
        row_r2c_split<A>(s, a, row0, log2W, tw, out, bidx, sEc, t0, nth);
    } else {
        cg::cluster_group cl = cg::this_cluster();
        const int E = A::kScaled ? scale_exp(sEc[0]) : 0;
        cl.sync();
        const int Lc = L / C, k20 = crank * Lc;
        constexpr int TPT = (EPT + C - 1) / C;
        cpx<T> v[TPT][C];
#pragma unroll
        for (int u = 0; u < TPT; ++u) {
            const int t = tid + u * nth;
            if (t < Lc) {
#pragma unroll
                for (int r = 0; r < C; ++r) v[u][r] = *cl.map_shared_rank(&s[pidx(k20 + t)], r);
                DFT<C, -1, T>::run(v[u]);
            }
        }
        cl.sync();
#pragma unroll
        for (int u = 0; u < TPT; ++u) {
            const int t = tid + u * nth;
            if (t < Lc)
#pragma unroll
                for (int k1 = 0; k1 < C; ++k1) s[pidx(t + Lc * k1)] = cnorm(v[u][k1]);
        }
        cl.sync();
        // my Z[k], k = k20 + (li % Lc) + L * (li / Lc), sit at local index li
        for (int li = t0; li < L; li += nth) {
            const int k1 = li / Lc, k2 = k20 + li % Lc;
            const int k = k2 + L * k1;
            const int kp = (M - k) % M;
            const int k2p = kp % L, cp = k2p / Lc;
            const int lip = (k2p - cp * Lc) + Lc * (kp / L);
            const cpx<T> za = s[pidx(li)];
            const cpx<T> zb = cconj(*cl.map_shared_rank(&s[pidx(lip)], cp));
            const cpx<T> e = chalf(za + zb), o = chalf(za - zb);
            const cpx<T> tk = cmul(tw[k], o);
            S *orow = out + row0 * a.out_stride;
            if (row0 < a.nrows) {
                if (A::kScaled && a.pairs_out) {
                    store_pair<A>(orow + 2 * (long long)k, e + mul_i<-1>(tk));
                    if (k == 0) {
                        store_pair<A>(orow + 2 * (long long)M, cconj(e + mul_i<+1>(tk)));
                        a.exp_out[(long long)bidx * a.exp_bstride + row0] = block_exp(sEc[0]);
                    }
                } else {
                    store_c<A>(orow + 2 * (long long)k, e + mul_i<-1>(tk), E);
                    if (k == 0) store_c<A>(orow + 2 * (long long)M, cconj(e + mul_i<+1>(tk)), E);
                }
            }
        }
        cl.sync();
    }
}

// Bring [p, p + bytes) into L2 with bulk prefetches of whole 16-byte units
// (the ragged ends are left out), spread over the CTA's threads.
__device__ __forceinline__ void prefetch_l2(const void *p, long long bytes)
{
    const uintptr_t b = ((uintptr_t)p + 15) & ~(uintptr_t)15;
    const uintptr_t e = ((uintptr_t)p + (uintptr_t)bytes) & ~(uintptr_t)15;
    constexpr uintptr_t kChunk = 16384;
    for (uintptr_t c = b + threadIdx.x * kChunk; c < e; c += blockDim.x * kChunk) {
        const unsigned sz = (unsigned)(e - c < kChunk ? e - c : kChunk);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(c), "r"(sz) : "memory");
    }
}

// Rows whose CTA fills an SM (compile-time shapes above kFixedThreadsMax
// threads: one 8192-pair float-float row) run persistent: a CTA walks row
// groups blockIdx.x, blockIdx.x + gridDim.x, ... and prefetches the next
// group's input into L2 while it transforms the current one, so its load
// phase no longer leaves the SM idle.  Smaller shapes run two CTAs per SM,
// which overlap each other (and the loop would cost them registers).
template <class A>
__host__ __device__ constexpr bool row_persistent(int C, int FL, int FW)
{
    return C == 1 && FL > 0 && fixed_threads(FL, FW, A::kEPTFixed) > kFixedThreadsMax;
}

template <class A, int C, int FL, int FW>
__global__ void HPXFFT_BOUNDS(A, FL) row_r2c_kernel(RowArgs a)
{
    if constexpr (row_persistent<A>(C, FL, FW)) {
        using S = typename A::S;
        const int log2W = FL > 0 ? FW : a.log2W;
        const int ngroups = (a.nrows + (1 << log2W) - 1) >> log2W;
        for (int group = blockIdx.x; group < ngroups; group += gridDim.x) {
            const int next = group + gridDim.x;
            if (a.prefetch && next < ngroups) {
                const int r0 = next << log2W, nr = min(1 << log2W, a.nrows - r0);
                const S *src = reinterpret_cast<const S *>(a.in) + (long long)blockIdx.y * a.in_bstride +
                               (long long)r0 * a.in_stride;
                prefetch_l2(src, (long long)nr * a.in_stride * (long long)sizeof(S));
            }
            row_r2c_body<A, 1, FL, FW>(a, group, blockIdx.y);
            __syncthreads();  // shared memory is reused by the next group
        }
    } else {
        if constexpr (C == 1) {
            if (a.prefetch_ahead) {
                using S = typename A::S;
                const int log2W = FL > 0 ? FW : a.log2W;
                const int next = (int)blockIdx.x + a.prefetch_ahead;
                if (next < (int)gridDim.x) {
                    const int r0 = next << log2W, nr = min(1 << log2W, a.nrows - r0);
                    const S *src = reinterpret_cast<const S *>(a.in) + (long long)blockIdx.y * a.in_bstride +
                                   (long long)r0 * a.in_stride;
                    if (nr > 0) prefetch_l2(src, (long long)nr * a.in_stride * (long long)sizeof(S));
                }
            }
        }
        row_r2c_body<A, C, FL, FW>(a, blockIdx.x / C, blockIdx.y);
    }
}

// ------------------------------------------------------------ row c2r kernel
// Unnormalised c2r of a Hermitian half spectrum X[0..M] (imaginary parts of
// X[0], X[M] ignored):  Z[k] = (X[k] + conj X[M-k]) + i W_2M^-k (X[k] - conj X[M-k]),
// z = IDFT_M(Z) unnormalised, x[2m] = Re z[m], x[2m+1] = Im z[m].  With
// `adjoint` the interior bins are halved first, which turns the c2r into the
// adjoint of the r2c.  No reference counterpart (the FFTW backward direction
// is declared in core/include/hpxfft/util/adapter_fftw.hpp:11 but unused).
template <class A, int C, int FL, int FW>
__global__ void HPXFFT_BOUNDS(A, FL) row_c2r_kernel(RowArgs a)
{
    using T = typename A::T;
    using S = typename A::S;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T> *s = reinterpret_cast<cpx<T> *>(smem_raw);
    __shared__ int sE[64], sEc[64];
    HPXFFT_SHAPE
    const int M = a.M;
    const int L = kFixed ? FL : M / C;
    const int nel = L << log2W;
    const int row0 = (blockIdx.x / C) * W;
    const S *in = reinterpret_cast<const S *>(a.in) + (long long)blockIdx.y * a.in_bstride;
    S *out = reinterpret_cast<S *>(a.out) + (long long)blockIdx.y * a.out_bstride;
    const cpx<T> *tw = reinterpret_cast<const cpx<T> *>(a.tw);
    const cpx<T> *ptab = reinterpret_cast<const cpx<T> *>(a.ptab);

    if constexpr (kFixed && C == 1 && !A::kScaled) {
        // FP32: Hermitian pre-processing and the first pass in registers from
        // global memory, the last pass straight to the real output rows
        constexpr int NT = fixed_threads(FL, FW, EPT);
        constexpr int R1 = fixed_radix(FL, 1, EPT), LR1 = FL / R1;
        constexpr int NTASK = LR1 << FW, TPT = (NTASK + NT - 1) / NT;
        const bool active = tid < NT;
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
            const int task = tid + t * NT;
            if (active && (NTASK % NT == 0 || task < NTASK)) {
                const int w = task & wmask, jj = task >> log2W, row = row0 + w;
                cpx<T> v[R1];
                constexpr int H = R1 > 8 ? 8 : R1;  // loads in flight per batch (register budget)
#pragma unroll
                for (int r0 = 0; r0 < R1; r0 += H) {
                    float2 xa[H], xb[H];
#pragma unroll
                    for (int h = 0; h < H; ++h) {
                        const int k = jj + (r0 + h) * LR1;
                        xa[h] = xb[h] = make_float2(0.f, 0.f);
                        if (row < a.nrows) {
                            xa[h] = ld_stream(in + row * a.in_stride + 2 * (long long)k);
                            xb[h] = ld_stream(in + row * a.in_stride + 2 * (long long)(M - k));
                        }
                    }
#pragma unroll
                    for (int h = 0; h < H; ++h) {
                        const int k = jj + (r0 + h) * LR1;
                        cpx<T> za{xa[h].x, xa[h].y}, zb{xb[h].x, xb[h].y};
                        if (k == 0) {
                            za.im = 0;
                            zb.im = 0;
                        } else if (a.adjoint) {
                            za = chalf(za);
                            zb = chalf(zb);
                        }
                        const cpx<T> zbc = cconj(zb);
                        v[r0 + h] = (za + zbc) + mul_i<+1>(cmul(twid<+1>(tw, k), za - zbc));
                    }
                }
                DFT<R1, +1, T>::run(v);
#pragma unroll
                for (int r = 0; r < R1; ++r) s[pidx(((jj * R1 + r) << log2W) + w)] = v[r];
            }
        }
        __syncthreads();
        constexpr int LSL = last_pass_ls(FL, EPT), RL = fixed_radix(FL, LSL, EPT), LRL = FL / RL;
        FixedPassRange<T, FL, (1 << FW), NT, +1, EPT, R1, 0, LSL>::run(s, ptab);
        constexpr int Off = pass_table_offset(FL, EPT, LSL);
        constexpr int NTL = LRL << FW, TPTL = (NTL + NT - 1) / NT;
#pragma unroll
        for (int t = 0; t < TPTL; ++t) {
            const int task = tid + t * NT;
            if (active && (NTL % NT == 0 || task < NTL)) {
                const int w = task & wmask, jj = task >> log2W, row = row0 + w;
                const int k = jj % LSL;
                cpx<T> v[RL];
#pragma unroll
                for (int r = 0; r < RL; ++r) v[r] = s[pidx(((jj + r * LRL) << log2W) + w)];
#pragma unroll
                for (int r = 1; r < RL; ++r) v[r] = cmul(v[r], twid<+1>(ptab + Off, (r - 1) * LSL + k));
                DFT<RL, +1, T>::run(v);
                if (row < a.nrows) {
                    const int base = (jj - k) * RL + k;
#pragma unroll
                    for (int r = 0; r < RL; ++r)
                        store_c<A>(out + row * a.out_stride + 2 * (long long)(base + r * LSL), v[r], 0);
                    if (task < (1 << log2W)) {  // jj == 0: the row's two pad reals
                        out[row * a.out_stride + 2 * (long long)M] = (S)0;
                        out[row * a.out_stride + 2 * (long long)M + 1] = (S)0;
                    }
                }
            }
        }
        return;
    }
    int emax = 0;
    if constexpr (A::kScaled) {
        if (tid < 64) sE[tid] = 0;
        __syncthreads();
        batched_loop<EPT / 2, double4>(
            nel, nth,
            [&](int t) {
                const int w = t & wmask, m = t >> log2W, row = row0 + w;
                const int k = crank + C * m;
                double2 v = make_double2(0.0, 0.0), u = make_double2(0.0, 0.0);
                if (row < a.nrows) {
                    v = ld_stream(in + row * a.in_stride + 2 * (long long)k);
                    u = ld_stream(in + row * a.in_stride + 2 * (long long)(M - k));
                }
                return make_double4(v.x, v.y, u.x, u.y);
            },
            [&](int t, double4 q) {
                reinterpret_cast<double2 *>(s)[pidx(t)] = make_double2(q.x, q.y);
                emax = max(emax, max(max(dbl_biased_exp(q.x), dbl_biased_exp(q.y)),
                                     max(dbl_biased_exp(q.z), dbl_biased_exp(q.w))));
            });
        reduce_exponents<C>(emax, log2W, sE, sEc);
    }
    for (int t = t0; t < nel; t += nth) {
        const int w = t & wmask, m = t >> log2W, row = row0 + w;
        const int k = crank + C * m;
        const int E = A::kScaled ? scale_exp(sEc[w]) : 0;
        cpx<T> xa = czero<T>(), xb = czero<T>();
        if (row < a.nrows) {
            if constexpr (A::kScaled) {
                const double2 v = reinterpret_cast<double2 *>(s)[pidx(t)];
                xa = cpx<ff>{ff_from_double(v.x, E), ff_from_double(v.y, E)};
            } else {
                xa = load_c<A>(in + row * a.in_stride + 2 * (long long)k, 0);
            }
            xb = load_c<A>(in + row * a.in_stride + 2 * (long long)(M - k), E);
        }
        if (k == 0) {
            xa.im = real_ops<T>::zero();
            xb.im = real_ops<T>::zero();
        } else if (a.adjoint) {
            xa = chalf(xa);
            xb = chalf(xb);
        }
        const cpx<T> xbc = cconj(xb);
        const cpx<T> sum = xa + xbc, dif = xa - xbc;
        s[pidx(t)] = cnorm(sum + mul_i<+1>(cmul(twid<+1>(tw, k), dif)));
    }
    __syncthreads();

    local_stage<A, +1, C, FL, FW, false>(s, L, log2W, a.pp, tw, a.Ltab, ptab, sEc, 2 * (int)crank);

    if constexpr (C == 1) {
        for (int t = t0; t < nel; t += nth) {
            const int w = t & wmask, m = t >> log2W, row = row0 + w;
            if (row >= a.nrows) continue;
            const int E = A::kScaled ? scale_exp(sEc[w]) : 0;
            store_c<A>(out + row * a.out_stride + 2 * (long long)m, s[pidx(t)], E);
            if (m == 0) {
                out[row * a.out_stride + 2 * (long long)M] = (S)0;
                out[row * a.out_stride + 2 * (long long)M + 1] = (S)0;
            }
        }
    } else {
        cg::cluster_group cl = cg::this_cluster();
        const int E = A::kScaled ? scale_exp(sEc[0]) : 0;
        cl.sync();
        const int Lc = L / C, k20 = crank * Lc;
        for (int t = t0; t < Lc; t += nth) {
            cpx<T> v[C];
#pragma unroll
            for (int r = 0; r < C; ++r) v[r] = *cl.map_shared_rank(&s[pidx(k20 + t)], r);
            DFT<C, +1, T>::run(v);
            if (row0 < a.nrows)
#pragma unroll
                for (int k1 = 0; k1 < C; ++k1)
                    store_c<A>(out + row0 * a.out_stride + 2 * (long long)(k20 + t + L * k1), v[k1], E);
        }
        if (crank == 0 && tid == 0 && row0 < a.nrows) {
            out[row0 * a.out_stride + 2 * (long long)M] = (S)0;
            out[row0 * a.out_stride + 2 * (long long)M + 1] = (S)0;
        }
        cl.sync();
    }
}

// ------------------------------------------------------------- column kernel
// In-place length-nx c2c on strips of W adjacent columns of the [kx][ky]
// array.  Replaces transpose -> FFTW c2c -> transpose back
// (core/src/shared/loop.cpp:72-102, fft_1d_c2c_inplace loop.cpp:11-15).
template <class A, int C, int DIR, int FL, int FW>
__device__ __forceinline__ void col_body(const ColArgs &a, int strip, int bidx)
{
    using T = typename A::T;
    using S = typename A::S;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T> *s = reinterpret_cast<cpx<T> *>(smem_raw);
    __shared__ int sE[64], sEc[64];
    HPXFFT_SHAPE
    const int L = kFixed ? FL : a.nx / C;
    const int nel = L << log2W;
    const int col0 = strip * W;
    S *data = reinterpret_cast<S *>(a.data) + (long long)bidx * a.bstride;
    const cpx<T> *tw = reinterpret_cast<const cpx<T> *>(a.tw);
    const cpx<T> *ptab = reinterpret_cast<const cpx<T> *>(a.ptab);

    if constexpr (kFixed && C == 1 && !A::kScaled) {
        // FP32: first pass from global memory into registers, last pass back
        // to it (in place is safe: every read of the strip precedes the CTA
        // barrier after the first pass, strips of other CTAs are disjoint)
        constexpr int NT = fixed_threads(FL, FW, EPT);
        constexpr int R1 = fixed_radix(FL, 1, EPT), LR1 = FL / R1;
        constexpr int NTASK = LR1 << FW, TPT = (NTASK + NT - 1) / NT;
        const bool active = tid < NT;
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
            const int task = tid + t * NT;
            if (active && (NTASK % NT == 0 || task < NTASK)) {
                const int w = task & wmask, jj = task >> log2W, col = col0 + w;
                float2 raw[R1];
#pragma unroll
                for (int r = 0; r < R1; ++r) {
                    raw[r] = make_float2(0.f, 0.f);
                    if (col < a.ncols) raw[r] = ld_stream(data + (long long)(jj + r * LR1) * a.row_stride + 2 * (long long)col);
                }
                cpx<T> v[R1];
#pragma unroll
                for (int r = 0; r < R1; ++r) v[r] = cpx<T>{raw[r].x, raw[r].y};
                DFT<R1, DIR, T>::run(v);
#pragma unroll
                for (int r = 0; r < R1; ++r) s[pidx(((jj * R1 + r) << log2W) + w)] = v[r];
            }
        }
        __syncthreads();
        constexpr int LSL = last_pass_ls(FL, EPT), RL = fixed_radix(FL, LSL, EPT), LRL = FL / RL;
        FixedPassRange<T, FL, (1 << FW), NT, DIR, EPT, R1, 0, LSL>::run(s, ptab);
        constexpr int Off = pass_table_offset(FL, EPT, LSL);
        constexpr int NTL = LRL << FW, TPTL = (NTL + NT - 1) / NT;
#pragma unroll
        for (int t = 0; t < TPTL; ++t) {
            const int task = tid + t * NT;
            if (active && (NTL % NT == 0 || task < NTL)) {
                const int w = task & wmask, jj = task >> log2W, col = col0 + w;
                const int k = jj % LSL;
                cpx<T> v[RL];
#pragma unroll
                for (int r = 0; r < RL; ++r) v[r] = s[pidx(((jj + r * LRL) << log2W) + w)];
#pragma unroll
                for (int r = 1; r < RL; ++r) v[r] = cmul(v[r], twid<DIR>(ptab + Off, (r - 1) * LSL + k));
                DFT<RL, DIR, T>::run(v);
                if (col < a.ncols) {
                    const int base = (jj - k) * RL + k;
#pragma unroll
                    for (int r = 0; r < RL; ++r)
                        store_c<A>(data + (long long)(base + r * LSL) * a.row_stride + 2 * (long long)col, v[r], 0);
                }
            }
        }
        return;
    }
    using V2 = typename std::conditional<sizeof(S) == 8, double2, float2>::type;
    auto ld_col = [&](int t) {
        const int w = t & wmask, m = t >> log2W, col = col0 + w;
        V2 v{};
        if (col < a.ncols) v = ld_stream(data + (crank + (long long)C * m) * a.row_stride + 2 * (long long)col);
        return v;
    };
    if constexpr (A::kScaled) {
        if (tid < 64) sE[tid] = 0;
        __syncthreads();
        int emax = 0;
        batched_loop<EPT, double2>(nel, nth, ld_col, [&](int t, double2 v) {
            reinterpret_cast<double2 *>(s)[pidx(t)] = v;
            emax = max(emax, max(dbl_biased_exp(v.x), dbl_biased_exp(v.y)));
        });
        reduce_exponents<C>(emax, log2W, sE, sEc);
        if constexpr (!kFixed) {
            for (int t = t0; t < nel; t += nth) {
                const double2 v = reinterpret_cast<double2 *>(s)[pidx(t)];
                const int E = scale_exp(sEc[t & wmask]);
                s[pidx(t)] = cpx<ff>{ff_from_double(v.x, E), ff_from_double(v.y, E)};
            }
        }
    } else {
        batched_loop<EPT, V2>(nel, nth, ld_col, [&](int t, V2 v) { s[pidx(t)] = cpx<T>{(T)v.x, (T)v.y}; });
    }
    __syncthreads();

    local_stage<A, DIR, C, FL, FW, A::kScaled>(s, L, log2W, a.pp, tw, a.Ltab, ptab, sEc, (int)crank);

    if constexpr (C == 1) {
        for (int t = t0; t < nel; t += nth) {
            const int w = t & wmask, k = t >> log2W, col = col0 + w;
            if (col >= a.ncols) continue;
            const int E = A::kScaled ? scale_exp(sEc[w]) : 0;
            store_c<A>(data + (long long)k * a.row_stride + 2 * (long long)col, s[pidx(t)], E);
        }
    } else {
        cg::cluster_group cl = cg::this_cluster();
        cl.sync();
        const int Lc = L / C, k20 = crank * Lc;
        const int ntask = Lc << log2W;
        for (int t = t0; t < ntask; t += nth) {
            const int w = t & wmask, k2 = k20 + (t >> log2W), col = col0 + w;
            cpx<T> v[C];
#pragma unroll
            for (int r = 0; r < C; ++r) v[r] = *cl.map_shared_rank(&s[pidx((k2 << log2W) + w)], r);
            DFT<C, DIR, T>::run(v);
            if (col < a.ncols) {
                const int E = A::kScaled ? scale_exp(sEc[w]) : 0;
#pragma unroll
                for (int k1 = 0; k1 < C; ++k1)
                    store_c<A>(data + (long long)(k2 + L * k1) * a.row_stride + 2 * (long long)col, v[k1], E);
            }
        }
        cl.sync();
    }
}

template <class A, int C, int DIR, int FL, int FW>
__global__ void HPXFFT_BOUNDS(A, FL) col_kernel(ColArgs a)
{
    col_body<A, C, DIR, FL, FW>(a, blockIdx.x / C, blockIdx.y);
}

// ------------------------------------------------------ column step kernel
// One step of a two-kernel four-step column FFT, nx = N1 * N2:
//   step A (group g = n1):  in rows g + N1*m  -> DFT_N2 over m, times W_nx^(g k)
//                           -> out rows g + N1*k
//   step B (group g = k2):  in rows N1*g + m  -> DFT_N1 over m
//                           -> out rows g + N2*k        (natural order)
// Each CTA owns a strip of W adjacent columns (W * 16 bytes per row segment)
// and never waits on another CTA.  A reads the data and writes a scratch
// array of the same layout, B reads the scratch and writes the data, so the
// column pass costs two HBM round trips instead of one but streams wide
// segments with full occupancy.
constexpr int kColStepMaxPairL = 256;  // longest step of the pair format (compiled shapes)

struct ColStepArgs {
    const void *in;
    void *out;
    long long row_stride;     // reals per row (both arrays)
    long long in_bstride, out_bstride;
    int ncols;
    int strips;               // column strips per group
    int in_step, out_step;    // row steps of m and k
    int in_gmul, out_gmul;    // row offset of group g: g * gmul
    int post;                 // multiply by W_nx^(g k) (step A)
    int L;                    // DFT length of this step
    int log2W;
    PassPlan pp;
    const void *tw;           // W_nx table (post twiddle) and runtime-plan twiddles
    int Ltab;                 // nx
    const void *ptab;
    // float-float pair format (compile-time chains only): input row r carries
    // exponent exp_in[(r % exp_rmod) * exp_rmul + (col0 >> exp_cshift)]
    // (per-row exponents of the row kernel, or per-block ones of step A);
    // pairs_out stores pairs and exp_out[blockIdx.x + gridDim.x * batch]
    // (from pair input or, in colstep_kernel, from double input)
    int pairs_in, pairs_out;
    const int *exp_in;
    int exp_rmod, exp_rmul, exp_cshift;
    long long exp_in_bstride;
    int *exp_out;
    // a launch over a subset of the groups (chunked host transfers): block b
    // of the launch is block block_offset + b of the full grid of
    // grid_blocks blocks (exponent slots are indexed by the full grid)
    int block_offset, grid_blocks;
    int warp_local;  // float-float with pair input: the warp-local kernel (colstep_warp_kernel)
    // per-row complex factors in the compute type (Bluestein's convolution):
    // input row r is multiplied by pre_tab[r] and rows r >= pre_rows read as
    // zero without a load; output row r is multiplied by post_tab[r] and
    // rows r >= post_rows are not written; both conjugated when tab_conj.
    // Null: none.  colstep_kernel applies both, colstep_warp_kernel the
    // output factors (the launcher routes input factors to colstep_kernel).
    const void *pre_tab, *post_tab;
    int pre_rows, post_rows;
    int tab_conj;
};

// tab[i], conjugated when conj
template <class T>
__device__ __forceinline__ cpx<T> row_factor(const cpx<T> *tab, long long i, int conj)
{
    const cpx<T> f = tab[i];
    return conj ? cconj(f) : f;
}

template <class A, int DIR, int FL, int FW>
__global__ void HPXFFT_BOUNDS(A, FL) colstep_kernel(ColStepArgs a)
{
    using T = typename A::T;
    using S = typename A::S;
    constexpr int C = 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T> *s = reinterpret_cast<cpx<T> *>(smem_raw);
    __shared__ int sE[64], sEc[64];
    HPXFFT_SHAPE
    const int L = kFixed ? FL : a.L;
    const int nel = L << log2W;
    const int bx = blockIdx.x + a.block_offset;
    const int g = bx / a.strips, col0 = (bx % a.strips) * W;
    const S *in = reinterpret_cast<const S *>(a.in) + (long long)blockIdx.y * a.in_bstride;
    S *out = reinterpret_cast<S *>(a.out) + (long long)blockIdx.y * a.out_bstride;
    const cpx<T> *tw = reinterpret_cast<const cpx<T> *>(a.tw);
    const cpx<T> *ptab = reinterpret_cast<const cpx<T> *>(a.ptab);
    const long long in_row0 = (long long)g * a.in_gmul, out_row0 = (long long)g * a.out_gmul;

    using V2 = typename std::conditional<sizeof(S) == 8, double2, float2>::type;
    const cpx<T> *pre = reinterpret_cast<const cpx<T> *>(a.pre_tab);
    const cpx<T> *post = reinterpret_cast<const cpx<T> *>(a.post_tab);
    auto ld = [&](int t) {
        const int w = t & wmask, m = t >> log2W, col = col0 + w;
        const long long row = in_row0 + (long long)a.in_step * m;
        V2 v{};
        if (col < a.ncols && (!pre || row < a.pre_rows)) v = ld_stream(in + row * a.row_stride + 2 * (long long)col);
        return v;
    };
    // element t of the tile times its input row's factor (rows past
    // pre_rows were loaded as zero)
    auto pre_mul = [&](int t, cpx<T> v) {
        const long long row = in_row0 + (long long)a.in_step * (t >> log2W);
        return row < a.pre_rows ? cmul(v, row_factor(pre, row, a.tab_conj)) : v;
    };
    int Eblk = kExpNone;  // pair format: the block's common exponent
    bool loaded = false;
    if constexpr (A::kScaled && kFixed) {
      if (a.pairs_in) {
        // exponents of the L input rows, their maximum, exact power-of-two
        // factors that bring every row to it
        __shared__ int sEm, sExp[kColStepMaxPairL];
        __shared__ float sFac[kColStepMaxPairL];
        if (tid == 0) sEm = kExpNone;
        __syncthreads();
        const int *ein = a.exp_in + (long long)blockIdx.y * a.exp_in_bstride;
        for (int m = tid; m < L; m += nth) {
            const int r = (int)(in_row0 + (long long)a.in_step * m);
            const int e = ein[(r % a.exp_rmod) * a.exp_rmul + (col0 >> a.exp_cshift)];
            sExp[m] = e;
            atomicMax(&sEm, e);
        }
        __syncthreads();
        Eblk = sEm;
        for (int m = tid; m < L; m += nth) sFac[m] = Eblk == kExpNone ? 1.0f : pow2_le0(sExp[m] - Eblk);
        __syncthreads();
        batched_loop<EPT, double2>(nel, nth, ld, [&](int t, double2 v) {
            const float4 q = *reinterpret_cast<const float4 *>(&v);
            const float f = sFac[t >> log2W];
            s[pidx(t)] = cpx<T>{ff{q.x * f, q.y * f}, ff{q.z * f, q.w * f}};
        });
        loaded = true;
      }
    }
    if (loaded) {
    } else if constexpr (A::kScaled) {
        if (tid < 64) sE[tid] = 0;
        __syncthreads();
        int emax = 0;
        batched_loop<EPT, double2>(nel, nth, ld, [&](int t, double2 v) {
            reinterpret_cast<double2 *>(s)[pidx(t)] = v;
            emax = max(emax, max(dbl_biased_exp(v.x), dbl_biased_exp(v.y)));
        });
        reduce_exponents<1>(emax, log2W, sE, sEc);
        // the runtime chain converts here; the compiled one in its first
        // pass, unless input factors need the pairs first
        if (!kFixed || pre) {
            for (int t = t0; t < nel; t += nth) {
                const double2 v = reinterpret_cast<double2 *>(s)[pidx(t)];
                const int E = scale_exp(sEc[t & wmask]);
                const cpx<ff> c{ff_from_double(v.x, E), ff_from_double(v.y, E)};
                s[pidx(t)] = pre ? pre_mul(t, c) : c;
            }
        }
    } else {
        batched_loop<EPT, V2>(nel, nth, ld, [&](int t, V2 v) { s[pidx(t)] = cpx<T>{(T)v.x, (T)v.y}; });
        if (pre) {  // a pass of its own: the batched loads keep their registers
            __syncthreads();
            for (int t = t0; t < nel; t += nth) s[pidx(t)] = pre_mul(t, s[pidx(t)]);
        }
    }
    __syncthreads();

    const bool pairs_in = A::kScaled && kFixed && a.pairs_in;
    if constexpr (kFixed)
        FixedPasses<T, FL, (1 << FW), fixed_threads(FL, FW, EPT), DIR, EPT, 1, 0, A::kScaled, false>::run(
            s, ptab, pairs_in || pre ? nullptr : sEc, tw, 0);
    else
        local_fft<T, DIR>(s, L, log2W, a.pp, tw, a.Ltab);

    // pairs out: pair input keeps its block exponent; double input (one
    // scale per column) takes the largest column exponent for the block and
    // rescales the other columns to it (exact powers of two)
    const bool pairs_out = A::kScaled && kFixed && a.pairs_out;
    __shared__ float sFo[64];  // per-column factors to the block exponent
    if constexpr (A::kScaled && kFixed) {
        if (pairs_out && !pairs_in) {
            __shared__ int sEo;
            if (tid == 0) {
                int m = kExpNone;
                for (int w = 0; w < (1 << log2W); ++w) m = max(m, block_exp(sEc[w]));
                sEo = m;
            }
            __syncthreads();
            Eblk = sEo;
            if (tid < (1 << log2W)) {
                const int ew = block_exp(sEc[tid]);
                sFo[tid] = ew == kExpNone || Eblk == kExpNone ? 0.0f : pow2_le0(ew - Eblk);
            }
            __syncthreads();
        }
    }
    if (pairs_out && tid == 0) a.exp_out[bx + (long long)a.grid_blocks * blockIdx.y] = Eblk;
    for (int t = t0; t < nel; t += nth) {
        const int w = t & wmask, k = t >> log2W, col = col0 + w;
        if (col >= a.ncols) continue;
        const int E = A::kScaled ? (pairs_in ? (Eblk == kExpNone ? 0 : Eblk) : scale_exp(sEc[w])) : 0;
        cpx<T> v = s[pidx(t)];
        if (a.post && g) v = cmul(v, twid<DIR>(tw, g * k));
        const long long orow = out_row0 + (long long)a.out_step * k;
        if (post) {
            if (orow >= a.post_rows) continue;
            v = cmul(v, row_factor(post, orow, a.tab_conj));
        }
        S *o = out + orow * a.row_stride + 2 * (long long)col;
        if (pairs_out) {
            if constexpr (A::kScaled) {
                if (!pairs_in) v = cpx<T>{ff_scale_pow2(v.re, sFo[w]), ff_scale_pow2(v.im, sFo[w])};
            }
            store_pair<A>(o, v);
        } else {
            store_c<A>(o, v, E);
        }
    }
}

// ---------------------------------------------- warp-local column steps
// The float-float column step with pair input, its passes warp-local: each
// column of the CTA's strip is owned by TPC = FL / 8 threads of one warp
// (32 / TPC columns per warp) and kept column-major in shared memory, so
// the Stockham passes exchange data with __syncwarp only.  The only
// CTA-wide barriers are after the coalesced load (row segments of the
// strip into the column-major tile) and before the coalesced store.  Same
// contract as colstep_kernel for pairs_in = 1 (both forward steps of the
// float-float pair exchange).
__host__ __device__ constexpr int wl_col_stride(int L) { return L + L / 16 + 1; }  // odd: load and store conflict-free

template <class T, int R, int L, int DIR, int Ls, int TPC>
__device__ __forceinline__ void warp_local_pass(cpx<T> *col, int t, const cpx<T> *__restrict__ tp)
{
    constexpr int LR = L / R, TPT = LR / TPC;
    static_assert(LR % TPC == 0, "tasks split evenly over the column's threads");
    cpx<T> v[TPT][R];
#pragma unroll
    for (int u = 0; u < TPT; ++u) {
        const int jj = t + u * TPC;
#pragma unroll
        for (int r = 0; r < R; ++r) v[u][r] = col[pidx(jj + r * LR)];
        if constexpr (Ls > 1) {
            const int k = jj % Ls;
#pragma unroll
            for (int r = 1; r < R; ++r) v[u][r] = cmul(v[u][r], twid<DIR>(tp, (r - 1) * Ls + k));
        }
        DFT<R, DIR, T>::run(v[u]);
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < TPT; ++u) {
        const int jj = t + u * TPC;
        const int k = jj % Ls;
        const int base = (jj - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if constexpr (renorm_after_pass<T, Ls>())
                col[pidx(base + r * Ls)] = cnorm(v[u][r]);
            else
                col[pidx(base + r * Ls)] = v[u][r];
        }
    }
    __syncwarp();
}

template <class T, int L, int DIR, int MAXR, int Ls, int Off, int TPC>
struct WarpLocalPasses {
    static __device__ __forceinline__ void run(cpx<T> *col, int t, const cpx<T> *__restrict__ ptab)
    {
        if constexpr (Ls < L) {
            constexpr int R = fixed_radix(L, Ls, MAXR);
            warp_local_pass<T, R, L, DIR, Ls, TPC>(col, t, ptab + Off);
            WarpLocalPasses<T, L, DIR, MAXR, Ls * R, Off + (Ls > 1 ? Ls * (R - 1) : 0), TPC>::run(col, t, ptab);
        }
    }
};

// RF: the instance that applies ColStepArgs' per-row output factors
template <class A, int DIR, int FL, int FW, bool RF = false>
__global__ void __launch_bounds__((FL << FW) / A::kEPTFixed, kFixedMinBlocks) colstep_warp_kernel(ColStepArgs a)
{
    using T = typename A::T;
    using S = typename A::S;
    constexpr int EPT = A::kEPTFixed, W = 1 << FW, NT = (FL << FW) / EPT, TPC = FL / EPT, CS = wl_col_stride(FL);
    static_assert(32 % TPC == 0 && NT % 32 == 0, "whole columns per warp");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T> *s = reinterpret_cast<cpx<T> *>(smem_raw);
    __shared__ int sEm, sExp[kColStepMaxPairL];
    __shared__ float sFac[kColStepMaxPairL];
    const int tid = threadIdx.x;
    const int bx = blockIdx.x + a.block_offset;
    const int g = bx / a.strips, col0 = (bx % a.strips) * W;
    const S *in = reinterpret_cast<const S *>(a.in) + (long long)blockIdx.y * a.in_bstride;
    S *out = reinterpret_cast<S *>(a.out) + (long long)blockIdx.y * a.out_bstride;
    const cpx<T> *tw = reinterpret_cast<const cpx<T> *>(a.tw);
    const cpx<T> *ptab = reinterpret_cast<const cpx<T> *>(a.ptab);
    const long long in_row0 = (long long)g * a.in_gmul, out_row0 = (long long)g * a.out_gmul;

    // exponents of the FL input rows, their maximum, exact power-of-two
    // factors that bring every row to it (as colstep_kernel)
    if (tid == 0) sEm = kExpNone;
    __syncthreads();
    const int *ein = a.exp_in + (long long)blockIdx.y * a.exp_in_bstride;
    for (int m = tid; m < FL; m += NT) {
        const int r = (int)(in_row0 + (long long)a.in_step * m);
        const int e = ein[(r % a.exp_rmod) * a.exp_rmul + (col0 >> a.exp_cshift)];
        sExp[m] = e;
        atomicMax(&sEm, e);
    }
    __syncthreads();
    const int Eblk = sEm;
    for (int m = tid; m < FL; m += NT) sFac[m] = Eblk == kExpNone ? 1.0f : pow2_le0(sExp[m] - Eblk);
    __syncthreads();

    // coalesced load: element (m, w) of the strip to column w, position m
    batched_loop<EPT, double2>(FL << FW, NT,
                               [&](int t) {
                                   const int w = t & (W - 1), m = t >> FW, col = col0 + w;
                                   double2 v{};
                                   if (col < a.ncols)
                                       v = ld_stream(in + (in_row0 + (long long)a.in_step * m) * a.row_stride +
                                                     2 * (long long)col);
                                   return v;
                               },
                               [&](int t, double2 v) {
                                   const int w = t & (W - 1), m = t >> FW;
                                   const float4 q = *reinterpret_cast<const float4 *>(&v);
                                   const float f = sFac[m];
                                   s[w * CS + pidx(m)] = cpx<T>{ff{q.x * f, q.y * f}, ff{q.z * f, q.w * f}};
                               });
    __syncthreads();

    // the column's passes, warp-local
    {
        const int c = tid / TPC, t = tid % TPC;
        WarpLocalPasses<T, FL, DIR, EPT, 1, 0, TPC>::run(s + c * CS, t, ptab);
    }
    __syncthreads();

    // coalesced store, times W_nx^(g k) when the step has a post twiddle
    const bool pairs_out = a.pairs_out != 0;
    if (pairs_out && tid == 0) a.exp_out[bx + (long long)a.grid_blocks * blockIdx.y] = Eblk;
    const int E = Eblk == kExpNone ? 0 : Eblk;
    for (int t = tid; t < (FL << FW); t += NT) {
        const int w = t & (W - 1), k = t >> FW, col = col0 + w;
        if (col >= a.ncols) continue;
        cpx<T> v = s[w * CS + pidx(k)];
        if (a.post && g) v = cmul(v, twid<DIR>(tw, g * k));
        if constexpr (RF) {  // per-row output factors (Bluestein)
            const long long orow = out_row0 + (long long)a.out_step * k;
            if (orow >= a.post_rows) continue;
            v = cmul(v, row_factor(reinterpret_cast<const cpx<T> *>(a.post_tab), orow, a.tab_conj));
        }
        S *o = out + (out_row0 + (long long)a.out_step * k) * a.row_stride + 2 * (long long)col;
        if (pairs_out)
            store_pair<A>(o, v);
        else
            store_c<A>(o, v, E);
    }
}

// The last pass of a compile-time column-step chain, from the shared-memory
// tile to global memory: outputs k = base + r LSL of column col0 + w go to
// row out_row0 + out_step k, times W_nx^(g k) when the step has a post
// twiddle.  NT threads (of a possibly larger CTA) share the tasks.
template <class A, int DIR, int FL, int W, int NT>
__device__ __forceinline__ void colstep_last_pass_global(const cpx<typename A::T> *s,
                                                         const cpx<typename A::T> *__restrict__ ptab,
                                                         const ColStepArgs &a, int g, int col0, typename A::S *out,
                                                         long long out_row0, int E, bool pairs_out)
{
    using T = typename A::T;
    using S = typename A::S;
    constexpr int EPT = A::kEPTFixed;
    constexpr int LSL = last_pass_ls(FL, EPT), RL = fixed_radix(FL, LSL, EPT), LRL = FL / RL;
    constexpr int Off = pass_table_offset(FL, EPT, LSL);
    constexpr int NTASK = LRL * W, TPT = (NTASK + NT - 1) / NT;
    const cpx<T> *tw = reinterpret_cast<const cpx<T> *>(a.tw);
    const cpx<T> *tp = ptab + Off;
    const int tid = threadIdx.x;
    if (tid >= NT) return;
#pragma unroll
    for (int t = 0; t < TPT; ++t) {
        const int task = tid + t * NT;
        if (NTASK % NT == 0 || task < NTASK) {
            const int w = task % W, jj = task / W, col = col0 + w;
            const int k = jj % LSL;
            cpx<T> v[RL];
#pragma unroll
            for (int r = 0; r < RL; ++r) v[r] = s[pidx((jj + r * LRL) * W + w)];
#pragma unroll
            for (int r = 1; r < RL; ++r) v[r] = cmul(v[r], twid<DIR>(tp, (r - 1) * LSL + k));
            DFT<RL, DIR, T>::run(v);
            if (col < a.ncols) {
                const int base = (jj - k) * RL + k;
#pragma unroll
                for (int r = 0; r < RL; ++r) {
                    const int kk = base + r * LSL;
                    cpx<T> o = v[r];
                    if (a.post && g) o = cmul(o, twid<DIR>(tw, g * kk));
                    S *dst = out + (out_row0 + (long long)a.out_step * kk) * a.row_stride + 2 * (long long)col;
                    if (pairs_out)
                        store_pair<A>(dst, o);
                    else
                        store_c<A>(dst, o, E);
                }
            }
        }
    }
}

// A column step with the first pass fed from global memory and the last
// pass written to it, so shared memory only carries the transposes between
// passes (one round trip for L = 128 in FP32 instead of three).  Same
// contract as colstep_kernel.  Written for FP32 and for float-float with
// pair input (the block's scale comes from the producers' exponents, so no
// data-dependent reduction has to precede the first pass); the launcher
// uses it for FP32.
// Body of block (bx, by) of the grid: group bx / strips, strip bx % strips,
// batch item by.  Threads past the shape's own count idle (the persistent
// batch kernel runs it in larger CTAs).
template <class A, int DIR, int FL, int FW>
__device__ __forceinline__ void colstep_direct_body(const ColStepArgs &a, int bx, int by, int gx)
{
    using T = typename A::T;
    using S = typename A::S;
    constexpr int EPT = A::kEPTFixed;
    constexpr int W = 1 << FW;
    constexpr int NT = fixed_threads(FL, FW, EPT);
    constexpr int R1 = fixed_radix(FL, 1, EPT), LR1 = FL / R1;
    constexpr int LSL = last_pass_ls(FL, EPT), RL = fixed_radix(FL, LSL, EPT), LRL = FL / RL;
    static_assert(LSL > 1, "at least two passes");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T> *s = reinterpret_cast<cpx<T> *>(smem_raw);
    const int tid = threadIdx.x;
    const int g = bx / a.strips, col0 = (bx % a.strips) * W;
    const S *in = reinterpret_cast<const S *>(a.in) + (long long)by * a.in_bstride;
    S *out = reinterpret_cast<S *>(a.out) + (long long)by * a.out_bstride;
    const cpx<T> *tw = reinterpret_cast<const cpx<T> *>(a.tw);
    const cpx<T> *ptab = reinterpret_cast<const cpx<T> *>(a.ptab);
    const long long in_row0 = (long long)g * a.in_gmul, out_row0 = (long long)g * a.out_gmul;

    int Eblk = kExpNone;
    [[maybe_unused]] float *fac = nullptr;
    if constexpr (A::kScaled) {
        __shared__ int sEm, sExp[kColStepMaxPairL];
        __shared__ float sFac[kColStepMaxPairL];
        if (tid == 0) sEm = kExpNone;
        __syncthreads();
        const int *ein = a.exp_in + (long long)by * a.exp_in_bstride;
        for (int m = tid; m < FL; m += NT) {
            const int r = (int)(in_row0 + (long long)a.in_step * m);
            const int e = ein[(r % a.exp_rmod) * a.exp_rmul + (col0 >> a.exp_cshift)];
            sExp[m] = e;
            atomicMax(&sEm, e);
        }
        __syncthreads();
        Eblk = sEm;
        for (int m = tid; m < FL; m += NT) sFac[m] = Eblk == kExpNone ? 1.0f : pow2_le0(sExp[m] - Eblk);
        __syncthreads();
        fac = sFac;
    }

    // first pass: task (jj, w) takes elements jj + LR1 r of column w
    {
        constexpr int NTASK = LR1 * W, TPT = (NTASK + NT - 1) / NT;
#pragma unroll
        for (int t = 0; t < TPT; ++t) {
            const int task = tid + t * NT;
            if (tid < NT && (NTASK % NT == 0 || task < NTASK)) {
                const int w = task % W, jj = task / W, col = col0 + w;
                const bool live = col < a.ncols;
                cpx<T> v[R1];
                using V2 = typename std::conditional<sizeof(S) == 8, double2, float2>::type;
                V2 raw[R1];
#pragma unroll
                for (int r = 0; r < R1; ++r) {
                    raw[r] = V2{};
                    if (live)
                        raw[r] = ld_stream(in + (in_row0 + (long long)a.in_step * (jj + r * LR1)) * a.row_stride +
                                           2 * (long long)col);
                }
#pragma unroll
                for (int r = 0; r < R1; ++r) {
                    if constexpr (A::kScaled) {
                        const float4 q = *reinterpret_cast<const float4 *>(&raw[r]);
                        const float f = fac[jj + r * LR1];
                        v[r] = cpx<T>{ff{q.x * f, q.y * f}, ff{q.z * f, q.w * f}};
                    } else {
                        v[r] = cpx<T>{(T)raw[r].x, (T)raw[r].y};
                    }
                }
                DFT<R1, DIR, T>::run(v);
#pragma unroll
                for (int r = 0; r < R1; ++r) s[pidx((jj * R1 + r) * W + w)] = v[r];  // pass 0: no renorm
            }
        }
    }
    __syncthreads();

    FixedPassRange<T, FL, W, NT, DIR, EPT, R1, 0, LSL>::run(s, ptab);

    // last pass: outputs k = base + r LSL go straight to their rows
    const bool pairs_out = A::kScaled && a.pairs_out;
    if (pairs_out && tid == 0) a.exp_out[bx + (long long)gx * by] = Eblk;
    colstep_last_pass_global<A, DIR, FL, W, NT>(s, ptab, a, g, col0, out, out_row0, Eblk == kExpNone ? 0 : Eblk,
                                                pairs_out);
}

template <class A, int DIR, int FL, int FW>
__global__ void __launch_bounds__(fixed_threads(FL, FW, A::kEPTFixed),
                                  fixed_threads(FL, FW, A::kEPTFixed) <= kFixedThreadsMax ? kFixedMinBlocks : 1)
    colstep_direct_kernel(ColStepArgs a)
{
    colstep_direct_body<A, DIR, FL, FW>(a, blockIdx.x + a.block_offset, blockIdx.y, a.grid_blocks);
}

// --------------------------------------------------------- twiddle tables
// W_N^e = exp(-2 pi i e / N) from FP64 sincospi, rounded once to the compute
// type (float-float keeps 48 of its 53 bits).
template <class T>
__global__ void twiddle_kernel(cpx<T> *tab, int N)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N) return;
    double sn, cs;
    sincospi(2.0 * (double)e / (double)N, &sn, &cs);
    const double re = cs, im = -sn;
    if constexpr (std::is_same<T, ff>::value) {
        ff r, i;
        r.hi = (float)re;
        r.lo = (float)(re - (double)r.hi);
        i.hi = (float)im;
        i.lo = (float)(im - (double)i.hi);
        tab[e] = cpx<ff>{r, i};
    } else {
        tab[e] = cpx<T>{(T)re, (T)im};
    }
}

// Per-pass table of a compile-time chain: out[(r-1)*Ls + k] = W_{Ls R}^{r k}.
template <class T>
__global__ void pass_twiddle_kernel(cpx<T> *out, int Ls, int R)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= Ls * (R - 1)) return;
    const int r = 1 + e / Ls, k = e % Ls;
    double sn, cs;
    sincospi(2.0 * (double)(r * k) / (double)(Ls * R), &sn, &cs);
    const double re = cs, im = -sn;
    if constexpr (std::is_same<T, ff>::value) {
        ff a, b;
        a.hi = (float)re;
        a.lo = (float)(re - (double)a.hi);
        b.hi = (float)im;
        b.lo = (float)(im - (double)b.hi);
        out[e] = cpx<ff>{a, b};
    } else {
        out[e] = cpx<T>{(T)re, (T)im};
    }
}

}  // namespace hpxfft_gpu
