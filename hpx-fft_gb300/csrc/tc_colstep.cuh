// Split-BF16 tensor-core column step and row r2c (precision
// HPXFFT_PREC_BF16X3).  The row kernel (bottom of this file) runs the same
// tensor-core stage on the first pass of its rows.
//
// Same contract as colstep_kernel (one step of the four-step column FFT,
// nx = N1 * N2), for DFT lengths L = 16 * L2, L2 in {2, 4, 8, 16}.  The first
// Stockham pass (radix 16, no twiddles) of every length-L transform runs on
// the tensor cores: a CTA holds NV (512 or 256) length-16 vectors x (vector (j, w) =
// elements j + (L/16) t, t = 0..15, of column w), and the 16-point complex DFT
// of all of them is one real matrix product
//     D[v][n] = sum_k A[v][k] B[k][n],   A[v] = (Re x_0..15, Im x_0..15),
//     B = [[C, S], [-S, C]],  C[t][q] = cos(2 pi q t / 16),
//                            S[t][q] = -+sin(2 pi q t / 16) (forward / inverse),
// so D[v] = (Re X_0..15, Im X_0..15).  A and B are each split into three BF16
// terms (x = x0 + x1 + x2 exactly to 24 bits) and the six products with
// i + j <= 2 accumulate in FP32 in tensor memory: NV / 128 blocks of 128 vectors,
// tcgen05.mma M = 128, N = 32, K = 6 x 32.  The remaining passes, the
// four-step twiddle and the stores run on the CUDA cores in FP32.
//
// Shared-memory operands use the no-swizzle K-major layout of 8 x 16-byte
// core matrices; core matrix (row group g, K chunk c) sits at g * 512 + c * 128
// (leading byte offset 128, stride byte offset 512), so one operand of 128
// rows x 32 K is 8 KB and every address the MMA forms stays inside it.
#pragma once
#include <cuda_bf16.h>

#include "fft_kernels.cuh"
#include "tc_ptx.cuh"

namespace hpxfft_gpu {

// NV = length-16 vectors per CTA (512: 2 CTAs per SM, 256: 4 CTAs per SM),
// one vector per thread, NV / 128 MMA row blocks.
constexpr int kTcOperandBytes = 128 * 32 * 2;               // one 128 x 32 BF16 operand
constexpr int kTcBSplitBytes = 32 * 32 * 2;                 // one 32 x 32 BF16 DFT matrix
constexpr int kTcBBytes = 3 * kTcBSplitBytes;               // its three splits
__host__ __device__ constexpr int tc_a_bytes(int NV) { return NV / 128 * 3 * kTcOperandBytes; }
__host__ __device__ constexpr size_t tc_smem(int NV) { return (size_t)tc_a_bytes(NV) + kTcBBytes + 128; }
__host__ __device__ constexpr int tc_tmem_cols(int NV) { return NV / 128 * 32; }  // FP32 accumulators
static_assert((size_t)padded_elems(256 * 16) * 8 <= (size_t)tc_a_bytes(256), "FP32 tile must fit the A region");
static_assert((size_t)padded_elems(512 * 16) * 8 <= (size_t)tc_a_bytes(512), "FP32 tile must fit the A region");

struct TcColStepArgs {
    ColStepArgs c;
    const void *dft;       // BF16 DFT-16 matrices: [forward, inverse][split] in the operand layout
    int *error;            // set to 1 when a tensor-core wait gives up
    long long spin_limit;  // polls of the MMA barrier before giving up
};


// Byte offset of (row, 16-byte K chunk) in an operand.
__device__ __forceinline__ int tc_row_offset(int row, int chunk) { return (row >> 3) * 512 + chunk * 128 + (row & 7) * 16; }

// x = h + m + l, each a BF16, for 8 reals; packed two per 32-bit word in K order
__device__ __forceinline__ void split3_bf16(const float (&v)[8], uint4 &h, uint4 &m, uint4 &l)
{
    uint32_t ph[4], pm[4], pl[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const __nv_bfloat162 bh = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
        const float2 fh = __bfloat1622float2(bh);
        const float r0 = v[2 * i] - fh.x, r1 = v[2 * i + 1] - fh.y;  // exact
        const __nv_bfloat162 bm = __floats2bfloat162_rn(r0, r1);
        const float2 fm = __bfloat1622float2(bm);
        const __nv_bfloat162 bl = __floats2bfloat162_rn(r0 - fm.x, r1 - fm.y);
        ph[i] = *reinterpret_cast<const uint32_t *>(&bh);
        pm[i] = *reinterpret_cast<const uint32_t *>(&bm);
        pl[i] = *reinterpret_cast<const uint32_t *>(&bl);
    }
    h = make_uint4(ph[0], ph[1], ph[2], ph[3]);
    m = make_uint4(pm[0], pm[1], pm[2], pm[3]);
    l = make_uint4(pl[0], pl[1], pl[2], pl[3]);
}

// ---- the tensor-core DFT-16 stage, shared by the column-step and row kernels

// Tensor memory for the accumulators (warp 0), the MMA barrier (thread 0)
// and the DFT matrix of direction dir into sB.  The caller's next CTA barrier
// (inside tc_dft16) publishes all three.
template <int NV>
__device__ __forceinline__ void tc_setup(uint32_t *tmem_slot, uint64_t *bar, unsigned char *sB, const void *dft,
                                         int dir)
{
    const int tid = threadIdx.x;
    if ((tid >> 5) == 0) {
        tc::tmem_alloc(tmem_slot, tc_tmem_cols(NV));
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        tc::fence_mbar_init();
    }
    const uint4 *src = reinterpret_cast<const uint4 *>(dft) + (dir < 0 ? 0 : kTcBBytes / 16);
    for (int i = tid; i < kTcBBytes / 16; i += NV) reinterpret_cast<uint4 *>(sB)[i] = src[i];
}

// DFT-16 of the CTA's NV vectors, one per thread: x = the thread's 16
// inputs, y = its 16 outputs (Re X_0..15, Im X_0..15).  Contains the CTA
// barriers.  Returns false in every thread if the MMA wait gave up (after
// flagging *error and waiting once more, bounded); on true the operand
// space is free again.
template <int NV>
__device__ __forceinline__ bool tc_dft16(const float2 (&x)[16], float (&y)[32], unsigned char *sA,
                                         const unsigned char *sB, const uint32_t *tmem_slot, uint64_t *bar,
                                         int *error, long long spin_limit)
{
    constexpr int kTcBlocks = NV / 128;
    const int tid = threadIdx.x, warp = tid >> 5;
    {
        // operand row tid & 127 of block tid >> 7; K chunks 0, 1: real parts, 2, 3: imaginary parts
        unsigned char *arow = sA + (tid >> 7) * 3 * kTcOperandBytes;
        const int row = tid & 127;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) v[e] = c < 2 ? x[8 * c + e].x : x[8 * (c - 2) + e].y;
            uint4 h, m, l;
            split3_bf16(v, h, m, l);
            const int off = tc_row_offset(row, c);
            *reinterpret_cast<uint4 *>(arow + off) = h;
            *reinterpret_cast<uint4 *>(arow + kTcOperandBytes + off) = m;
            *reinterpret_cast<uint4 *>(arow + 2 * kTcOperandBytes + off) = l;
        }
    }
    tc::fence_proxy_async();  // generic-proxy operand stores -> tensor core
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    if (tid == 0) {
        constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 32);
        // products A_i B_j, i + j <= 2, smallest terms first
        constexpr int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
        const uint32_t a0 = tc::smem_addr(sA), b0 = tc::smem_addr(sB);
#pragma unroll
        for (int blk = 0; blk < kTcBlocks; ++blk) {
#pragma unroll
            for (int q = 0; q < 6; ++q) {
#pragma unroll
                for (int ks = 0; ks < 2; ++ks) {  // K = 16 per instruction: two 16-byte chunks
                    const uint64_t ad = tc::smem_desc(a0 + (blk * 3 + pa[q]) * kTcOperandBytes + ks * 256, 128, 512);
                    const uint64_t bd = tc::smem_desc(b0 + pb[q] * kTcBSplitBytes + ks * 256, 128, 512);
                    tc::mma_f16(tmem + blk * 32, ad, bd, idesc, (q | ks) ? 1u : 0u);
                }
            }
        }
        tc::mma_commit(bar);
    }

    int ok = 1;
    for (long long spins = 0; !tc::mbar_try_wait(bar, 0);) {
        if (++spins > spin_limit) {
            ok = 0;
            break;
        }
    }
    const int all_ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    if (all_ok) {
        // warp w reads TMEM lanes 32 (w % 4).. of block w / 4: row tid & 127 of block tid >> 7, its own vector
        tc::tmem_ld_32x32b_x32(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(32 * (warp >> 2)), y);
    } else if (tid == 0) {
        atomicExch(error, 1);
        // one more bounded wait for the MMAs in flight before their TMEM is freed
        for (long long spins = 0; !tc::mbar_try_wait(bar, 0) && spins < spin_limit; ++spins) {
        }
    }
    return all_ok != 0;
}

// Free the tensor memory once every thread's loads from it are done.
template <int NV>
__device__ __forceinline__ void tc_teardown(const uint32_t *tmem_slot)
{
    tc::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(*tmem_slot, tc_tmem_cols(NV));
    }
}

template <int DIR, int FL, int NV>
__global__ void __launch_bounds__(NV, 2 * 512 / NV) colstep_tc_kernel(TcColStepArgs ta)
{
    constexpr int LR = FL / 16;                // vectors per column
    constexpr int W = NV / LR;                 // columns per CTA
    constexpr int log2W = ilog2c(W);
    static_assert(FL % 16 == 0 && (1 << log2W) == W, "length must be 16 times a power of two");
    const ColStepArgs &a = ta.c;
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t s_bar;
    __shared__ uint32_t s_tmem;
    unsigned char *base = smem_raw + ((128 - (tc::smem_addr(smem_raw) & 127)) & 127);
    unsigned char *sA = base;
    unsigned char *sB = base + tc_a_bytes(NV);
    cpx<float> *s = reinterpret_cast<cpx<float> *>(base);  // FP32 tile once the MMAs are done

    const int tid = threadIdx.x;
    const int bx = blockIdx.x + a.block_offset;
    const int g = bx / a.strips, col0 = (bx % a.strips) * W;
    const float *in = reinterpret_cast<const float *>(a.in) + (long long)blockIdx.y * a.in_bstride;
    float *out = reinterpret_cast<float *>(a.out) + (long long)blockIdx.y * a.out_bstride;
    const cpx<float> *ptab = reinterpret_cast<const cpx<float> *>(a.ptab);
    const long long in_row0 = (long long)g * a.in_gmul, out_row0 = (long long)g * a.out_gmul;

    tc_setup<NV>(&s_tmem, &s_bar, sB, ta.dft, DIR);
    // this thread's vector: column w, elements jj + LR t
    const int jj = tid >> log2W, w = tid & (W - 1), col = col0 + w;
    float2 x[16];
    {
        const bool live = col < a.ncols;
        const float *src = in + (in_row0 + (long long)a.in_step * jj) * a.row_stride + 2 * (long long)col;
        const long long tstride = (long long)a.in_step * LR * a.row_stride;
#pragma unroll
        for (int t = 0; t < 16; ++t) x[t] = live ? ld_stream(src + t * tstride) : make_float2(0.f, 0.f);
    }
    float y[32];
    const bool ok = tc_dft16<NV>(x, y, sA, sB, &s_tmem, &s_bar, ta.error, ta.spin_limit);
    if (ok)  // Stockham order after the first radix-16 pass: output q of vector jj at element 16 jj + q
#pragma unroll
        for (int q = 0; q < 16; ++q) s[pidx(((16 * jj + q) << log2W) + w)] = cpx<float>{y[q], y[16 + q]};
    tc_teardown<NV>(&s_tmem);
    if (!ok) return;

    // remaining FP32 passes; the last one writes its rows directly
    FixedPassRange<float, FL, W, NV, DIR, 16, 16, 0, last_pass_ls(FL, 16)>::run(s, ptab);
    colstep_last_pass_global<ArithF32, DIR, FL, W, NV>(s, ptab, a, g, col0, out, out_row0, 0, false);
}

// Row r2c with the first radix-16 pass on the tensor cores: W rows of M = FL
// packed-real points per CTA (NV = FL W / 16 vectors, one per thread; vector
// (jj, w) = z[jj + (FL/16) t] of row w), then the FP32 passes and the
// packed-real split, as row_r2c_kernel.
struct TcRowArgs {
    RowArgs r;
    const void *dft;
    int *error;
    long long spin_limit;
};

template <int FL, int FW>
__global__ void __launch_bounds__(FL * (1 << FW) / 16, 1024 / (FL * (1 << FW) / 16)) row_r2c_tc_kernel(TcRowArgs ta)
{
    constexpr int W = 1 << FW, NV = FL * W / 16, LR = FL / 16;
    static_assert(NV == 128 || NV == 256 || NV == 512, "128, 256 or 512 vectors per CTA");
    static_assert(FL >= 32, "a pass after the tensor-core one");
    const RowArgs &a = ta.r;
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t s_bar;
    __shared__ uint32_t s_tmem;
    unsigned char *base = smem_raw + ((128 - (tc::smem_addr(smem_raw) & 127)) & 127);
    unsigned char *sA = base;
    unsigned char *sB = base + tc_a_bytes(NV);
    cpx<float> *s = reinterpret_cast<cpx<float> *>(base);

    const int tid = threadIdx.x, bidx = blockIdx.y, row0 = blockIdx.x * W;
    const float *in = reinterpret_cast<const float *>(a.in) + (long long)bidx * a.in_bstride;
    float *out = reinterpret_cast<float *>(a.out) + (long long)bidx * a.out_bstride;
    const cpx<float> *tw = reinterpret_cast<const cpx<float> *>(a.tw);
    const cpx<float> *ptab = reinterpret_cast<const cpx<float> *>(a.ptab);

    tc_setup<NV>(&s_tmem, &s_bar, sB, ta.dft, -1);
    const int jj = tid >> FW, w = tid & (W - 1), row = row0 + w;
    float2 x[16];
    {
        const bool live = row < a.nrows;
        const float *src = in + (long long)row * a.in_stride + 2 * (long long)jj;
#pragma unroll
        for (int t = 0; t < 16; ++t) x[t] = live ? ld_stream(src + 2 * (long long)LR * t) : make_float2(0.f, 0.f);
    }
    float y[32];
    const bool ok = tc_dft16<NV>(x, y, sA, sB, &s_tmem, &s_bar, ta.error, ta.spin_limit);
    if (ok)
#pragma unroll
        for (int q = 0; q < 16; ++q) s[pidx(((16 * jj + q) << FW) + w)] = cpx<float>{y[q], y[16 + q]};
    tc_teardown<NV>(&s_tmem);
    if (!ok) return;

    constexpr int LSL = last_pass_ls(FL, 16);
    if constexpr (fixed_radix(FL, LSL, 16) <= 8) {  // last pass fused with the packed-real split
        FixedPassRange<float, FL, W, NV, -1, 16, 16, 0, LSL>::run(s, ptab);
        row_last_pass_split<ArithF32, FL, FW, NV>(s, ptab, a, row0, tw, out, bidx, nullptr);
    } else {
        FixedPassRange<float, FL, W, NV, -1, 16, 16, 0, FL>::run(s, ptab);
        row_r2c_split<ArithF32>(s, a, row0, FW, tw, out, bidx, nullptr, tid, NV);
    }
}

// The three BF16 splits of the real DFT-16 matrix B (K-major: row n of the
// operand holds B[0..31][n]), forward then inverse, from FP64 sincospi.
__global__ void tc_dft16_table_kernel(__nv_bfloat16 *out)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 2 * 32 * 32) return;
    const int inv = e >> 10, n = (e >> 5) & 31, k = e & 31;
    const int q = n & 15, t = k & 15;
    double sn, cs;
    sincospi(2.0 * (double)((q * t) & 15) / 16.0, &sn, &cs);
    const double s = inv ? sn : -sn;  // Im exp(-+2 pi i q t / 16)
    const double v = (k < 16) == (n < 16) ? cs : (k < 16 ? s : -s);
    const float f = (float)v;
    const __nv_bfloat16 h = __float2bfloat16_rn(f);
    const float r = f - __bfloat162float(h);
    const __nv_bfloat16 m = __float2bfloat16_rn(r);
    const __nv_bfloat16 l = __float2bfloat16_rn(r - __bfloat162float(m));
    const int off = ((n >> 3) * 512 + (k >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2) / 2;  // BF16 elements
    __nv_bfloat16 *dst = out + inv * (kTcBBytes / 2);
    dst[off] = h;
    dst[kTcBSplitBytes / 2 + off] = m;
    dst[kTcBSplitBytes + off] = l;
}

}  // namespace hpxfft_gpu
