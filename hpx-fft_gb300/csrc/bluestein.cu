// Bluestein's convolution and the transposed row pass: the host-built
// tables and the elementwise / transposing kernels around the column
// transforms (the plan logic that strings them together is in plan.cu).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "bluestein.cuh"
#include "fft_kernels.cuh"

namespace hpxfft_gpu {

// ------------------------------------------------------------ host tables

size_t bluestein_length(size_t L)
{
    size_t M = 1;
    while (M < 2 * L - 1) M <<= 1;
    return M;
}

// exp(-2 pi i num / den), 0 <= num < den, in FP64 (angle error below 1e-15)
static void cis(uint64_t num, uint64_t den, double &re, double &im)
{
    const double a = 6.283185307179586476925286766559 * (double)num / (double)den;
    re = std::cos(a);
    im = -std::sin(a);
}

// In-place forward DFT of a power-of-two length: iterative radix-2
// decimation in time in FP64, twiddles from cos/sin of each angle.
static void host_fft_pow2(std::vector<double> &re, std::vector<double> &im)
{
    const size_t n = re.size();
    for (size_t i = 1, j = 0; i < n; ++i) {  // bit-reversed order
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            std::swap(re[i], re[j]);
            std::swap(im[i], im[j]);
        }
    }
    std::vector<double> wr(n / 2 + 1), wi(n / 2 + 1);
    for (size_t k = 0; k < n / 2; ++k) cis(k, n, wr[k], wi[k]);
    for (size_t len = 2; len <= n; len <<= 1) {
        const size_t half = len / 2, step = n / len;
        for (size_t s = 0; s < n; s += len)
            for (size_t j = 0; j < half; ++j) {
                const double xr = wr[j * step], xi = wi[j * step];
                const size_t a = s + j, b = a + half;
                const double tr = re[b] * xr - im[b] * xi, ti = re[b] * xi + im[b] * xr;
                re[b] = re[a] - tr;
                im[b] = im[a] - ti;
                re[a] += tr;
                im[a] += ti;
            }
    }
}

// chirp (2 L doubles, interleaved) and kernel (2 M doubles) for (L, M);
// kernels up to 2^20 entries are kept for the next plan of the same length
static void host_tables(size_t L, size_t M, std::vector<double> &chirp, std::vector<double> &kernel)
{
    static std::mutex mu;
    static std::map<std::pair<size_t, size_t>, std::vector<double>> cache;
    chirp.assign(2 * L, 0.0);
    for (size_t n = 0; n < L; ++n) {
        const uint64_t r = (uint64_t)((unsigned __int128)n * n % (2 * L));  // n^2 mod 2L
        cis(r, 2 * L, chirp[2 * n], chirp[2 * n + 1]);
    }
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find({L, M});
        if (it != cache.end()) {
            kernel = it->second;
            return;
        }
    }
    std::vector<double> re(M, 0.0), im(M, 0.0);
    for (size_t m = 0; m < L; ++m) {  // b[m] = b[M - m] = conj c[m]
        re[m] = chirp[2 * m];
        im[m] = -chirp[2 * m + 1];
        if (m) {
            re[M - m] = re[m];
            im[M - m] = im[m];
        }
    }
    host_fft_pow2(re, im);
    kernel.resize(2 * M);
    const double s = 1.0 / (double)M;
    for (size_t k = 0; k < M; ++k) {
        kernel[2 * k] = re[k] * s;
        kernel[2 * k + 1] = im[k] * s;
    }
    if (M <= ((size_t)1 << 20)) {
        std::lock_guard<std::mutex> lock(mu);
        cache[{L, M}] = kernel;
    }
}

// allocate and fill a device table from interleaved doubles
static cudaError_t upload(const std::vector<double> &v, int fmt, void **dst)
{
    *dst = nullptr;
    cudaError_t e;
    if (fmt == kTabF32 || fmt == kTabFF) {
        // float-float: each double d as hi = fl(d), lo = fl(d - hi)
        std::vector<float> f(fmt == kTabFF ? 2 * v.size() : v.size());
        for (size_t i = 0; i < v.size(); ++i) {
            if (fmt == kTabF32) {
                f[i] = (float)v[i];
            } else {
                f[2 * i] = (float)v[i];
                f[2 * i + 1] = (float)(v[i] - (double)f[2 * i]);
            }
        }
        if ((e = cudaMalloc(dst, f.size() * sizeof(float))) != cudaSuccess) return e;
        e = cudaMemcpy(*dst, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice);
    } else {
        if ((e = cudaMalloc(dst, v.size() * sizeof(double))) != cudaSuccess) return e;
        e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        cudaFree(*dst);
        *dst = nullptr;
    }
    return e;
}

cudaError_t bluestein_tables(size_t L, size_t M, int fmt, void **chirp, void **kernel)
{
    *chirp = *kernel = nullptr;
    std::vector<double> c, k;
    host_tables(L, M, c, k);
    cudaError_t e = upload(c, fmt, chirp);
    if (e == cudaSuccess) e = upload(k, fmt, kernel);
    return e;
}

cudaError_t split_table(size_t h, int fmt, void **w)
{
    std::vector<double> v(2 * (h + 1));
    for (size_t k = 0; k <= h; ++k) cis(k, 2 * h, v[2 * k], v[2 * k + 1]);
    return upload(v, fmt, w);
}

// ---------------------------------------------------------------- kernels

// Storage and arithmetic of the three modes: FP32; FP64 on the DFMA pipe;
// FP64 storage with float-float arithmetic on the FP32 pipes (the FP64
// pipe runs 1/67 of the FP32 rate on this part).  Float-float values are
// scaled by 2^-E, E the larger exponent of the doubles they came from
// (integer-only conversions, exact scaling).
template <int MODE>
struct Elem;
template <>
struct Elem<kTabF32> {
    using V = float2;
    using T = float;
    static __device__ __forceinline__ int exp_of(V) { return 0; }
    static __device__ __forceinline__ cpx<T> in(V v, int) { return cpx<T>{v.x, v.y}; }
    static __device__ __forceinline__ V out(cpx<T> v, int) { return make_float2(v.re, v.im); }
};
template <>
struct Elem<kTabF64> {
    using V = double2;
    using T = double;
    static __device__ __forceinline__ int exp_of(V) { return 0; }
    static __device__ __forceinline__ cpx<T> in(V v, int) { return cpx<T>{v.x, v.y}; }
    static __device__ __forceinline__ V out(cpx<T> v, int) { return make_double2(v.re, v.im); }
};
template <>
struct Elem<kTabFF> {
    using V = double2;
    using T = ff;
    static __device__ __forceinline__ int exp_of(V v)
    {
        const int e = max(dbl_biased_exp(v.x), dbl_biased_exp(v.y));
        return (e == 0 || e == 0x7ff) ? 0 : e - 1023;
    }
    static __device__ __forceinline__ cpx<T> in(V v, int E)
    {
        return cpx<T>{ff_from_double(v.x, E), ff_from_double(v.y, E)};
    }
    static __device__ __forceinline__ V out(cpx<T> v, int E)
    {
        return make_double2(ff_to_double(renorm(v.re), E), ff_to_double(renorm(v.im), E));
    }
};

template <class V>
__device__ __forceinline__ V vzero()
{
    V r;
    r.x = 0;
    r.y = 0;
    return r;
}

template <class T>
__device__ __forceinline__ cpx<T> tab_at(const cpx<T> *tab, long long i, int conj)
{
    const cpx<T> f = tab[i];
    return conj ? cconj(f) : f;
}

// f v in the mode's arithmetic, back to storage
template <int MODE>
__device__ __forceinline__ typename Elem<MODE>::V scaled(typename Elem<MODE>::V v, cpx<typename Elem<MODE>::T> f)
{
    using E_ = Elem<MODE>;
    const int E = E_::exp_of(v);
    return E_::out(cmul(E_::in(v, E), f), E);
}

template <int MODE>
__global__ void __launch_bounds__(256)
    scale_rows_kernel(const typename Elem<MODE>::V *in, long long in_rs, long long in_bs, typename Elem<MODE>::V *out,
                      long long out_rs, long long out_bs, const cpx<typename Elem<MODE>::T> *tab, int conj,
                      long long rows_in, long long rows_out, long long ncols)
{
    using V = typename Elem<MODE>::V;
    const long long b = blockIdx.z;
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncols) return;
    for (long long r = (long long)blockIdx.y * blockDim.y + threadIdx.y; r < rows_out;
         r += (long long)gridDim.y * blockDim.y) {
        V v = vzero<V>();
        if (r < rows_in) v = scaled<MODE>(in[b * in_bs + r * in_rs + j], tab_at(tab, r, conj));
        out[b * out_bs + r * out_rs + j] = v;
    }
}

// 32 x 32 tiles through shared memory (odd row pitch: no bank conflicts for
// 8- or 16-byte elements), 256 threads, 4 elements per thread each way;
// blockIdx.x = row tile * col_tiles + col tile of the destination
template <int MODE>
__global__ void __launch_bounds__(256)
    transpose_scaled_kernel(const typename Elem<MODE>::V *src, long long s_rs, long long s_bs, long long src_rows,
                            long long src_cols, typename Elem<MODE>::V *dst, long long d_rs, long long d_bs,
                            long long dst_rows, long long dst_cols, unsigned col_tiles,
                            const cpx<typename Elem<MODE>::T> *tab, int tab_on_col, int conj)
{
    using V = typename Elem<MODE>::V;
    __shared__ V tile[32][33];
    const long long r0 = (long long)(blockIdx.x / col_tiles) * 32, c0 = (long long)(blockIdx.x % col_tiles) * 32;
    const long long b = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const long long c = c0 + ty + 8 * q, r = r0 + tx;  // source row c, source column r
        V v = vzero<V>();
        if (c < src_rows && r < src_cols) {
            v = src[b * s_bs + c * s_rs + r];
            if (tab) v = scaled<MODE>(v, tab_at(tab, tab_on_col ? c : r, conj));
        }
        tile[ty + 8 * q][tx] = v;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const long long r = r0 + ty + 8 * q, c = c0 + tx;
        if (r < dst_rows && c < dst_cols) dst[b * d_bs + r * d_rs + c] = tile[tx][ty + 8 * q];
    }
}

// blockIdx.x = k tile * i_tiles + i tile
template <int MODE>
__global__ void __launch_bounds__(256)
    r2c_split_kernel(const typename Elem<MODE>::V *t, long long t_rs, long long t_bs, long long h,
                     const cpx<typename Elem<MODE>::T> *chirp, const cpx<typename Elem<MODE>::T> *w,
                     typename Elem<MODE>::V *out, long long o_rs, long long o_bs, long long nrows, unsigned i_tiles)
{
    using E_ = Elem<MODE>;
    using V = typename E_::V;
    using T = typename E_::T;
    __shared__ cpx<T> za[32][33], zb[32][33];
    __shared__ int ze[32][33];
    const long long k0 = (long long)(blockIdx.x / i_tiles) * 32, i0 = (long long)(blockIdx.x % i_tiles) * 32;
    const long long b = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const long long k = k0 + ty + 8 * q, i = i0 + tx;
        const bool live = k <= h && i < nrows;
        const long long ka = k == h ? 0 : k, kb = k == 0 ? 0 : h - k;
        V a2 = vzero<V>(), c2 = vzero<V>();
        if (live) {
            a2 = t[b * t_bs + ka * t_rs + i];
            c2 = t[b * t_bs + kb * t_rs + i];
        }
        const int E = max(E_::exp_of(a2), E_::exp_of(c2));  // one scale for the pair
        cpx<T> a = E_::in(a2, E), c = E_::in(c2, E);
        if (chirp && live) {
            a = cmul(a, chirp[ka]);
            c = cmul(c, chirp[kb]);
        }
        za[ty + 8 * q][tx] = a;
        zb[ty + 8 * q][tx] = c;
        ze[ty + 8 * q][tx] = E;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const long long i = i0 + ty + 8 * q, k = k0 + tx;
        if (k <= h && i < nrows) {
            const cpx<T> a = za[tx][ty + 8 * q], c = cconj(zb[tx][ty + 8 * q]);  // Z[k], conj Z[h-k]
            const cpx<T> e = chalf(a + c), o = chalf(a - c);
            const cpx<T> wo = cmul(w[k], o);
            const cpx<T> x{e.re + wo.im, e.im - wo.re};  // e - i wo
            out[b * o_bs + i * o_rs + k] = E_::out(x, ze[tx][ty + 8 * q]);
        }
    }
}

// blockIdx.x = k tile * i_tiles + i tile
template <int MODE>
__global__ void __launch_bounds__(256)
    c2r_merge_kernel(const typename Elem<MODE>::V *in, long long i_rs, long long i_bs, long long nrows, long long h,
                     const cpx<typename Elem<MODE>::T> *chirp, const cpx<typename Elem<MODE>::T> *w, int adjoint,
                     typename Elem<MODE>::V *t, long long t_rs, long long t_bs, long long t_rows, long long t_cols,
                     unsigned i_tiles)
{
    using E_ = Elem<MODE>;
    using V = typename E_::V;
    using T = typename E_::T;
    __shared__ V tile[32][33];
    const long long k0 = (long long)(blockIdx.x / i_tiles) * 32, i0 = (long long)(blockIdx.x % i_tiles) * 32;
    const long long b = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const long long k = k0 + tx, i = i0 + ty + 8 * q;
        V zo = vzero<V>();
        if (k < h && i < nrows) {
            V a2 = in[b * i_bs + i * i_rs + k], c2 = in[b * i_bs + i * i_rs + (h - k)];
            if (k == 0) {  // X[0] and X[h]: imaginary parts ignored
                a2.y = 0;
                c2.y = 0;
            }
            const int E = max(E_::exp_of(a2), E_::exp_of(c2));
            cpx<T> a = E_::in(a2, E), c = E_::in(c2, E);
            if (adjoint && k > 0) {  // interior bins halved
                a = chalf(a);
                c = chalf(c);
            }
            c = cconj(c);
            const cpx<T> s = a + c, d = a - c;  // X[k] +- conj X[h-k]
            const cpx<T> wd = cmul(tab_at(w, k, 1), d);
            cpx<T> z{s.re - wd.im, s.im + wd.re};  // s + i wd
            if (chirp) z = cmul(z, tab_at(chirp, k, 1));
            zo = E_::out(z, E);
        }
        tile[ty + 8 * q][tx] = zo;  // [i][k]
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const long long k = k0 + ty + 8 * q, i = i0 + tx;
        if (k < t_rows && i < t_cols) t[b * t_bs + k * t_rs + i] = tile[tx][ty + 8 * q];
    }
}

// blockIdx.x = row * chunks + chunk; thread k of the chunk handles the
// output pair (k, 2L - k), k = 0..L
__global__ void __launch_bounds__(256)
    combine_halves_kernel(const cpx<ff> *y, long long y_bs, const int *y_exp, long long ye_bs, int L,
                          const cpx<ff> *wz, const cpx<ff> *ws, double *out, long long o_rs, long long o_bs,
                          int pairs_out, int *exp_out, long long eo_bs, long long nrows, unsigned chunks)
{
    const long long r = blockIdx.x / chunks, b = blockIdx.z;
    const int k = (int)(blockIdx.x % chunks) * 256 + (int)threadIdx.x;
    const int M = 2 * L;
    if (r >= nrows || k > L) return;
    const int e0 = y_exp[b * ye_bs + 2 * r], e1 = y_exp[b * ye_bs + 2 * r + 1];
    const int E = max(e0, e1);  // kExpNone never wins against a real exponent
    const float f0 = E == kExpNone || e0 == kExpNone ? 0.0f : pow2_le0(e0 - E);
    const float f1 = E == kExpNone || e1 == kExpNone ? 0.0f : pow2_le0(e1 - E);
    const cpx<ff> *y0 = y + b * y_bs + 2 * r * (long long)L, *y1 = y0 + L;
    const int k1 = k == L ? 0 : k, k2 = (L - k1) % L;  // j mod L for j = k and j = M - k
    auto ld = [&](const cpx<ff> *p, int i, float f) {
        const float4 q = __ldcs(reinterpret_cast<const float4 *>(p + i));
        return cpx<ff>{ff{q.x * f, q.y * f}, ff{q.z * f, q.w * f}};
    };
    const cpx<ff> w = wz[k];  // W_M^k; W_M^(M-k) = conj W_M^k
    const cpx<ff> zk = ld(y0, k1, f0) + cmul(w, ld(y1, k1, f1));
    const cpx<ff> zp = ld(y0, k2, f0) + cmul(cconj(w), ld(y1, k2, f1));  // Z[M - k]
    const cpx<ff> zb = cconj(zp);
    const cpx<ff> e = chalf(zk + zb), o = chalf(zk - zb);
    const cpx<ff> tk = cmul(ws[k], o);
    const cpx<ff> xk = e + mul_i<-1>(tk), xm = cconj(e + mul_i<+1>(tk));  // X[k], X[M - k]
    double *orow = out + b * o_bs + r * o_rs;
    if (pairs_out) {
        auto st = [&](long long i, cpx<ff> v) {
            const ff re = renorm(v.re), im = renorm(v.im);
            __stcs(reinterpret_cast<float4 *>(orow + 2 * i), make_float4(re.hi, re.lo, im.hi, im.lo));
        };
        st(k, xk);
        if (M - k != k) st(M - k, xm);
        if (k == 0) exp_out[b * eo_bs + r] = E;
    } else {
        const int Eo = E == kExpNone ? 0 : E;
        auto st = [&](long long i, cpx<ff> v) {
            __stcs(reinterpret_cast<double2 *>(orow + 2 * i),
                   make_double2(ff_to_double(renorm(v.re), Eo), ff_to_double(renorm(v.im), Eo)));
        };
        st(k, xk);
        if (M - k != k) st(M - k, xm);
    }
}

// ---------------------------------------------------------------- launchers

static long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }

template <int MODE>
using VT = typename Elem<MODE>::V;
template <int MODE>
using CT = cpx<typename Elem<MODE>::T>;

cudaError_t scale_rows(int mode, const void *in, long long in_rs, long long in_bs, void *out, long long out_rs,
                       long long out_bs, const void *tab, int conj, long long rows_in, long long rows_out,
                       long long ncols, int batch, cudaStream_t st)
{
    if (rows_out <= 0 || ncols <= 0 || batch <= 0) return cudaSuccess;
    int bx = 32;
    while (bx > 1 && bx / 2 >= ncols) bx /= 2;
    const int by = 256 / bx;
    const long long gx = ceil_div(ncols, bx);
    long long gy = ceil_div(rows_out, 4LL * by);
    if (gy > 65535) gy = 65535;
    if (gx > 0x7fffffffLL || batch > 65535) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)batch), block(bx, by);
#define HPXFFT_M(MODE)                                                                                           \
    scale_rows_kernel<MODE><<<grid, block, 0, st>>>((const VT<MODE> *)in, in_rs, in_bs, (VT<MODE> *)out, out_rs, \
                                                    out_bs, (const CT<MODE> *)tab, conj, rows_in, rows_out, ncols)
    switch (mode) {
    case kTabF32: HPXFFT_M(kTabF32); break;
    case kTabF64: HPXFFT_M(kTabF64); break;
    case kTabFF: HPXFFT_M(kTabFF); break;
    default: return cudaErrorInvalidValue;
    }
#undef HPXFFT_M
    return cudaGetLastError();
}

// tiles of the destination (rows x cols) as one grid dimension
static bool tile_grid(long long rows, long long cols, int batch, dim3 &grid, unsigned &col_tiles)
{
    const long long rt = ceil_div(rows, 32), ct = ceil_div(cols, 32);
    if (rt * ct > 0x7fffffffLL || ct > 0xffffffffLL || batch > 65535) return false;
    grid = dim3((unsigned)(rt * ct), 1, (unsigned)batch);
    col_tiles = (unsigned)ct;
    return true;
}

cudaError_t transpose_scaled(int mode, const void *src, long long s_rs, long long s_bs, long long src_rows,
                             long long src_cols, void *dst, long long d_rs, long long d_bs, long long dst_rows,
                             long long dst_cols, const void *tab, int tab_on_col, int conj, int batch,
                             cudaStream_t st)
{
    if (dst_rows <= 0 || dst_cols <= 0 || batch <= 0) return cudaSuccess;
    dim3 grid;
    unsigned ct = 0;
    if (!tile_grid(dst_rows, dst_cols, batch, grid, ct)) return cudaErrorInvalidValue;
    const dim3 block(32, 8);
#define HPXFFT_M(MODE)                                                                                    \
    transpose_scaled_kernel<MODE><<<grid, block, 0, st>>>((const VT<MODE> *)src, s_rs, s_bs, src_rows,    \
                                                          src_cols, (VT<MODE> *)dst, d_rs, d_bs, dst_rows, \
                                                          dst_cols, ct, (const CT<MODE> *)tab, tab_on_col, conj)
    switch (mode) {
    case kTabF32: HPXFFT_M(kTabF32); break;
    case kTabF64: HPXFFT_M(kTabF64); break;
    case kTabFF: HPXFFT_M(kTabFF); break;
    default: return cudaErrorInvalidValue;
    }
#undef HPXFFT_M
    return cudaGetLastError();
}

cudaError_t r2c_split(int mode, const void *t, long long t_rs, long long t_bs, long long h, const void *chirp,
                      const void *w, void *out, long long o_rs, long long o_bs, long long nrows, int batch,
                      cudaStream_t st)
{
    if (h <= 0 || nrows <= 0 || batch <= 0) return cudaSuccess;
    dim3 grid;
    unsigned it = 0;
    if (!tile_grid(h + 1, nrows, batch, grid, it)) return cudaErrorInvalidValue;
    const dim3 block(32, 8);
#define HPXFFT_M(MODE)                                                                                          \
    r2c_split_kernel<MODE><<<grid, block, 0, st>>>((const VT<MODE> *)t, t_rs, t_bs, h, (const CT<MODE> *)chirp, \
                                                   (const CT<MODE> *)w, (VT<MODE> *)out, o_rs, o_bs, nrows, it)
    switch (mode) {
    case kTabF32: HPXFFT_M(kTabF32); break;
    case kTabF64: HPXFFT_M(kTabF64); break;
    case kTabFF: HPXFFT_M(kTabFF); break;
    default: return cudaErrorInvalidValue;
    }
#undef HPXFFT_M
    return cudaGetLastError();
}

cudaError_t c2r_merge(int mode, const void *in, long long i_rs, long long i_bs, long long nrows, long long h,
                      const void *chirp, const void *w, int adjoint, void *t, long long t_rs, long long t_bs,
                      long long t_rows, long long t_cols, int batch, cudaStream_t st)
{
    if (t_rows <= 0 || t_cols <= 0 || batch <= 0) return cudaSuccess;
    dim3 grid;
    unsigned it = 0;
    if (!tile_grid(t_rows, t_cols, batch, grid, it)) return cudaErrorInvalidValue;
    const dim3 block(32, 8);
#define HPXFFT_M(MODE)                                                                                         \
    c2r_merge_kernel<MODE><<<grid, block, 0, st>>>((const VT<MODE> *)in, i_rs, i_bs, nrows, h,                 \
                                                   (const CT<MODE> *)chirp, (const CT<MODE> *)w, adjoint,     \
                                                   (VT<MODE> *)t, t_rs, t_bs, t_rows, t_cols, it)
    switch (mode) {
    case kTabF32: HPXFFT_M(kTabF32); break;
    case kTabF64: HPXFFT_M(kTabF64); break;
    case kTabFF: HPXFFT_M(kTabFF); break;
    default: return cudaErrorInvalidValue;
    }
#undef HPXFFT_M
    return cudaGetLastError();
}

cudaError_t combine_halves_split(const void *y, long long y_bs, const int *y_exp, long long ye_bs, int L,
                                 const void *wz, const void *ws, void *out, long long o_rs, long long o_bs,
                                 int pairs_out, int *exp_out, long long eo_bs, long long nrows, int batch,
                                 cudaStream_t st)
{
    if (nrows <= 0 || batch <= 0 || L <= 0) return cudaSuccess;
    const long long chunks = ceil_div(L + 1, 256);
    if (nrows * chunks > 0x7fffffffLL || batch > 65535) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)(nrows * chunks), 1, (unsigned)batch);
    combine_halves_kernel<<<grid, 256, 0, st>>>((const cpx<ff> *)y, y_bs, y_exp, ye_bs, L, (const cpx<ff> *)wz,
                                               (const cpx<ff> *)ws, (double *)out, o_rs, o_bs, pairs_out, exp_out,
                                               eo_bs, nrows, (unsigned)chunks);
    return cudaGetLastError();
}

}  // namespace hpxfft_gpu
