// Dimensions the direct kernels do not cover.  FFTW, which the reference
// calls for both passes (core/src/util/adapter_fftw.cpp:6-34, planned in
// core/src/shared/loop.cpp:163-182), takes any length; the direct kernels
// here take lengths without a prime factor above 13 that one CTA cluster
// holds (and power-of-two columns through the two-kernel pass).  Two
// mechanisms cover the rest, both built on the column kernels:
//
//   * Bluestein's chirp-z convolution for a length L with a large prime
//     factor.  With c[n] = exp(-i pi n^2 / L) and nk = (n^2 + k^2 - (k-n)^2)/2,
//       X[k] = sum_n x[n] W_L^(nk) = c[k] sum_n (x[n] c[n]) conj(c[k - n]),
//     a cyclic convolution of length M >= 2L - 1 (a power of two) with
//     b[m] = conj(c[m]) for 0 <= m < L, b[M - m] = b[m], zero elsewhere:
//       y = IDFT_M(DFT_M(pad_M(x c)) * DFT_M(b));  X[k] = c[k] y[k] / M.
//     DFT_M(b) / M is computed once per plan on the host in FP64.  The
//     inverse DFT uses conj(c) and conj(DFT_M(b)) (b is even, so
//     DFT_M(conj b) = conj DFT_M(b)).
//   * The row pass on a transposed copy, for rows whose half length has no
//     single-cluster plan (a large prime factor: through Bluestein; a long
//     smooth length: the column kernels of that length directly).  The
//     packed rows z_i[n] = x_i[2n] + i x_i[2n+1] become the columns of a
//     scratch array, the column kernels transform them, and the r2c split
//     (the row kernel's post-processing) runs while transposing back.
//
// Every kernel here is an elementwise or 32 x 32 tiled-transpose pass in one
// of three modes (TableFormat): FP32; FP64 on the DFMA pipe (the DFMA
// plan); FP64 storage with float-float arithmetic (the FP64 plan: the FP64
// pipe runs 1/67 of the FP32 rate on this part).  A plan's tables are in
// its mode's format, which is also the column steps' compute type.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace hpxfft_gpu {

// Smallest power of two >= 2 L - 1: the convolution length for length L.
size_t bluestein_length(size_t L);

// Arithmetic modes and table formats: FP32 complex, FP64 complex,
// float-float complex (hi, lo per part).
enum TableFormat { kTabF32 = 0, kTabF64 = 1, kTabFF = 2 };

// Device tables for length L, convolution length M:
// chirp[n] = exp(-i pi n^2 / L), n < L, and kernel[k] = DFT_M(b)[k] / M, k < M.
// Allocates both (cudaMalloc); the caller frees them.
cudaError_t bluestein_tables(size_t L, size_t M, int fmt, void **chirp, void **kernel);

// Device table w[k] = W_2h^k = exp(-i pi k / h), k = 0..h (the r2c split of
// rows of 2h reals).  Allocates; the caller frees.
cudaError_t split_table(size_t h, int fmt, void **w);

// out[b][r][j] = f(r) in[b][r][j] for r < rows_in, 0 for rows_in <= r < rows_out
// (j < ncols); f(r) = tab[r], conjugated when conj.  Strides in complex
// elements; `in` may be `out`.
cudaError_t scale_rows(int mode, const void *in, long long in_rs, long long in_bs, void *out, long long out_rs,
                       long long out_bs, const void *tab, int conj, long long rows_in, long long rows_out,
                       long long ncols, int batch, cudaStream_t st);

// dst[b][r][c] = f src[b][c][r] for c < src_rows and r < src_cols, 0 elsewhere
// (r < dst_rows, c < dst_cols); f = tab[r] (tab_on_col 0) or tab[c]
// (tab_on_col 1), conjugated when conj, or 1 when tab is null.  `src` and
// `dst` must not overlap.
cudaError_t transpose_scaled(int mode, const void *src, long long s_rs, long long s_bs, long long src_rows,
                             long long src_cols, void *dst, long long d_rs, long long d_bs, long long dst_rows,
                             long long dst_cols, const void *tab, int tab_on_col, int conj, int batch,
                             cudaStream_t st);

// The r2c split while transposing back: Z_i[k] = f(k) t[b][k][i] for k < h
// (f = chirp[k], or 1 when chirp is null) are the length-h DFTs of the
// packed rows; row i of `out` gets, for k = 0..h,
//   X[k] = (Z[k] + conj Z[h-k]) / 2 - (i / 2) W_2h^k (Z[k] - conj Z[h-k])
// (indices mod h), the same split the row kernel applies.
cudaError_t r2c_split(int mode, const void *t, long long t_rs, long long t_bs, long long h, const void *chirp,
                      const void *w, void *out, long long o_rs, long long o_bs, long long nrows, int batch,
                      cudaStream_t st);

// The c2r merge while transposing: from the half spectra X_i (row i of `in`,
// h + 1 values) t[b][k][i] = f(k) Z_i[k] for k < h and i < nrows, 0
// elsewhere (k < t_rows, i < t_cols), with
//   Z[k] = (X[k] + conj X[h-k]) + i conj(W_2h^k) (X[k] - conj X[h-k]),
// Im X[0] and Im X[h] taken as zero, the interior bins halved when adjoint,
// f = conj chirp[k] (or 1 when chirp is null).  The inverse DFT of Z gives
// the packed rows, as in the row kernel's c2r.
cudaError_t c2r_merge(int mode, const void *in, long long i_rs, long long i_bs, long long nrows, long long h,
                      const void *chirp, const void *w, int adjoint, void *t, long long t_rs, long long t_bs,
                      long long t_rows, long long t_cols, int batch, cudaStream_t st);

// Rows of 2L float-float pairs from the DFTs of their halves (sub-row c =
// pairs 2m + c, raw pairs y[b][2r + c][L] with one exponent each in y_exp):
//   Z[j] = Y0[j mod L] + W_2L^j Y1[j mod L],  j < 2L,
// then the packed-real split X[k], k = 0..2L, the row kernel's.  Written as
// raw pairs with one exponent per row (pairs_out, exp_out) or as doubles.
// wz[k] = W_2L^k and ws[k] = W_4L^k, k = 0..L (float-float tables).
cudaError_t combine_halves_split(const void *y, long long y_bs, const int *y_exp, long long ye_bs, int L,
                                 const void *wz, const void *ws, void *out, long long o_rs, long long o_bs,
                                 int pairs_out, int *exp_out, long long eo_bs, long long nrows, int batch,
                                 cudaStream_t st);

}  // namespace hpxfft_gpu
