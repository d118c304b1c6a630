/*
 * CPU oracle for the HPX-FFT 2D real-to-complex path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker: a plain-C FP64 restatement of the reference's
 * hpxfft::shared::loop algorithm (core/src/shared/loop.cpp:56-113 and
 * :158-189).  Only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it.  The product (libhpxfft_gb300.so) never links it and
 * has no CPU fallback.
 *
 * FFTW 3.3.10 (the reference's 1D engine, third-party and not vendored) is
 * absent from this machine, so the 1D transforms are a project-written
 * mixed-radix Cooley-Tukey restatement of the published DFT definition that
 * FFTW computes:  r2c  X[k] = sum_j x[j] exp(-2 pi i j k / n), k = 0..n/2, and
 * the forward c2c with the same sign, both unnormalised.
 */
#ifndef HPXFFT_ORACLE_H
#define HPXFFT_ORACLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* In-place 1D complex DFT of length n (interleaved re,im).  sign = -1 forward
 * (FFTW_FORWARD), +1 backward (FFTW_BACKWARD, unnormalised). */
int oracle_c2c_1d(double *data, size_t n, int sign);

/* 1D r2c of n real values (n even) into n/2+1 interleaved complex values.
 * in and out may alias (the reference's in-place padded row,
 * core/src/shared/loop.cpp:6-9). */
int oracle_r2c_1d(const double *in, double *out, size_t n);

/* The reference's 2D r2c (hpxfft::shared::loop::fft_2d_r2c_par,
 * core/src/shared/loop.cpp:56-113) on the padded in-place layout:
 * values is n_row x n_col doubles, n_col = 2*(ny/2+1), the first ny doubles of
 * each row are data.  On return row kx holds the n_col/2 complex outputs
 * X[kx][ky].  nthreads worker threads split each of the four phases, like the
 * reference's for_loop(par).  times (may be NULL) receives the phase times in
 * seconds: total, first_fftw, first_trans, second_fftw, second_trans. */
int oracle_fft_2d_r2c(double *values, size_t n_row, size_t n_col, int nthreads, double *times);

/* Adjoint of oracle_fft_2d_r2c: given the upstream gradient G of a real loss
 * w.r.t. the complex half spectrum (n_row x n_col/2 complex, [kx][ky], in the
 * padded buffer), overwrite the buffer with dL/dx (first ny doubles of each
 * row; the 2 pad doubles are set to 0):
 *   dx[i][j] = Re sum_{kx} sum_{ky=0}^{ny/2} G[kx][ky] exp(+2 pi i (kx i/nx + ky j/ny)). */
int oracle_fft_2d_r2c_adjoint(double *values, size_t n_row, size_t n_col, int nthreads);

/* Unnormalised 2D c2r (inverse of oracle_fft_2d_r2c up to a factor nx*ny):
 * Hermitian half spectrum in, real padded layout out.  The imaginary parts of
 * the ky = 0 and ky = ny/2 bins are ignored, as FFTW's c2r does. */
int oracle_fft_2d_c2r(double *values, size_t n_row, size_t n_col, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
