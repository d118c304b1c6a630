/*
 * CPU oracle for the HPX-FFT 2D real-to-complex path -- TEST INFRASTRUCTURE.
 *
 * Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
 * load this file's library; it is the checker, never the product.
 *
 * What it restates (reference file:line, paths within the HPX-FFT project):
 *   - hpxfft::shared::loop::fft_2d_r2c_par   core/src/shared/loop.cpp:56-113
 *       phase 1 row r2c in place             core/src/shared/loop.cpp:61-69, 6-9
 *       phase 2 transpose y->x               core/src/shared/loop.cpp:72-80, 18-25
 *       phase 3 column c2c (forward)         core/src/shared/loop.cpp:83-91, 11-15
 *       phase 4 transpose x->y               core/src/shared/loop.cpp:94-102, 46-53
 *   - the dimension bookkeeping of initialize core/src/shared/loop.cpp:163-167
 *   - the 1D engines: fftw_plan_dft_r2c_1d / fftw_plan_dft_1d(FFTW_FORWARD)
 *       core/src/util/adapter_fftw.cpp:9,14,28,34.  FFTW 3.3.10 (pinned by
 *       spack-repo/environments/hpxfft_ci.yaml:4) is not vendored and not
 *       installed here, so the published transform it computes (unnormalised
 *       DFT, forward sign -1, r2c keeps k = 0..n/2) is restated below with a
 *       mixed-radix Cooley-Tukey recursion of our own.
 *
 * Twiddles are computed in long double and rounded once to double.
 */
#include "hpxfft_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct {
    double re, im;
} cplx;

/* ------------------------------------------------------------------ */
/* twiddle tables W_n^k = exp(-2 pi i k / n), cached per length        */
/* ------------------------------------------------------------------ */
#define TW_CACHE 64
static struct {
    size_t n;
    cplx *w;
} tw_cache[TW_CACHE];
static int tw_count = 0;
static pthread_mutex_t tw_lock = PTHREAD_MUTEX_INITIALIZER;

static void exact_cis(size_t k, size_t n, cplx *out)
{
    /* exp(-2 pi i k/n) with octant symmetry so the long double argument
     * stays in [0, pi/4]. */
    const long double two_pi = 6.283185307179586476925286766559005768L;
    size_t k8 = (8 * (k % n));
    /* reduce to k/n in [0, 1) and use symmetry around multiples of 1/8 */
    size_t oct = k8 / n;          /* 0..7 */
    size_t rem = k8 - oct * n;    /* numerator of the fractional octant */
    long double c, s;
    if (oct % 2 == 0) {
        long double a = two_pi * (long double)rem / (long double)(8 * n);
        c = cosl(a);
        s = sinl(a);
    } else {
        long double a = two_pi * (long double)(n - rem) / (long double)(8 * n);
        /* angle = (oct+1)*pi/4 - a */
        c = sinl(a);
        s = cosl(a);
    }
    /* (c, s) = (cos, sin) of the angle within the first quadrant-pair; rotate */
    long double cr, sr;
    switch (oct) {
    case 0: cr = c;  sr = s;  break;  /* [0, pi/4) */
    case 1: cr = c;  sr = s;  break;  /* [pi/4, pi/2) via complement */
    case 2: cr = -s; sr = c;  break;
    case 3: cr = -s; sr = c;  break;
    case 4: cr = -c; sr = -s; break;
    case 5: cr = -c; sr = -s; break;
    case 6: cr = s;  sr = -c; break;
    default: cr = s; sr = -c; break;
    }
    out->re = (double)cr;
    out->im = (double)(-sr);
}

static const cplx *get_twiddles(size_t n)
{
    pthread_mutex_lock(&tw_lock);
    for (int i = 0; i < tw_count; ++i) {
        if (tw_cache[i].n == n) {
            const cplx *w = tw_cache[i].w;
            pthread_mutex_unlock(&tw_lock);
            return w;
        }
    }
    cplx *w = (cplx *)malloc(sizeof(cplx) * (n ? n : 1));
    if (w) {
        for (size_t k = 0; k < n; ++k) exact_cis(k, n, &w[k]);
        int slot = tw_count < TW_CACHE ? tw_count++ : (int)(n % TW_CACHE);
        if (tw_count == TW_CACHE && tw_cache[slot].w) {
            /* table evicted while another thread may hold it: keep it alive
             * (tiny, bounded leak) rather than free under a reader */
        }
        tw_cache[slot].n = n;
        tw_cache[slot].w = w;
    }
    pthread_mutex_unlock(&tw_lock);
    return w;
}

/* ------------------------------------------------------------------ */
/* 1D complex DFT: recursive decimation in time, out of place          */
/* ------------------------------------------------------------------ */
static size_t first_factor(size_t n)
{
    if (n % 4 == 0) return 4;
    if (n % 2 == 0) return 2;
    if (n % 3 == 0) return 3;
    if (n % 5 == 0) return 5;
    for (size_t p = 7; p * p <= n; p += 2)
        if (n % p == 0) return p;
    return n;
}

static inline cplx cmul(cplx a, cplx b)
{
    cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}

/* W_N^e for the sign in use; tw holds exp(-2 pi i k/N). */
static inline cplx wpow(const cplx *tw, size_t N, size_t e, int sign)
{
    cplx w = tw[e % N];
    if (sign > 0) w.im = -w.im;
    return w;
}

/* out[0..n) = DFT_n of in[0], in[istride], ..., tw is the table of the full
 * length N (n divides N). */
static void dft_rec(const cplx *in, size_t istride, cplx *out, size_t n, const cplx *tw, size_t N, int sign,
                    cplx *tmp)
{
    if (n == 1) {
        out[0] = in[0];
        return;
    }
    size_t p = first_factor(n);
    size_t m = n / p;
    for (size_t q = 0; q < p; ++q) dft_rec(in + q * istride, istride * p, out + q * m, m, tw, N, sign, tmp);
    const size_t step = N / n; /* W_n^j = W_N^(j*step) */
    for (size_t k = 0; k < m; ++k) {
        /* gather + twiddle: a_q = W_n^{qk} * sub_q[k] */
        for (size_t q = 0; q < p; ++q) {
            cplx v = out[q * m + k];
            tmp[q] = q == 0 ? v : cmul(v, wpow(tw, N, q * k * step, sign));
        }
        if (p == 2) {
            cplx a = tmp[0], b = tmp[1];
            out[k].re = a.re + b.re;
            out[k].im = a.im + b.im;
            out[k + m].re = a.re - b.re;
            out[k + m].im = a.im - b.im;
        } else if (p == 4) {
            cplx a = tmp[0], b = tmp[1], c = tmp[2], d = tmp[3];
            cplx s0 = {a.re + c.re, a.im + c.im}, d0 = {a.re - c.re, a.im - c.im};
            cplx s1 = {b.re + d.re, b.im + d.im}, d1 = {b.re - d.re, b.im - d.im};
            /* multiply d1 by -i (forward) or +i (backward) */
            cplx j1 = sign < 0 ? (cplx){d1.im, -d1.re} : (cplx){-d1.im, d1.re};
            out[k].re = s0.re + s1.re;
            out[k].im = s0.im + s1.im;
            out[k + m].re = d0.re + j1.re;
            out[k + m].im = d0.im + j1.im;
            out[k + 2 * m].re = s0.re - s1.re;
            out[k + 2 * m].im = s0.im - s1.im;
            out[k + 3 * m].re = d0.re - j1.re;
            out[k + 3 * m].im = d0.im - j1.im;
        } else {
            /* generic small DFT: out[k + m t] = sum_q a_q W_p^{q t} */
            const size_t pstep = N / p;
            for (size_t t = 0; t < p; ++t) {
                cplx acc = tmp[0];
                for (size_t q = 1; q < p; ++q) {
                    cplx w = wpow(tw, N, ((q * t) % p) * pstep, sign);
                    cplx v = cmul(tmp[q], w);
                    acc.re += v.re;
                    acc.im += v.im;
                }
                tmp[p + t] = acc;
            }
            for (size_t t = 0; t < p; ++t) out[k + m * t] = tmp[p + t];
        }
    }
}

static int c2c_into(const cplx *in, cplx *out, size_t n, int sign)
{
    if (n == 0) return 0;
    const cplx *tw = get_twiddles(n);
    if (!tw) return 3;
    /* the generic radix-p combine needs 2p scratch slots; p <= n */
    cplx *tmp = (cplx *)malloc(sizeof(cplx) * (2 * n + 64));
    if (!tmp) return 3;
    dft_rec(in, 1, out, n, tw, n, sign, tmp);
    free(tmp);
    return 0;
}

int oracle_c2c_1d(double *data, size_t n, int sign)
{
    if (n == 0) return 0;
    cplx *in = (cplx *)malloc(sizeof(cplx) * n);
    if (!in) return 3;
    memcpy(in, data, sizeof(cplx) * n);
    int rc = c2c_into(in, (cplx *)data, n, sign);
    free(in);
    return rc;
}

/* r2c via the half-length complex transform:
 *   z[m] = x[2m] + i x[2m+1], Z = DFT_M(z), M = n/2,
 *   X[k] = (Z[k] + conj Z[M-k])/2 - (i/2) W_n^k (Z[k] - conj Z[M-k]),  k = 0..M. */
int oracle_r2c_1d(const double *in, double *out, size_t n)
{
    if (n == 0 || n % 2) return 2;
    size_t M = n / 2;
    cplx *z = (cplx *)malloc(sizeof(cplx) * M);
    cplx *Z = (cplx *)malloc(sizeof(cplx) * M);
    if (!z || !Z) {
        free(z);
        free(Z);
        return 3;
    }
    memcpy(z, in, sizeof(double) * n);
    int rc = c2c_into(z, Z, M, -1);
    const cplx *twn = get_twiddles(n);
    if (rc == 0 && !twn) rc = 3;
    if (rc == 0) {
        cplx *X = (cplx *)out;
        for (size_t k = 0; k <= M; ++k) {
            cplx a = Z[k % M];
            cplx b = Z[(M - k) % M];
            b.im = -b.im; /* conj Z[M-k] */
            cplx e = {0.5 * (a.re + b.re), 0.5 * (a.im + b.im)};
            cplx o = {0.5 * (a.re - b.re), 0.5 * (a.im - b.im)};
            cplx w = twn[k % n];
            cplx wo = cmul(w, o);
            /* -i * wo = (wo.im, -wo.re) */
            X[k].re = e.re + wo.im;
            X[k].im = e.im - wo.re;
        }
    }
    free(z);
    free(Z);
    return rc;
}

/* unnormalised c2r of n/2+1 complex into n reals (in may alias out) */
static int c2r_1d(const double *in, double *out, size_t n)
{
    if (n == 0 || n % 2) return 2;
    size_t M = n / 2;
    cplx *X = (cplx *)malloc(sizeof(cplx) * (M + 1));
    cplx *Z = (cplx *)malloc(sizeof(cplx) * M);
    if (!X || !Z) {
        free(X);
        free(Z);
        return 3;
    }
    memcpy(X, in, sizeof(cplx) * (M + 1));
    X[0].im = 0.0;
    X[M].im = 0.0;
    const cplx *twn = get_twiddles(n);
    if (!twn) {
        free(X);
        free(Z);
        return 3;
    }
    for (size_t k = 0; k < M; ++k) {
        cplx a = X[k];
        cplx b = X[M - k];
        b.im = -b.im;
        cplx s = {a.re + b.re, a.im + b.im};
        cplx d = {a.re - b.re, a.im - b.im};
        cplx w = twn[k];
        w.im = -w.im; /* W_n^{-k} */
        cplx wd = cmul(w, d);
        /* + i * wd = (-wd.im, wd.re) */
        Z[k].re = s.re - wd.im;
        Z[k].im = s.im + wd.re;
    }
    int rc = c2c_into(Z, (cplx *)out, M, +1);
    free(X);
    free(Z);
    return rc;
}

/* ------------------------------------------------------------------ */
/* parallel for over [0, n) (the reference's for_loop(par))             */
/* ------------------------------------------------------------------ */
typedef void (*body_fn)(void *ctx, size_t i);
typedef struct {
    body_fn fn;
    void *ctx;
    size_t lo, hi;
} chunk_t;

static void *run_chunk(void *arg)
{
    chunk_t *c = (chunk_t *)arg;
    for (size_t i = c->lo; i < c->hi; ++i) c->fn(c->ctx, i);
    return NULL;
}

static void parallel_for(size_t n, int nthreads, body_fn fn, void *ctx)
{
    if (nthreads <= 1 || n < 2) {
        for (size_t i = 0; i < n; ++i) fn(ctx, i);
        return;
    }
    if ((size_t)nthreads > n) nthreads = (int)n;
    pthread_t th[256];
    chunk_t ch[256];
    int joined[256];
    if (nthreads > 256) nthreads = 256;
    size_t per = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        ch[t].fn = fn;
        ch[t].ctx = ctx;
        ch[t].lo = (size_t)t * per < n ? (size_t)t * per : n;
        ch[t].hi = ch[t].lo + per < n ? ch[t].lo + per : n;
        joined[t] = 0;
        if (t == 0 || ch[t].lo >= ch[t].hi) continue; /* chunk 0 runs on the caller */
        if (pthread_create(&th[t], NULL, run_chunk, &ch[t]) == 0)
            joined[t] = 1;
        else
            run_chunk(&ch[t]);
    }
    run_chunk(&ch[0]);
    for (int t = 1; t < nthreads; ++t)
        if (joined[t]) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* 2D r2c: the four phases of core/src/shared/loop.cpp:56-113           */
/* ------------------------------------------------------------------ */
typedef struct {
    double *values;     /* values_vec_: dim_c_x x 2*dim_c_y */
    double *trans;      /* trans_values_vec_: dim_c_y x 2*dim_c_x */
    size_t dim_c_x, dim_c_y, dim_r_y;
    int status;
    int sign;
} loop_ctx;

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* fft_1d_r2c_inplace, core/src/shared/loop.cpp:6-9 */
static void body_r2c(void *p, size_t i)
{
    loop_ctx *c = (loop_ctx *)p;
    double *row = c->values + i * 2 * c->dim_c_y;
    if (oracle_r2c_1d(row, row, c->dim_r_y) != 0) c->status = 3;
}

/* transpose_shared_y_to_x, core/src/shared/loop.cpp:18-25 */
static void body_trans_y_to_x(void *p, size_t index)
{
    loop_ctx *c = (loop_ctx *)p;
    const size_t ncv = 2 * c->dim_c_y, nct = 2 * c->dim_c_x;
    for (size_t t = 0; t < c->dim_c_x; ++t) {
        c->trans[index * nct + 2 * t] = c->values[t * ncv + 2 * index];
        c->trans[index * nct + 2 * t + 1] = c->values[t * ncv + 2 * index + 1];
    }
}

/* fft_1d_c2c_inplace, core/src/shared/loop.cpp:11-15 */
static void body_c2c(void *p, size_t i)
{
    loop_ctx *c = (loop_ctx *)p;
    if (oracle_c2c_1d(c->trans + i * 2 * c->dim_c_x, c->dim_c_x, c->sign) != 0) c->status = 3;
}

/* transpose_shared_x_to_y, core/src/shared/loop.cpp:46-53 */
static void body_trans_x_to_y(void *p, size_t index_trans)
{
    loop_ctx *c = (loop_ctx *)p;
    const size_t ncv = 2 * c->dim_c_y, nct = 2 * c->dim_c_x;
    for (size_t index = 0; index < c->dim_c_x; ++index) {
        c->values[index * ncv + 2 * index_trans] = c->trans[index_trans * nct + 2 * index];
        c->values[index * ncv + 2 * index_trans + 1] = c->trans[index_trans * nct + 2 * index + 1];
    }
}

static int check_dims(size_t n_row, size_t n_col)
{
    if (n_row == 0 || n_col < 4 || n_col % 2) return 1;
    return 0;
}

int oracle_fft_2d_r2c(double *values, size_t n_row, size_t n_col, int nthreads, double *times)
{
    if (!values || check_dims(n_row, n_col)) return 1;
    loop_ctx c;
    c.values = values;
    c.dim_c_x = n_row;           /* loop.cpp:163 */
    c.dim_c_y = n_col / 2;       /* loop.cpp:164 */
    c.dim_r_y = 2 * c.dim_c_y - 2; /* loop.cpp:165 */
    c.status = 0;
    c.sign = -1;
    c.trans = (double *)malloc(sizeof(double) * c.dim_c_y * 2 * c.dim_c_x); /* loop.cpp:167 */
    if (!c.trans) return 3;
    double t0 = now_s();
    parallel_for(c.dim_c_x, nthreads, body_r2c, &c);
    double t1 = now_s();
    parallel_for(c.dim_c_y, nthreads, body_trans_y_to_x, &c);
    double t2 = now_s();
    parallel_for(c.dim_c_y, nthreads, body_c2c, &c);
    double t3 = now_s();
    parallel_for(c.dim_c_y, nthreads, body_trans_x_to_y, &c);
    double t4 = now_s();
    free(c.trans);
    if (times) {
        times[0] = t4 - t0;
        times[1] = t1 - t0;
        times[2] = t2 - t1;
        times[3] = t3 - t2;
        times[4] = t4 - t3;
    }
    return c.status;
}

/* ------------------------------------------------------------------ */
/* c2r and the adjoint (no reference counterpart; checker for the      */
/* backward kernels)                                                   */
/* ------------------------------------------------------------------ */
static void body_c2r(void *p, size_t i)
{
    loop_ctx *c = (loop_ctx *)p;
    double *row = c->values + i * 2 * c->dim_c_y;
    if (c2r_1d(row, row, c->dim_r_y) != 0) c->status = 3;
    row[c->dim_r_y] = 0.0;
    row[c->dim_r_y + 1] = 0.0;
}

static int inverse_columns_then_rows(double *values, size_t n_row, size_t n_col, int nthreads)
{
    loop_ctx c;
    c.values = values;
    c.dim_c_x = n_row;
    c.dim_c_y = n_col / 2;
    c.dim_r_y = 2 * c.dim_c_y - 2;
    c.status = 0;
    c.sign = +1;
    c.trans = (double *)malloc(sizeof(double) * c.dim_c_y * 2 * c.dim_c_x);
    if (!c.trans) return 3;
    parallel_for(c.dim_c_y, nthreads, body_trans_y_to_x, &c);
    parallel_for(c.dim_c_y, nthreads, body_c2c, &c);
    parallel_for(c.dim_c_y, nthreads, body_trans_x_to_y, &c);
    free(c.trans);
    parallel_for(c.dim_c_x, nthreads, body_c2r, &c);
    return c.status;
}

int oracle_fft_2d_c2r(double *values, size_t n_row, size_t n_col, int nthreads)
{
    if (!values || check_dims(n_row, n_col)) return 1;
    return inverse_columns_then_rows(values, n_row, n_col, nthreads);
}

int oracle_fft_2d_r2c_adjoint(double *values, size_t n_row, size_t n_col, int nthreads)
{
    if (!values || check_dims(n_row, n_col)) return 1;
    const size_t dcy = n_col / 2;
    /* half weights on the interior bins: a c2r counts them twice */
    for (size_t i = 0; i < n_row; ++i)
        for (size_t k = 1; k + 1 < dcy; ++k) {
            values[i * n_col + 2 * k] *= 0.5;
            values[i * n_col + 2 * k + 1] *= 0.5;
        }
    return inverse_columns_then_rows(values, n_row, n_col, nthreads);
}
