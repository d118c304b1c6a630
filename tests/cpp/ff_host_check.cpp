// Host build of the float-float conversions and arithmetic (ff.cuh) for CPU
// unit tests: the same source the kernels use, compiled by g++.
#include <cstddef>

#include "../../hpx-fft_gb300/csrc/ff.cuh"

using hpxfft_gpu::ff;

extern "C" {
// x -> pair (scale 2^-E) -> double (scale 2^E)
void ff_roundtrip(const double *x, double *y, size_t n, int E)
{
    for (size_t i = 0; i < n; ++i) y[i] = hpxfft_gpu::ff_to_double(hpxfft_gpu::renorm(hpxfft_gpu::ff_from_double(x[i], E)), E);
}
// split only: hi, lo as floats
void ff_split(const double *x, float *hi, float *lo, size_t n, int E)
{
    for (size_t i = 0; i < n; ++i) {
        ff v = hpxfft_gpu::ff_from_double(x[i], E);
        hi[i] = v.hi;
        lo[i] = v.lo;
    }
}
// a op b in float-float, result back to double (op: 0 add, 1 sub, 2 mul)
void ff_binop(const double *a, const double *b, double *y, size_t n, int op)
{
    for (size_t i = 0; i < n; ++i) {
        ff x = hpxfft_gpu::ff_from_double(a[i], 0), z = hpxfft_gpu::ff_from_double(b[i], 0), r;
        if (op == 0) r = x + z;
        else if (op == 1) r = x - z;
        else r = x * z;
        y[i] = hpxfft_gpu::ff_to_double(hpxfft_gpu::renorm(r), 0);
    }
}
int dbl_exp(double x) { return hpxfft_gpu::dbl_biased_exp(x); }
// renormalised pair (hi, lo) -> double with scale 2^E
void ff_pair_to_double(const float *hi, const float *lo, double *y, size_t n, int E)
{
    for (size_t i = 0; i < n; ++i) y[i] = hpxfft_gpu::ff_to_double(hpxfft_gpu::renorm(ff{hi[i], lo[i]}), E);
}
}
