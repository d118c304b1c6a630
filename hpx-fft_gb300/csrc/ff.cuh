// Float-float ("double-float") arithmetic for the FP64 drop-in path.
//
// A GB300 SM retires 58x more FP32 FMAs than FP64 FMAs (measured: 69.5 vs
// 1.19 TFLOP/s), so the FP64 transform keeps its data in HBM as IEEE doubles
// but computes on the FP32 pipes with an unevaluated pair hi + lo of floats
// (about 48 significant bits).  The error-free transformations are Knuth's
// two-sum and the FMA-based two-product; the pair is renormalised with
// Dekker's fast-two-sum once per butterfly pass.
//
// Conversions double <-> pair use integer bit manipulation only, so no
// instruction of the data path runs on the slow FP64 pipe.  A per-transform
// power-of-two scale 2^E keeps the pair inside the float exponent range.
#pragma once
#include <cstdint>
#include <cstring>

#ifndef HPXFFT_HD
#ifdef __CUDACC__
#define HPXFFT_HD __host__ __device__ __forceinline__
#else
#define HPXFFT_HD inline  // host-only builds (unit tests of the conversions)
#endif
#endif
#include <cmath>

namespace hpxfft_gpu {

struct ff {
    float hi, lo;
};

HPXFFT_HD uint64_t dbl_bits(double x)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
#endif
}
HPXFFT_HD double bits_dbl(uint64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    std::memcpy(&x, &b, 8);
    return x;
#endif
}
HPXFFT_HD uint32_t flt_bits(float x)
{
#ifdef __CUDA_ARCH__
    return (uint32_t)__float_as_uint(x);
#else
    uint32_t b;
    std::memcpy(&b, &x, 4);
    return b;
#endif
}
HPXFFT_HD float bits_flt(uint32_t b)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float x;
    std::memcpy(&x, &b, 4);
    return x;
#endif
}

// round-to-nearest primitives that the compiler may not contract or reorder
HPXFFT_HD float fadd(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;
    return r;
#endif
}
HPXFFT_HD float fsub(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    volatile float r = a - b;
    return r;
#endif
}
HPXFFT_HD float fmul(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    volatile float r = a * b;
    return r;
#endif
}
HPXFFT_HD float ffma(float a, float b, float c)
{
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

// s + e == a + b exactly (Knuth)
HPXFFT_HD void two_sum(float a, float b, float &s, float &e)
{
    s = fadd(a, b);
    float bb = fsub(s, a);
    e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
}

// h + l == s + e exactly when |s| >= |e| (Dekker)
HPXFFT_HD ff renorm(ff x)
{
    ff r;
    r.hi = fadd(x.hi, x.lo);
    r.lo = fsub(x.lo, fsub(r.hi, x.hi));
    return r;
}

// unnormalised sum: hi part is the rounded sum of the hi parts, lo collects
// its exact rounding error and both lo parts
HPXFFT_HD ff operator+(ff a, ff b)
{
    ff r;
    float e;
    two_sum(a.hi, b.hi, r.hi, e);
    r.lo = fadd(e, fadd(a.lo, b.lo));
    return r;
}
HPXFFT_HD ff operator-(ff a)
{
    ff r = {-a.hi, -a.lo};
    return r;
}
HPXFFT_HD ff operator-(ff a, ff b) { return a + (-b); }

// product: exact hi*hi via FMA, first-order cross terms, lo*lo dropped
HPXFFT_HD ff operator*(ff a, ff b)
{
    ff r;
    r.hi = fmul(a.hi, b.hi);
    float e = ffma(a.hi, b.hi, -r.hi);
    e = ffma(a.hi, b.lo, e);
    r.lo = ffma(a.lo, b.hi, e);
    return r;
}

HPXFFT_HD ff ff_scale_pow2(ff a, float p2)  // exact for powers of two
{
    ff r = {a.hi * p2, a.lo * p2};
    return r;
}

// ------------------------------------------------------------------------
// double <-> pair conversions (integer pipe only)
// ------------------------------------------------------------------------

// Biased exponent field of a double (0 for zero / subnormal, 2047 inf/nan).
HPXFFT_HD int dbl_biased_exp(double x) { return (int)((dbl_bits(x) >> 52) & 0x7ff); }

// x * 2^-E as hi + lo.  hi takes the top 24 significant bits of x (truncated),
// lo the next 29 bits rounded to 24.  Values whose scaled magnitude falls
// below the float normal range are flushed to zero: with E the exponent of
// the transform's largest input they are < 2^-126 of it.
HPXFFT_HD ff ff_from_double_int(double x, int E)
{
    const uint64_t b = dbl_bits(x);
    const uint32_t hi32 = (uint32_t)(b >> 32);
    const uint32_t lo32 = (uint32_t)b;
    const uint32_t sign = hi32 & 0x80000000u;
    const int e = (int)((hi32 >> 20) & 0x7ff);
    const int fe = e - 1023 + 127 - E;
    ff r;
    if (e == 0x7ff) {  // inf / nan propagate
        r.hi = bits_flt(sign | 0x7f800000u | ((hi32 & 0xfffff) ? 0x400000u : 0u));
        r.lo = 0.0f;
        return r;
    }
    if (e == 0 || fe <= 0) {
        r.hi = bits_flt(sign);
        r.lo = bits_flt(sign);
        return r;
    }
    if (fe >= 255) {  // cannot happen with E = max exponent of the block
        r.hi = bits_flt(sign | 0x7f800000u);
        r.lo = 0.0f;
        return r;
    }
    const uint32_t top23 = ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
    r.hi = bits_flt(sign | ((uint32_t)fe << 23) | top23);
    const uint32_t rest29 = lo32 & 0x1fffffffu;
    // rest29 is in units of 2^(fe - 127 - 52)
    const int se = fe - 52;
    if (se >= 1 && rest29) {
        float mag = (float)rest29 * bits_flt((uint32_t)se << 23);
        r.lo = sign ? -mag : mag;
    } else {
        r.lo = bits_flt(sign);
    }
    return r;
}

// The same for the common case (scaled exponent well inside the float range,
// not inf / nan / zero / subnormal): hi from the top bits by a funnel shift,
// lo = (next 29 bits, converted and rounded to 24) * 2^(fe - 179).
HPXFFT_HD ff ff_from_double(double x, int E)
{
    const uint64_t b = dbl_bits(x);
    const uint32_t hi32 = (uint32_t)(b >> 32);
    const uint32_t lo32 = (uint32_t)b;
    const int e = (int)((hi32 >> 20) & 0x7ff);
    const int fe = e - 1023 + 127 - E;
    if (e == 0 || e == 0x7ff || fe < 60 || fe > 254) return ff_from_double_int(x, E);
    const uint32_t sign = hi32 & 0x80000000u;
    const uint32_t top23 = (uint32_t)(b >> 29) & 0x7fffffu;
    ff r;
    r.hi = bits_flt(sign | ((uint32_t)fe << 23) | top23);
    const float mag = (float)(lo32 & 0x1fffffffu) * bits_flt((uint32_t)(fe - 52) << 23);
    r.lo = bits_flt(flt_bits(mag) ^ sign);
    return r;
}

// (hi + lo) * 2^E as a double, integer operations only.  The pair must be renormalised
// (|lo| <= ulp(hi) / 2).  In units u = ulp(hi) / 2^29 the hi significand is
// H = (2^23 + m_hi) 2^29 in [2^52, 2^53) and |lo| <= 2^28 u, so lo fits a
// 32-bit integer (rounded to u: error <= 2^-53 relative) and H +- lo needs
// at most one left shift to be normalised again.
HPXFFT_HD double ff_to_double_int(ff v, int E)
{
    const uint32_t hb = flt_bits(v.hi);
    const int fe = (int)((hb >> 23) & 0xff);
    const uint64_t sign = (uint64_t)(hb >> 31) << 63;
    if (fe == 0 || fe == 0xff) {
        if (fe == 0xff)  // inf / nan
            return bits_dbl(sign | 0x7ff0000000000000ull | ((hb & 0x7fffffu) ? 0x8000000000000ull : 0ull));
        // zero or float subnormal: tiny relative to the block; value from hi only
        if ((hb & 0x7fffffu) == 0) return bits_dbl(sign);
        const double m = (double)(hb & 0x7fffffu);
        double r = m * bits_dbl((uint64_t)(1023 - 149 + E > 0 ? 1023 - 149 + E : 1) << 52);
        return (hb >> 31) ? -r : r;
    }
    const uint32_t lb = flt_bits(v.lo);
    const int le = (int)((lb >> 23) & 0xff);
    const uint32_t ml = (lb & 0x7fffffu) | 0x800000u;
    const int sh = le - fe + 29;  // lo = ml 2^sh u, sh <= 5
    uint32_t L = 0;
    if (le != 0 && le != 0xff) L = sh >= 0 ? ml << sh : (sh > -25 ? (ml + (1u << (-sh - 1))) >> -sh : 0u);
    uint64_t H = (uint64_t)((hb & 0x7fffffu) | 0x800000u) << 29;
    H = ((hb ^ lb) >> 31) ? H - L : H + L;
    int de = fe - 127 + 1023 + E;
    if (H < (1ull << 52)) {  // hi a power of two, lo of the other sign
        H <<= 1;
        --de;
    }
    if (de <= 0) return bits_dbl(sign);  // below the double normal range
    if (de >= 2047) return bits_dbl(sign | 0x7ff0000000000000ull);
    return bits_dbl(sign | ((uint64_t)de << 52) | (H & 0xfffffffffffffull));
}

HPXFFT_HD int f2i_rn(float x)
{
#ifdef __CUDA_ARCH__
    return __float2int_rn(x);
#else
    return (int)std::lrintf(x);
#endif
}

// The same, with the float unit doing the alignment: lo, with the sign of hi
// folded in, times 2^(179 - fe) is |lo| in units u = 2^(fe - 179) (exact:
// a power-of-two scale), rounded to an integer (|L| <= 2^28); then one 64-bit
// add onto the hi significand.  Exponents near the ends of the float or
// double range take the integer path.
HPXFFT_HD double ff_to_double(ff v, int E)
{
    const uint32_t hb = flt_bits(v.hi);
    const int fe = (int)((hb >> 23) & 0xff);
    const int de = fe - 127 + 1023 + E;
    if (fe < 60 || fe == 0xff || de < 2 || de > 2045) return ff_to_double_int(v, E);
    const float lo_rel = bits_flt(flt_bits(v.lo) ^ (hb & 0x80000000u));
    const int L = f2i_rn(lo_rel * bits_flt((uint32_t)(306 - fe) << 23));
    const uint64_t H = ((uint64_t)((hb & 0x7fffffu) | 0x800000u) << 29) + (uint64_t)(int64_t)L;
    uint64_t bits;
    if (H >> 52)
        bits = ((uint64_t)de << 52) | (H & 0xfffffffffffffull);
    else  // hi a power of two, lo of the other sign: one bit lower
        bits = ((uint64_t)(de - 1) << 52) | ((H << 1) & 0xfffffffffffffull);
    return bits_dbl(((uint64_t)(hb >> 31) << 63) | bits);
}

}  // namespace hpxfft_gpu
