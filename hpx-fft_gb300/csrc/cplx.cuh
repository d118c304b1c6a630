// Complex arithmetic and compile-time DFT butterflies, written once for the
// three compute types of the transform: float (FP32 path), double (native
// FP64, kept for cross-checks) and ff (float-float, the FP64 drop-in).
#pragma once
#include <type_traits>

#include "ff.cuh"

namespace hpxfft_gpu {

template <class T>
struct cpx {
    T re, im;
};

// --------------------------------------------------------------- real helpers
template <class T>
struct real_ops;

template <>
struct real_ops<float> {
    static constexpr HPXFFT_HD float cst(double c) { return (float)c; }
    static HPXFFT_HD float norm(float x) { return x; }
    static HPXFFT_HD float zero() { return 0.0f; }
};
template <>
struct real_ops<double> {
    static constexpr HPXFFT_HD double cst(double c) { return c; }
    static HPXFFT_HD double norm(double x) { return x; }
    static HPXFFT_HD double zero() { return 0.0; }
};
template <>
struct real_ops<ff> {
    // evaluated at compile time: every call site binds it to a constexpr
    static constexpr HPXFFT_HD ff cst(double c) { return ff{(float)c, (float)(c - (double)(float)c)}; }
    static HPXFFT_HD ff norm(ff x) { return renorm(x); }
    static HPXFFT_HD ff zero()
    {
        ff r = {0.0f, 0.0f};
        return r;
    }
};

// ------------------------------------------------------------ complex helpers
template <class T>
HPXFFT_HD cpx<T> operator+(cpx<T> a, cpx<T> b)
{
    return cpx<T>{a.re + b.re, a.im + b.im};
}
template <class T>
HPXFFT_HD cpx<T> operator-(cpx<T> a, cpx<T> b)
{
    return cpx<T>{a.re - b.re, a.im - b.im};
}
template <class T>
HPXFFT_HD cpx<T> cmul(cpx<T> a, cpx<T> b)
{
    return cpx<T>{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class T>
HPXFFT_HD cpx<T> cconj(cpx<T> a)
{
    return cpx<T>{a.re, -a.im};
}
template <class T>
HPXFFT_HD cpx<T> cnorm(cpx<T> a)
{
    return cpx<T>{real_ops<T>::norm(a.re), real_ops<T>::norm(a.im)};
}
template <class T>
HPXFFT_HD cpx<T> czero()
{
    return cpx<T>{real_ops<T>::zero(), real_ops<T>::zero()};
}
// a / 2, exact in every compute type
template <class T>
HPXFFT_HD cpx<T> chalf(cpx<T> a)
{
    if constexpr (std::is_same<T, ff>::value)
        return cpx<T>{ff_scale_pow2(a.re, 0.5f), ff_scale_pow2(a.im, 0.5f)};
    else
        return cpx<T>{a.re * (T)0.5, a.im * (T)0.5};
}
// a * (DIR * i): DIR = -1 multiplies by -i (forward), +1 by +i (inverse)
template <int DIR, class T>
HPXFFT_HD cpx<T> mul_i(cpx<T> a)
{
    if constexpr (DIR < 0)
        return cpx<T>{a.im, -a.re};
    else
        return cpx<T>{-a.im, a.re};
}

// cos(2 pi m / 16) and sin(2 pi m / 16), m = 0..15
constexpr double kCos16[16] = {1.0,
                               0.92387953251128673848,
                               0.70710678118654752440,
                               0.38268343236508977173,
                               0.0,
                               -0.38268343236508977173,
                               -0.70710678118654752440,
                               -0.92387953251128673848,
                               -1.0,
                               -0.92387953251128673848,
                               -0.70710678118654752440,
                               -0.38268343236508977173,
                               0.0,
                               0.38268343236508977173,
                               0.70710678118654752440,
                               0.92387953251128673848};
constexpr double kSin16[16] = {0.0,
                               0.38268343236508977173,
                               0.70710678118654752440,
                               0.92387953251128673848,
                               1.0,
                               0.92387953251128673848,
                               0.70710678118654752440,
                               0.38268343236508977173,
                               0.0,
                               -0.38268343236508977173,
                               -0.70710678118654752440,
                               -0.92387953251128673848,
                               -1.0,
                               -0.92387953251128673848,
                               -0.70710678118654752440,
                               -0.38268343236508977173};

// a * W16^m with W16 = exp(DIR * 2 pi i / 16)
template <int M, int DIR, class T>
HPXFFT_HD cpx<T> mul_w16(cpx<T> a)
{
    constexpr int m = ((M % 16) + 16) % 16;
    if constexpr (m == 0) {
        return a;
    } else if constexpr (m == 4) {
        return mul_i<DIR>(a);
    } else if constexpr (m == 8) {
        return cpx<T>{-a.re, -a.im};
    } else if constexpr (m == 12) {
        return mul_i<-DIR>(a);
    } else if constexpr (m == 2 || m == 6 || m == 10 || m == 14) {
        // (+-1 +- i) / sqrt 2: two adds and two constant products
        constexpr T r = real_ops<T>::cst(0.70710678118654752440);
        constexpr double c = kCos16[m];
        constexpr double s = DIR * kSin16[m];
        // a * (c + i s) with |c| = |s| = r
        T re, im;
        if constexpr ((c > 0) == (s > 0)) {
            // c = s: (x + iy)(1 + i) r  or  (x + iy)(-1 - i) r
            re = a.re - a.im;
            im = a.re + a.im;
        } else {
            // c = -s: (x + iy)(1 - i) r  or  (x + iy)(-1 + i) r
            re = a.re + a.im;
            im = a.im - a.re;
        }
        if constexpr (c > 0)
            return cpx<T>{re * r, im * r};
        else
            return cpx<T>{-(re * r), -(im * r)};
    } else {
        constexpr cpx<T> w = {real_ops<T>::cst(kCos16[m]), real_ops<T>::cst(DIR * kSin16[m])};
        return cmul(a, w);
    }
}

// -------------------------------------------------------------- butterflies
// In place: v[t] <- sum_q v[q] exp(DIR 2 pi i q t / R), natural order.
template <int R, int DIR, class T>
struct DFT;

template <int DIR, class T>
struct DFT<1, DIR, T> {
    static HPXFFT_HD void run(cpx<T> *) {}
};

template <int DIR, class T>
struct DFT<2, DIR, T> {
    static HPXFFT_HD void run(cpx<T> *v)
    {
        cpx<T> a = v[0], b = v[1];
        v[0] = a + b;
        v[1] = a - b;
    }
};

template <int DIR, class T>
HPXFFT_HD void dft4(cpx<T> &x0, cpx<T> &x1, cpx<T> &x2, cpx<T> &x3)
{
    cpx<T> s0 = x0 + x2, d0 = x0 - x2;
    cpx<T> s1 = x1 + x3, d1 = mul_i<DIR>(x1 - x3);
    x0 = s0 + s1;
    x2 = s0 - s1;
    x1 = d0 + d1;
    x3 = d0 - d1;
}

template <int DIR, class T>
struct DFT<4, DIR, T> {
    static HPXFFT_HD void run(cpx<T> *v) { dft4<DIR>(v[0], v[1], v[2], v[3]); }
};

template <int DIR, class T>
struct DFT<8, DIR, T> {
    static HPXFFT_HD void run(cpx<T> *v)
    {
        // even / odd halves, then radix-2 combine with W8^k = W16^(2k)
        cpx<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
        cpx<T> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
        dft4<DIR>(e0, e1, e2, e3);
        dft4<DIR>(o0, o1, o2, o3);
        o1 = mul_w16<2, DIR>(o1);
        o2 = mul_w16<4, DIR>(o2);
        o3 = mul_w16<6, DIR>(o3);
        v[0] = e0 + o0;
        v[4] = e0 - o0;
        v[1] = e1 + o1;
        v[5] = e1 - o1;
        v[2] = e2 + o2;
        v[6] = e2 - o2;
        v[3] = e3 + o3;
        v[7] = e3 - o3;
    }
};

template <int DIR, class T>
struct DFT<16, DIR, T> {
    static HPXFFT_HD void run(cpx<T> *v)
    {
        // n = q + 4 n2, k = t1 + 4 t2:  X[t1 + 4 t2] = sum_q W4^{q t2} W16^{q t1} A_q[t1]
        dft4<DIR>(v[0], v[4], v[8], v[12]);
        dft4<DIR>(v[1], v[5], v[9], v[13]);
        dft4<DIR>(v[2], v[6], v[10], v[14]);
        dft4<DIR>(v[3], v[7], v[11], v[15]);
        // A_q[t1] sits at v[q + 4 t1]
        v[5] = mul_w16<1, DIR>(v[5]);
        v[9] = mul_w16<2, DIR>(v[9]);
        v[13] = mul_w16<3, DIR>(v[13]);
        v[6] = mul_w16<2, DIR>(v[6]);
        v[10] = mul_w16<4, DIR>(v[10]);
        v[14] = mul_w16<6, DIR>(v[14]);
        v[7] = mul_w16<3, DIR>(v[7]);
        v[11] = mul_w16<6, DIR>(v[11]);
        v[15] = mul_w16<9, DIR>(v[15]);
        // DFT4 over q for each t1; result t2 lands in v[q = t2 + 4 t1] -> X[t1 + 4 t2]
        dft4<DIR>(v[0], v[1], v[2], v[3]);
        dft4<DIR>(v[4], v[5], v[6], v[7]);
        dft4<DIR>(v[8], v[9], v[10], v[11]);
        dft4<DIR>(v[12], v[13], v[14], v[15]);
        // transpose the 4x4 index grid: v[t2 + 4 t1] holds X[t1 + 4 t2]
        cpx<T> t;
        t = v[1], v[1] = v[4], v[4] = t;
        t = v[2], v[2] = v[8], v[8] = t;
        t = v[3], v[3] = v[12], v[12] = t;
        t = v[6], v[6] = v[9], v[9] = t;
        t = v[7], v[7] = v[13], v[13] = t;
        t = v[11], v[11] = v[14], v[14] = t;
    }
};

template <int DIR, class T>
struct DFT<3, DIR, T> {
    static HPXFFT_HD void run(cpx<T> *v)
    {
        constexpr T h = real_ops<T>::cst(0.5);
        constexpr T s = real_ops<T>::cst(0.86602540378443864676);  // sin(2 pi / 3)
        cpx<T> t = v[1] + v[2];
        cpx<T> d = v[1] - v[2];
        cpx<T> m = cpx<T>{v[0].re - t.re * h, v[0].im - t.im * h};
        cpx<T> j = mul_i<DIR>(cpx<T>{d.re * s, d.im * s});
        v[0] = v[0] + t;
        v[1] = m + j;
        v[2] = m - j;
    }
};

template <int DIR, class T>
struct DFT<5, DIR, T> {
    static HPXFFT_HD void run(cpx<T> *v)
    {
        constexpr T c1 = real_ops<T>::cst(0.30901699437494742410);   // cos(2 pi / 5)
        constexpr T c2 = real_ops<T>::cst(-0.80901699437494742410);  // cos(4 pi / 5)
        constexpr T s1 = real_ops<T>::cst(0.95105651629515357212);   // sin(2 pi / 5)
        constexpr T s2 = real_ops<T>::cst(0.58778525229247312917);   // sin(4 pi / 5)
        cpx<T> t1 = v[1] + v[4], t2 = v[2] + v[3];
        cpx<T> d1 = v[1] - v[4], d2 = v[2] - v[3];
        cpx<T> a1 = cpx<T>{v[0].re + t1.re * c1 + t2.re * c2, v[0].im + t1.im * c1 + t2.im * c2};
        cpx<T> a2 = cpx<T>{v[0].re + t1.re * c2 + t2.re * c1, v[0].im + t1.im * c2 + t2.im * c1};
        cpx<T> b1 = cpx<T>{d1.re * s1 + d2.re * s2, d1.im * s1 + d2.im * s2};
        cpx<T> b2 = cpx<T>{d1.re * s2 - d2.re * s1, d1.im * s2 - d2.im * s1};
        // forward: X1 = a1 - i b1; inverse: X1 = a1 + i b1
        cpx<T> jb1 = mul_i<DIR>(b1), jb2 = mul_i<DIR>(b2);
        v[0] = v[0] + t1 + t2;
        v[1] = a1 + jb1;
        v[4] = a1 - jb1;
        v[2] = a2 + jb2;
        v[3] = a2 - jb2;
    }
};

// ------------------------------------------------------ odd prime radices
#ifdef __CUDACC__
#define HPXFFT_CONSTEXPR_HD constexpr __host__ __device__
#else
#define HPXFFT_CONSTEXPR_HD constexpr
#endif
// Compile-time cos / sin (Taylor series after reduction to |x| <= pi/4) so
// the constants of the length-7, 11 and 13 butterflies are literals.
constexpr long double kPiL = 3.141592653589793238462643383279502884L;
HPXFFT_CONSTEXPR_HD long double taylor_sin(long double x)
{
    long double term = x, sum = x;
    for (int k = 1; k < 16; ++k) {
        term *= -x * x / ((2 * k) * (2 * k + 1));
        sum += term;
    }
    return sum;
}
HPXFFT_CONSTEXPR_HD long double taylor_cos(long double x)
{
    long double term = 1, sum = 1;
    for (int k = 1; k < 16; ++k) {
        term *= -x * x / ((2 * k - 1) * (2 * k));
        sum += term;
    }
    return sum;
}
// cos and sin of 2 pi m / n
HPXFFT_CONSTEXPR_HD double cos2pi(int m, int n)
{
    m = ((m % n) + n) % n;
    // octant reduction of the angle 2 pi m / n
    const long double a = 2 * kPiL * (long double)m / (long double)n;
    if (8 * m <= n) return (double)taylor_cos(a);
    if (8 * m <= 3 * n) return (double)taylor_sin(kPiL / 2 - a);
    if (8 * m <= 5 * n) return (double)(-taylor_cos(kPiL - a));
    if (8 * m <= 7 * n) return (double)taylor_sin(a - 3 * kPiL / 2);
    return (double)taylor_cos(2 * kPiL - a);
}
HPXFFT_CONSTEXPR_HD double sin2pi(int m, int n) { return cos2pi(4 * m - n, 4 * n); }  // sin(x) = cos(x - pi/2)

// Constants of an odd-length butterfly, split into the compute type at
// compile time: c[q][t] = cos(2 pi (q+1)(t+1) / R), s likewise.
template <int R, class T>
struct OddConsts {
    T c[(R - 1) / 2][(R - 1) / 2];
    T s[(R - 1) / 2][(R - 1) / 2];
};
template <int R, class T>
HPXFFT_CONSTEXPR_HD OddConsts<R, T> make_odd_consts()
{
    OddConsts<R, T> k{};
    for (int q = 0; q < (R - 1) / 2; ++q)
        for (int t = 0; t < (R - 1) / 2; ++t) {
            k.c[q][t] = real_ops<T>::cst(cos2pi((q + 1) * (t + 1), R));
            k.s[q][t] = real_ops<T>::cst(sin2pi((q + 1) * (t + 1), R));
        }
    return k;
}

// Odd length R: pairs q, R-q share the real and imaginary sums
//   X_t     = v0 + sum_q (v_q + v_{R-q}) cos(2 pi q t / R) + DIR i sum_q (v_q - v_{R-q}) sin(2 pi q t / R)
//   X_{R-t} = same with the sine term negated.
template <int R, int DIR, class T>
struct DFTOdd {
    static HPXFFT_HD void run(cpx<T> *v)
    {
        constexpr int H = (R - 1) / 2;
        constexpr OddConsts<R, T> K = make_odd_consts<R, T>();
        cpx<T> a[H], b[H];
#pragma unroll
        for (int q = 1; q <= H; ++q) {
            a[q - 1] = v[q] + v[R - q];
            b[q - 1] = v[q] - v[R - q];
        }
        cpx<T> out[R];
        cpx<T> x0 = v[0];
#pragma unroll
        for (int q = 0; q < H; ++q) x0 = x0 + a[q];
        out[0] = x0;
#pragma unroll
        for (int t = 1; t <= H; ++t) {
            cpx<T> re = v[0], im = czero<T>();
#pragma unroll
            for (int q = 1; q <= H; ++q) {
                const T c = K.c[q - 1][t - 1];
                const T s = K.s[q - 1][t - 1];
                re = cpx<T>{re.re + a[q - 1].re * c, re.im + a[q - 1].im * c};
                im = cpx<T>{im.re + b[q - 1].re * s, im.im + b[q - 1].im * s};
            }
            const cpx<T> j = mul_i<DIR>(im);
            out[t] = re + j;
            out[R - t] = re - j;
        }
#pragma unroll
        for (int t = 0; t < R; ++t) v[t] = out[t];
    }
};
template <int DIR, class T>
struct DFT<7, DIR, T> : DFTOdd<7, DIR, T> {};
template <int DIR, class T>
struct DFT<11, DIR, T> : DFTOdd<11, DIR, T> {};
template <int DIR, class T>
struct DFT<13, DIR, T> : DFTOdd<13, DIR, T> {};

}  // namespace hpxfft_gpu
