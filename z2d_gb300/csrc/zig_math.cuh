// zig_math.cuh -- the Zig standard-library math that z2d's colour and
// gradient code calls, for host and device.
//
// z2d is a freestanding Zig library (it links no libc), so its f32 @exp and
// @log lower to Zig's compiler_rt expf / logf, which are ports of musl's
// expf.c / logf.c (the FreeBSD msun e_expf.c / e_logf.c forms).
// std.math.pow (lib/std/math/pow.zig) is Zig's port of Go's math.Pow, and
// std.math.atan2 / atan (lib/std/math/atan2.zig, atan.zig) are ports of
// musl's atan2.c / atan.c (FreeBSD e_atan2.c / s_atan.c).  These are
// written from those published algorithms.  With --fmad=false and IEEE
// division every operation rounds as in Zig, so the device and the host get
// the same bits as z2d instead of the host libm's or CUDA's results.
//
// Callers in z2d: std.math.pow(f32, x, 2.2 or 1/2.2) for sRGB gamma
// (src/color.zig:336-351, src/internal/color_vector.zig:210-240) and
// std.math.atan2(f64) for the conic gradient (src/gradient.zig:739).
#pragma once
#include <stdint.h>
#include <string.h>

#ifndef Z2D_HD
#define Z2D_HD __host__ __device__ __forceinline__
#endif

namespace z2dg {
namespace zm {

Z2D_HD uint32_t fbits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
Z2D_HD float ffrom(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
Z2D_HD uint32_t dhi(double d) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2hiint(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return (uint32_t)(u >> 32);
#endif
}
Z2D_HD uint32_t dlo(double d) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2loint(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return (uint32_t)u;
#endif
}

// 2^n as a float for -126 <= n <= 127
Z2D_HD float pow2f(int n) { return ffrom((uint32_t)(0x7F + n) << 23); }

// x * 2^n: exact while the result is normal; otherwise the last multiply
// rounds once (std.math.scalbn).
Z2D_HD float scalbnf(float x, int n) {
    if (n > 127) {
        x *= pow2f(127);
        n -= 127;
        if (n > 127) {
            x *= pow2f(127);
            n -= 127;
            if (n > 127) n = 127;
        }
    } else if (n < -126) {
        x *= pow2f(-102);
        n += 102;
        if (n < -126) {
            x *= pow2f(-102);
            n += 102;
            if (n < -126) n = -126;
        }
    }
    return x * pow2f(n);
}

// expf: k = round(x / ln2), r = x - k*ln2 split in two parts (k*ln2hi is
// exact), exp(r) = 1 + r + r*c/(2-c) with c = r - r^2 (P1 + r^2 P2).
Z2D_HD float expf_(float x) {
    const float ln2hi = ffrom(0x3F317200u);   // 6.9314575195e-1
    const float ln2lo = ffrom(0x35BFBE8Eu);   // 1.4286067653e-6
    const float invln2 = ffrom(0x3FB8AA3Bu);  // 1.4426950216
    const float P1 = ffrom(0x3E2AAA8Fu);      // 0xaaaa8f * 2^-26 = 1.6666625440e-1
    const float P2 = ffrom(0xBB355215u);      // -0xb55215 * 2^-32 = -2.7667332906e-3
    uint32_t hx = fbits(x);
    const int neg = (int)(hx >> 31);
    hx &= 0x7FFFFFFFu;
    if (hx >= 0x42AEAC50u) {  // |x| >= 87.33655, or NaN
        if (hx > 0x7F800000u) return x;
        if (hx >= 0x42B17218u && !neg) return x * pow2f(127);
        if (neg && hx >= 0x42CFF1B5u) return 0.0f;
    }
    int k;
    float hi, lo;
    if (hx > 0x3EB17218u) {  // |x| > ln2 / 2
        k = (hx > 0x3F851592u) ? (int)(invln2 * x + (neg ? -0.5f : 0.5f)) : 1 - neg - neg;
        const float fk = (float)k;
        hi = x - fk * ln2hi;
        lo = fk * ln2lo;
        x = hi - lo;
    } else if (hx > 0x39000000u) {  // |x| > 2^-14
        k = 0;
        hi = x;
        lo = 0.0f;
    } else {
        return 1.0f + x;
    }
    const float xx = x * x;
    const float c = x - xx * (P1 + xx * P2);
    const float y = 1.0f + (x * c / (2.0f - c) - lo + hi);
    return k == 0 ? y : scalbnf(y, k);
}

// logf: x = 2^k * (1 + f) with 1 + f in [sqrt(2)/2, sqrt(2)],
// s = f / (2 + f), log(1 + f) = f - f^2/2 + s (f^2/2 + R(s^2)).
Z2D_HD float logf_(float x) {
    const float ln2_hi = ffrom(0x3F317180u);  // 6.9313812256e-01
    const float ln2_lo = ffrom(0x3717F7D1u);  // 9.0580006145e-06
    const float Lg1 = ffrom(0x3F2AAAAAu);     // 0xaaaaaa * 2^-24
    const float Lg2 = ffrom(0x3ECCCE13u);     // 0xccce13 * 2^-25
    const float Lg3 = ffrom(0x3E91E9EEu);     // 0x91e9ee * 2^-25
    const float Lg4 = ffrom(0x3E789E26u);     // 0xf89e26 * 2^-26
    uint32_t ix = fbits(x);
    int k = 0;
    if (ix < 0x00800000u || (ix >> 31)) {
        if ((ix << 1) == 0) return -ffrom(0x7F800000u);
        if (ix >> 31) return ffrom(0x7FC00000u);
        k = -25;
        x *= pow2f(25);
        ix = fbits(x);
    } else if (ix >= 0x7F800000u) {
        return x;
    } else if (ix == 0x3F800000u) {
        return 0.0f;
    }
    ix += 0x3F800000u - 0x3F3504F3u;
    k += (int)(ix >> 23) - 0x7F;
    x = ffrom((ix & 0x007FFFFFu) + 0x3F3504F3u);
    const float f = x - 1.0f;
    const float s = f / (2.0f + f);
    const float z = s * s;
    const float w = z * z;
    const float R = z * (Lg1 + w * Lg3) + w * (Lg2 + w * Lg4);
    const float hfsq = 0.5f * f * f;
    const float dk = (float)k;
    return s * (hfsq + R) + dk * ln2_lo - hfsq + f + dk * ln2_hi;
}

// frexp: x = m * 2^e, m in [0.5, 1)
Z2D_HD float frexpf_(float x, int &e) {
    uint32_t u = fbits(x);
    int ex = (int)((u >> 23) & 0xFFu);
    e = 0;
    if (ex == 0xFF || (u << 1) == 0) return x;
    int adj = 0;
    if (ex == 0) {
        x *= pow2f(64);
        u = fbits(x);
        ex = (int)((u >> 23) & 0xFFu);
        adj = 64;
    }
    e = ex - 126 - adj;
    return ffrom((u & 0x807FFFFFu) | 0x3F000000u);
}

Z2D_HD bool odd_integer(float y) {
    if (!(y == y) || y >= 16777216.0f || y <= -16777216.0f) return false;
    const int64_t t = (int64_t)y;
    return (float)t == y && (t & 1) != 0;
}

Z2D_HD float inf_f() { return ffrom(0x7F800000u); }

// std.math.pow(f32): the special cases in Go's order, then
// x^y = exp(yf * log(x)) * x^yi, with yf moved into (-0.5, 0.5] and x^yi
// by binary powering of frexp(x) (mantissa kept in [0.5, 1), exponent
// accumulated), the exponent applied last.
Z2D_HD float powf_(float x, float y) {
    if (y == 0.0f || x == 1.0f) return 1.0f;
    if (!(x == x) || !(y == y)) return ffrom(0x7FC00000u);
    if (y == 1.0f) return x;
    const float ax = x < 0.0f ? -x : x, ay = y < 0.0f ? -y : y;
    if (x == 0.0f) {
        if (y < 0.0f) return odd_integer(y) ? (fbits(x) >> 31 ? -inf_f() : inf_f()) : inf_f();
        return odd_integer(y) ? x : 0.0f;
    }
    if (ay == inf_f()) {
        if (x == -1.0f) return 1.0f;
        return ((ax < 1.0f) == (y > 0.0f)) ? 0.0f : inf_f();
    }
    if (ax == inf_f()) {
        if (x < 0.0f) {  // pow(-inf, y) = pow(-0, -y)
            if (-y < 0.0f) return odd_integer(-y) ? -inf_f() : inf_f();
            return odd_integer(-y) ? -0.0f : 0.0f;
        }
        return y < 0.0f ? 0.0f : inf_f();
    }
#ifdef __CUDA_ARCH__
    if (y == 0.5f) return __fsqrt_rn(x);
    if (y == -0.5f) return 1.0f / __fsqrt_rn(x);
    float yi = truncf(ay);
#else
    if (y == 0.5f) return sqrtf(x);
    if (y == -0.5f) return 1.0f / sqrtf(x);
    float yi = truncf(ay);
#endif
    float yf = ay - yi;
    if (yf != 0.0f && x < 0.0f) return ffrom(0x7FC00000u);
    if (yi >= 2147483648.0f) {
        if (x == -1.0f) return 1.0f;
        return ((ax < 1.0f) == (y > 0.0f)) ? 0.0f : inf_f();
    }
    float a1 = 1.0f;
    int ae = 0;
    if (yf != 0.0f) {
        if (yf > 0.5f) {
            yf -= 1.0f;
            yi += 1.0f;
        }
        a1 = expf_(yf * logf_(x));
    }
    int xe;
    float x1 = frexpf_(x, xe);
    for (int32_t i = (int32_t)yi; i != 0; i >>= 1) {
        if (xe < -512 || 512 < xe) {
            ae += xe;
            break;
        }
        if (i & 1) {
            a1 *= x1;
            ae += xe;
        }
        x1 *= x1;
        xe *= 2;
        if (x1 < 0.5f) {
            x1 += x1;
            xe -= 1;
        }
    }
    if (y < 0.0f) {
        a1 = 1.0f / a1;
        ae = -ae;
    }
    return scalbnf(a1, ae);
}

// atan (f64): |x| reduced around 0.5, 1, 1.5 or infinity (atan of the
// break point in a hi + lo pair), then an odd polynomial in x^2 evaluated as
// two Horner chains in x^4.
Z2D_HD double atan_(double x) {
    const double hi0 = 4.63647609000806093515e-01, hi1 = 7.85398163397448278999e-01;
    const double hi2 = 9.82793723247329054082e-01, hi3 = 1.57079632679489655800e+00;
    const double lo0 = 2.26987774529616870924e-17, lo1 = 3.06161699786838301793e-17;
    const double lo2 = 1.39033110312309984516e-17, lo3 = 6.12323399573676603587e-17;
    const double T0 = 3.33333333333329318027e-01, T1 = -1.99999999998764832476e-01;
    const double T2 = 1.42857142725034663711e-01, T3 = -1.11111104054623557880e-01;
    const double T4 = 9.09088713343650656196e-02, T5 = -7.69187620504482999495e-02;
    const double T6 = 6.66107313738753120669e-02, T7 = -5.83357013379057348645e-02;
    const double T8 = 4.97687799461593236017e-02, T9 = -3.65315727442169155270e-02;
    const double T10 = 1.62858201153657823623e-02;
    uint32_t ix = dhi(x);
    const bool neg = (ix >> 31) != 0;
    ix &= 0x7FFFFFFFu;
    if (ix >= 0x44100000u) {  // |x| >= 2^66
        if (!(x == x)) return x;
        const double z = hi3 + 0x1p-120;
        return neg ? -z : z;
    }
    double bhi = 0.0, blo = 0.0;
    bool reduced = true;
    if (ix < 0x3FDC0000u) {  // |x| < 7/16
        if (ix < 0x3E400000u) return x;
        reduced = false;
    } else {
        x = x < 0.0 ? -x : x;
        if (ix < 0x3FE60000u) {         // [7/16, 11/16)
            bhi = hi0; blo = lo0;
            x = (2.0 * x - 1.0) / (2.0 + x);
        } else if (ix < 0x3FF30000u) {  // [11/16, 19/16)
            bhi = hi1; blo = lo1;
            x = (x - 1.0) / (x + 1.0);
        } else if (ix < 0x40038000u) {  // [19/16, 39/16)
            bhi = hi2; blo = lo2;
            x = (x - 1.5) / (1.0 + 1.5 * x);
        } else {
            bhi = hi3; blo = lo3;
            x = -1.0 / x;
        }
    }
    const double z = x * x;
    const double w = z * z;
    const double s1 = z * (T0 + w * (T2 + w * (T4 + w * (T6 + w * (T8 + w * T10)))));
    const double s2 = w * (T1 + w * (T3 + w * (T5 + w * (T7 + w * T9))));
    if (!reduced) return x - x * (s1 + s2);
    const double r = bhi - ((x * (s1 + s2) - blo) - x);
    return neg ? -r : r;
}

// atan2 (f64): quadrant from the signs (m = 2*sign(x) + sign(y)), zero and
// infinite operands, |y/x| beyond 2^64 either way, else atan(|y/x|) moved
// into the quadrant with pi split in hi + lo.
Z2D_HD double atan2_(double y, double x) {
    const double pi = 3.1415926535897931160E+00, pi_lo = 1.2246467991473531772E-16;
    if (!(x == x) || !(y == y)) return x + y;
    uint32_t ix = dhi(x), iy = dhi(y);
    const uint32_t lx = dlo(x), ly = dlo(y);
    if (((ix - 0x3FF00000u) | lx) == 0) return atan_(y);
    const uint32_t m = ((iy >> 31) & 1u) | ((ix >> 30) & 2u);
    ix &= 0x7FFFFFFFu;
    iy &= 0x7FFFFFFFu;
    if ((iy | ly) == 0) return m <= 1 ? y : (m == 2 ? pi : -pi);
    if ((ix | lx) == 0) return (m & 1) ? -pi / 2 : pi / 2;
    if (ix == 0x7FF00000u) {
        if (iy == 0x7FF00000u) {
            const double q = (m & 2) ? 3 * pi / 4 : pi / 4;
            return (m & 1) ? -q : q;
        }
        const double q = (m & 2) ? pi : 0.0;
        return (m & 1) ? -q : q;
    }
    if (ix + (64u << 20) < iy || iy == 0x7FF00000u) return (m & 1) ? -pi / 2 : pi / 2;
    double z;
    if ((m & 2) && iy + (64u << 20) < ix) {
        z = 0.0;
    } else {
        const double q = y / x;
        z = atan_(q < 0.0 ? -q : q);
    }
    switch (m) {
        case 0: return z;
        case 1: return -z;
        case 2: return pi - (z - pi_lo);
        default: return (z - pi_lo) - pi;
    }
}

}  // namespace zm
}  // namespace z2dg
