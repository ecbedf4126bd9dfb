// zig_trig.cuh -- the f64 trigonometry and integer powers z2d's arcs call,
// for host and device.
//
// src/internal/arc.zig computes the arc splines with @sin, @cos and @tan on
// f64 and std.math.pow(f64, x, 6 or 2).  Zig lowers the f64 builtins to its
// compiler_rt sin / cos / tan, ports of musl's sin.c / cos.c / tan.c with
// the kernels __sin / __cos / __tan (FreeBSD msun k_sin.c, k_cos.c, k_tan.c)
// and the argument reduction __rem_pio2 (e_rem_pio2.c); std.math.pow is the
// port of Go's math.Pow whose integer-exponent part is a square-and-multiply
// on frexp's significand.  These are written from those published
// algorithms.  The reduction covers |x| < 2^20 * pi/2 (the medium case,
// Cody-Waite in up to three steps, exact to 151 bits); larger arguments
// (Payne-Hanek in musl) are reported to the caller, which rejects them.
#pragma once
#include <stdint.h>
#include <string.h>

#include "zig_math.cuh"

namespace z2dg {
namespace zm {

Z2D_HD uint64_t dbits(double d) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
#endif
}
Z2D_HD double dfrom(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}
Z2D_HD double with_low_zero(double d) { return dfrom(dbits(d) & 0xFFFFFFFF00000000ull); }

// __rem_pio2 (medium arguments): x = n * pi/2 + (y0 + y1), |y0 + y1| <= pi/4.
// Returns false for |x| >= 2^20 * pi/2 (the large case) and for inf / NaN.
Z2D_HD bool rem_pio2_(double x, int &n, double &y0, double &y1) {
    const double toint = 6755399441055744.0;  // 1.5 / DBL_EPSILON
    const double pio4 = 7.85398163397448278999e-01;
    const double invpio2 = 6.36619772367581382433e-01;
    const double pio2_1 = 1.57079632673412561417e+00, pio2_1t = 6.07710050650619224932e-11;
    const double pio2_2 = 6.07710050630396597660e-11, pio2_2t = 2.02226624879595063154e-21;
    const double pio2_3 = 2.02226624871116645580e-21, pio2_3t = 8.47842766036889956997e-32;
    const uint64_t u = dbits(x);
    const bool sign = (u >> 63) != 0;
    const uint32_t ix = (uint32_t)(u >> 32) & 0x7FFFFFFFu;
    double z;
    bool medium = false;
    if (ix <= 0x400F6A7Au) {  // |x| ~<= 5pi/4
        if ((ix & 0xFFFFFu) == 0x921FBu) {
            medium = true;  // |x| ~= pi/2 or 2pi/2: cancellation
        } else if (ix <= 0x4002D97Cu) {  // |x| ~<= 3pi/4
            if (!sign) {
                z = x - pio2_1;
                y0 = z - pio2_1t;
                y1 = (z - y0) - pio2_1t;
                n = 1;
            } else {
                z = x + pio2_1;
                y0 = z + pio2_1t;
                y1 = (z - y0) + pio2_1t;
                n = -1;
            }
            return true;
        } else {
            if (!sign) {
                z = x - 2 * pio2_1;
                y0 = z - 2 * pio2_1t;
                y1 = (z - y0) - 2 * pio2_1t;
                n = 2;
            } else {
                z = x + 2 * pio2_1;
                y0 = z + 2 * pio2_1t;
                y1 = (z - y0) + 2 * pio2_1t;
                n = -2;
            }
            return true;
        }
    } else if (ix <= 0x401C463Bu) {  // |x| ~<= 9pi/4
        if (ix <= 0x4015FDBCu) {     // |x| ~<= 7pi/4
            if (ix == 0x4012D97Cu) {
                medium = true;  // |x| ~= 3pi/2
            } else {
                if (!sign) {
                    z = x - 3 * pio2_1;
                    y0 = z - 3 * pio2_1t;
                    y1 = (z - y0) - 3 * pio2_1t;
                    n = 3;
                } else {
                    z = x + 3 * pio2_1;
                    y0 = z + 3 * pio2_1t;
                    y1 = (z - y0) + 3 * pio2_1t;
                    n = -3;
                }
                return true;
            }
        } else {
            if (ix == 0x401921FBu) {
                medium = true;  // |x| ~= 4pi/2
            } else {
                if (!sign) {
                    z = x - 4 * pio2_1;
                    y0 = z - 4 * pio2_1t;
                    y1 = (z - y0) - 4 * pio2_1t;
                    n = 4;
                } else {
                    z = x + 4 * pio2_1;
                    y0 = z + 4 * pio2_1t;
                    y1 = (z - y0) + 4 * pio2_1t;
                    n = -4;
                }
                return true;
            }
        }
    }
    if (!medium && ix >= 0x413921FBu) return false;  // large, inf or NaN
    // rint(x / (pi/2)), then x - fn * pi/2 in one to three Cody-Waite steps
    double fn = x * invpio2 + toint - toint;
    n = (int32_t)fn;
    double r = x - fn * pio2_1;
    double w = fn * pio2_1t;
    if (r - w < -pio4) {  // only with directed rounding
        n--;
        fn--;
        r = x - fn * pio2_1;
        w = fn * pio2_1t;
    } else if (r - w > pio4) {
        n++;
        fn++;
        r = x - fn * pio2_1;
        w = fn * pio2_1t;
    }
    y0 = r - w;
    const int ex = (int)(ix >> 20);
    int ey = (int)((dbits(y0) >> 52) & 0x7FF);
    if (ex - ey > 16) {  // second step, good to 118 bits
        double t = r;
        w = fn * pio2_2;
        r = t - w;
        w = fn * pio2_2t - ((t - r) - w);
        y0 = r - w;
        ey = (int)((dbits(y0) >> 52) & 0x7FF);
        if (ex - ey > 49) {  // third step, good to 151 bits
            t = r;
            w = fn * pio2_3;
            r = t - w;
            w = fn * pio2_3t - ((t - r) - w);
            y0 = r - w;
        }
    }
    y1 = (r - y0) - w;
    return true;
}

// __sin: sin(x + y) on [-pi/4, pi/4]; iy = 0 when y is 0
Z2D_HD double k_sin(double x, double y, int iy) {
    const double S1 = -1.66666666666666324348e-01, S2 = 8.33333333332248946124e-03,
                 S3 = -1.98412698298579493134e-04, S4 = 2.75573137070700676789e-06,
                 S5 = -2.50507602534068634195e-08, S6 = 1.58969099521155010221e-10;
    const double z = x * x;
    const double w = z * z;
    const double r = S2 + z * (S3 + z * S4) + z * w * (S5 + z * S6);
    const double v = z * x;
    if (iy == 0) return x + v * (S1 + z * r);
    return x - ((z * (0.5 * y - v * r) - y) - v * S1);
}

// __cos: cos(x + y) on [-pi/4, pi/4]
Z2D_HD double k_cos(double x, double y) {
    const double C1 = 4.16666666666666019037e-02, C2 = -1.38888888888741095749e-03,
                 C3 = 2.48015872894767294178e-05, C4 = -2.75573143513906633035e-07,
                 C5 = 2.08757232129817482790e-09, C6 = -1.13596475577881948265e-11;
    const double z = x * x;
    double w = z * z;
    const double r = z * (C1 + z * (C2 + z * C3)) + w * w * (C4 + z * (C5 + z * C6));
    const double hz = 0.5 * z;
    w = 1.0 - hz;
    return w + (((1.0 - w) - hz) + (z * r - x * y));
}

// __tan: tan(x + y) (odd = 0) or -1 / tan(x + y) (odd = 1) on [-pi/4, pi/4]
Z2D_HD double k_tan(double x, double y, int odd) {
    const double T0 = 3.33333333333334091986e-01, T1 = 1.33333333333201242699e-01,
                 T2 = 5.39682539762260521377e-02, T3 = 2.18694882948595424599e-02,
                 T4 = 8.86323982359930005737e-03, T5 = 3.59207910759131235356e-03,
                 T6 = 1.45620945432529025516e-03, T7 = 5.88041240820264096874e-04,
                 T8 = 2.46463134818469906812e-04, T9 = 7.81794442939557092300e-05,
                 T10 = 7.14072491382608190305e-05, T11 = -1.85586374855275456654e-05,
                 T12 = 2.59073051863633712884e-05;
    const double pio4 = 7.85398163397448278999e-01, pio4lo = 3.06161699786838301793e-17;
    const uint32_t hx = dhi(x);
    const bool big = (hx & 0x7FFFFFFFu) >= 0x3FE59428u;  // |x| >= 0.6744
    bool sign = false;
    if (big) {
        sign = (hx >> 31) != 0;
        if (sign) {
            x = -x;
            y = -y;
        }
        x = (pio4 - x) + (pio4lo - y);
        y = 0.0;
    }
    const double z = x * x;
    double w = z * z;
    double r = T1 + w * (T3 + w * (T5 + w * (T7 + w * (T9 + w * T11))));
    double v = z * (T2 + w * (T4 + w * (T6 + w * (T8 + w * (T10 + w * T12)))));
    double s = z * x;
    r = y + z * (s * (r + v) + y) + s * T0;
    w = x + r;
    if (big) {
        s = 1 - 2 * odd;
        v = s - 2.0 * (x + (r - w * w / (w + s)));
        return sign ? -v : v;
    }
    if (!odd) return w;
    // -1 / (x + r) accurately: split w and the quotient at their low words
    const double w0 = with_low_zero(w);
    v = r - (w0 - x);
    const double a = -1.0 / w;
    const double a0 = with_low_zero(a);
    return a0 + a * (1.0 + a0 * w0 + a0 * v);
}

// sin / cos / tan; `ok` is cleared for arguments beyond the medium range
Z2D_HD double sin_(double x, bool &ok) {
    const uint32_t ix = dhi(x) & 0x7FFFFFFFu;
    if (ix <= 0x3FE921FBu) {  // |x| ~< pi/4
        if (ix < 0x3E500000u) return x;  // |x| < 2^-26
        return k_sin(x, 0.0, 0);
    }
    if (ix >= 0x7FF00000u) return x - x;
    int n;
    double y0, y1;
    if (!rem_pio2_(x, n, y0, y1)) {
        ok = false;
        return 0.0;
    }
    switch (n & 3) {
        case 0: return k_sin(y0, y1, 1);
        case 1: return k_cos(y0, y1);
        case 2: return -k_sin(y0, y1, 1);
        default: return -k_cos(y0, y1);
    }
}
Z2D_HD double cos_(double x, bool &ok) {
    const uint32_t ix = dhi(x) & 0x7FFFFFFFu;
    if (ix <= 0x3FE921FBu) {
        if (ix < 0x3E46A09Eu) return 1.0;  // |x| < 2^-27 * sqrt(2)
        return k_cos(x, 0.0);
    }
    if (ix >= 0x7FF00000u) return x - x;
    int n;
    double y0, y1;
    if (!rem_pio2_(x, n, y0, y1)) {
        ok = false;
        return 0.0;
    }
    switch (n & 3) {
        case 0: return k_cos(y0, y1);
        case 1: return -k_sin(y0, y1, 1);
        case 2: return -k_cos(y0, y1);
        default: return k_sin(y0, y1, 1);
    }
}
Z2D_HD double tan_(double x, bool &ok) {
    const uint32_t ix = dhi(x) & 0x7FFFFFFFu;
    if (ix <= 0x3FE921FBu) {
        if (ix < 0x3E400000u) return x;  // |x| < 2^-27
        return k_tan(x, 0.0, 0);
    }
    if (ix >= 0x7FF00000u) return x - x;
    int n;
    double y0, y1;
    if (!rem_pio2_(x, n, y0, y1)) {
        ok = false;
        return 0.0;
    }
    return k_tan(y0, y1, n & 1);
}

// frexp / scalbn on f64 (exact; scalbn steps through the exponent range
// like musl's so that only the last multiplication can round)
Z2D_HD double frexp_(double x, int &e) {
    const uint64_t u = dbits(x);
    const int ee = (int)((u >> 52) & 0x7FF);
    if (ee == 0) {
        if (x == 0.0) {
            e = 0;
            return x;
        }
        const double r = frexp_(x * 18446744073709551616.0, e);  // 2^64
        e -= 64;
        return r;
    }
    if (ee == 0x7FF) {
        e = 0;
        return x;
    }
    e = ee - 0x3FE;
    return dfrom((u & 0x800FFFFFFFFFFFFFull) | 0x3FE0000000000000ull);
}
Z2D_HD double scalbn_(double x, int n) {
    double y = x;
    if (n > 1023) {
        y *= 8.98846567431157953865e+307;  // 2^1023
        n -= 1023;
        if (n > 1023) {
            y *= 8.98846567431157953865e+307;
            n -= 1023;
            if (n > 1023) n = 1023;
        }
    } else if (n < -1022) {
        // 2^-1022 * 2^53: avoids double rounding in the subnormal range
        y *= 2.2250738585072014e-308 * 9007199254740992.0;
        n += 1022 - 53;
        if (n < -1022) {
            y *= 2.2250738585072014e-308 * 9007199254740992.0;
            n += 1022 - 53;
            if (n < -1022) n = -1022;
        }
    }
    return y * dfrom((uint64_t)(0x3FF + n) << 52);
}

// std.math.pow(f64, x, y) for the integer y arc.zig uses (y = 2, 6): the
// special cases of x, then x^y = frexp significand squared-and-multiplied
// with the exponent carried apart, scaled back by scalbn.
Z2D_HD double powi_(double x, int y) {
    if (y == 0 || x == 1.0) return 1.0;
    if (x != x) return x;
    if (y == 1) return x;
    if (x == 0.0) return (y > 0 && (y & 1) == 0) ? 0.0 : (y > 0 ? x : dfrom(0x7FF0000000000000ull));
    int xe;
    double x1 = frexp_(x, xe);
    if (xe == 0 && (dbits(x) & 0x7FF0000000000000ull) == 0x7FF0000000000000ull) {  // inf
        const bool neg = x < 0 && (y & 1);
        if (y < 0) return neg ? -0.0 : 0.0;
        return neg ? -x : (x < 0 ? -x : x);
    }
    double a1 = 1.0;
    int ae = 0;
    long long i = y < 0 ? -(long long)y : (long long)y;
    for (; i != 0; i >>= 1) {
        if (xe < -(1 << 12) || (1 << 12) < xe) {  // xe would overflow the shift below
            ae += xe;
            break;
        }
        if (i & 1) {
            a1 *= x1;
            ae += xe;
        }
        x1 *= x1;
        xe <<= 1;
        if (x1 < 0.5) {
            x1 += x1;
            xe -= 1;
        }
    }
    if (y < 0) {
        a1 = 1.0 / a1;
        ae = -ae;
    }
    return scalbn_(a1, ae);
}

}  // namespace zm
}  // namespace z2dg
