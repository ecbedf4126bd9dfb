// grad_fast.cuh -- gradient offsets in double-word f32 arithmetic, exact to
// the f64 evaluation.
//
// Gradient.getOffset (src/gradient.zig:239-243, 349-372, 605-648, 731-741)
// computes in f64 and rounds the offset to f32.  This GPU runs f64 at a
// small fraction of its f32 rate, so the f64 chain is most of the cost of a
// gradient pixel.  Here the same expression is evaluated on double-word
// numbers (an unevaluated sum hi + lo of two floats, about 48 significant
// bits) together with a bound e on |double-word value - f64 value|.  When
// every value within e of the double-word result rounds to the same float
// (and every comparison the f64 code makes is decided the same way for all
// of them), that float IS the f64 code's result; otherwise the caller runs
// the f64 code.  The bound is e = 2^-38 x the expression evaluated on
// absolute values, about ten times the sum of both evaluations' rounding
// errors (f64: k * 2^-53, double-word: about 2^-45.7 per operation, see
// Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", ACM TOMS 44(2), 2017), so the
// slow path runs for roughly one pixel in 2^13, where the f32 rounding is
// genuinely close.
//
// Constants enter as double-word splits of the gradient's f64 values (error
// <= 2^-48 relative; the fast path is only taken when every nonzero
// constant lies in [2^-60, 2^60], so both words are normal floats) and pixel
// coordinates below 2^22 (exact as floats).  An intermediate that overflows
// makes its bound infinite or NaN, which sends the pixel to the f64 code;
// one that underflows errs by at most 2^-149, which the bound's floor of
// 2^-100 covers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace z2dg {

struct DW {
    float h, l;
};

// Per-gradient double-word constants, filled on the host.
struct GradFast {
    // kFastNone: f64 only; kFastVoid: every offset is -1 (zero-length
    // linear, radial with both radii 0); else the kind of evaluation
    int32_t mode;
    int32_t pad_;
    DW tf[6];    // inverse transformation
    DW g0, g1;   // start point (linear) / inner centre (radial) / centre (conic)
    // linear: dx, dy, 1 / |d|^2; radial: cdx, cdy, inner_r * dr,
    // -inner_r * inner_r, a, 1 / a, dr, min_dr; conic: angle
    DW k[8];
};

enum : int32_t { kFastNone = 0, kFastLinear = 1, kFastRadial = 2, kFastRadialA0 = 3, kFastConic = 4, kFastVoid = 5 };

#if defined(__CUDACC__)

// ----------------------------------------------------- error-free steps
__device__ __forceinline__ DW two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return DW{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DW fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    const float s = a + b;
    return DW{s, b - (s - a)};
}
__device__ __forceinline__ DW two_prod(float a, float b) {
    const float p = a * b;
    return DW{p, __fmaf_rn(a, b, -p)};
}

// ------------------------------------------------ double-word operations
// AccurateDWPlusDW (relative error <= 3u^2)
__device__ __forceinline__ DW dw_add(DW x, DW y) {
    const DW s = two_sum(x.h, y.h), t = two_sum(x.l, y.l);
    const DW v = fast_two_sum(s.h, s.l + t.h);
    return fast_two_sum(v.h, t.l + v.l);
}
__device__ __forceinline__ DW dw_neg(DW x) { return DW{-x.h, -x.l}; }
__device__ __forceinline__ DW dw_sub(DW x, DW y) { return dw_add(x, dw_neg(y)); }
// DWPlusFP (relative error <= 2u^2)
__device__ __forceinline__ DW dw_add_f(DW x, float y) {
    const DW s = two_sum(x.h, y);
    return fast_two_sum(s.h, x.l + s.l);
}
// DWTimesDW with FMA (relative error <= 5u^2)
__device__ __forceinline__ DW dw_mul(DW x, DW y) {
    const DW c = two_prod(x.h, y.h);
    const float t = __fmaf_rn(x.l, y.h, __fmaf_rn(x.h, y.l, x.l * y.l));
    return fast_two_sum(c.h, c.l + t);
}
// DWTimesFP with FMA (relative error <= 2u^2)
__device__ __forceinline__ DW dw_mul_f(DW x, float y) {
    const DW c = two_prod(x.h, y);
    return fast_two_sum(c.h, __fmaf_rn(x.l, y, c.l));
}
// x / y: a float quotient, then the double-word remainder divided once more
__device__ __forceinline__ DW dw_div(DW x, DW y) {
    const float q1 = __fdiv_rn(x.h, y.h);
    const DW r = dw_sub(x, dw_mul_f(y, q1));
    return fast_two_sum(q1, __fdiv_rn(r.h, y.h));
}
// sqrt(x), x > 0: the float root, then one Newton correction from the
// exact residual x.h - s^2
__device__ __forceinline__ DW dw_sqrt(DW x) {
    const float s = __fsqrt_rn(x.h);
    const float r = __fmaf_rn(-s, s, x.h);
    return fast_two_sum(s, __fdiv_rn(r + x.l, 2.0f * s));
}
__device__ __forceinline__ float dw_abs_h(DW x) { return fabsf(x.h); }

constexpr float kFastErr = 0x1p-38f;   // bound factor on the absolute-value expression
constexpr float kFastFloor = 0x1p-100f;
// For the conic's short chains (one to four operations from exact or split
// inputs) the sum of both evaluations' errors is below 2^-43.7 x the
// absolute-value expression; 2^-42 keeps a margin of three and leaves the
// 1 / r amplification near the centre room.
constexpr float kFastErrShort = 0x1p-42f;

// The f32 that every value within e of x rounds to, clamped to [0, 1]
// (round and clamp commute: 0 and 1 are floats); false when they differ.
__device__ __forceinline__ bool dw_round(DW x, float e, bool clamp, float &out) {
    if (!(e < 0x1p60f) || !(fabsf(x.h) < 0x1p60f)) return false;
    float lo = x.h + __fsub_rd(x.l, e);
    float hi = x.h + __fadd_ru(x.l, e);
    if (clamp) {
        lo = fminf(fmaxf(lo, 0.0f), 1.0f);
        hi = fminf(fmaxf(hi, 0.0f), 1.0f);
    }
    if (!(lo == hi)) return false;
    out = lo;
    return true;
}

// The pixel centre after the inverse transformation, with the magnitude of
// its terms (|tf0 x| + |tf1 y| + |tf4|).
__device__ __forceinline__ void fast_point(const GradFast &F, bool has_tf, float fx, float fy, DW &px, DW &py, float &ax,
                                           float &ay) {
    if (has_tf) {
        px = dw_add(dw_add(dw_mul_f(F.tf[0], fx), dw_mul_f(F.tf[1], fy)), F.tf[4]);
        py = dw_add(dw_add(dw_mul_f(F.tf[2], fx), dw_mul_f(F.tf[3], fy)), F.tf[5]);
        ax = dw_abs_h(F.tf[0]) * fabsf(fx) + dw_abs_h(F.tf[1]) * fabsf(fy) + dw_abs_h(F.tf[4]);
        ay = dw_abs_h(F.tf[2]) * fabsf(fx) + dw_abs_h(F.tf[3]) * fabsf(fy) + dw_abs_h(F.tf[5]);
    } else {
        px = DW{fx, 0.0f};
        py = DW{fy, 0.0f};
        ax = fabsf(fx);
        ay = fabsf(fy);
    }
}

// Linear.getOffset: clamp((d . (p - start)) / |d|^2, 0, 1).  Returns 1 and
// the offset when decided, 0 to take the f64 path.
__device__ __forceinline__ int fast_linear(const GradFast &F, bool has_tf, float fx, float fy, float &out) {
    DW px, py;
    float ax, ay;
    fast_point(F, has_tf, fx, fy, px, py, ax, ay);
    const DW sx = dw_sub(px, F.g0), sy = dw_sub(py, F.g1);
    ax += dw_abs_h(F.g0);
    ay += dw_abs_h(F.g1);
    const DW q = dw_mul(dw_add(dw_mul(F.k[0], sx), dw_mul(F.k[1], sy)), F.k[2]);
    const float m = (dw_abs_h(F.k[0]) * ax + dw_abs_h(F.k[1]) * ay) * dw_abs_h(F.k[2]);
    return dw_round(q, m * kFastErr + kFastFloor, true, out) ? 1 : 0;
}

// Radial.getOffset (two-circle form).  Every comparison of the f64 code
// (b == 0, discr >= 0, t * dr >= min_dr) is taken only when the interval
// of its operand excludes the threshold.  -1 is the invalid offset.
__device__ __forceinline__ int fast_radial(const GradFast &F, bool has_tf, bool a_zero, float fx, float fy,
                                           float &out) {
    DW px, py;
    float ax, ay;
    fast_point(F, has_tf, fx, fy, px, py, ax, ay);
    const DW dx = dw_sub(px, F.g0), dy = dw_sub(py, F.g1);
    ax += dw_abs_h(F.g0);
    ay += dw_abs_h(F.g1);
    const DW cdx = F.k[0], cdy = F.k[1], ir_dr = F.k[2], nir2 = F.k[3], a = F.k[4], inv_a = F.k[5], dr = F.k[6],
             min_dr = F.k[7];
    const DW b = dw_add(dw_add(dw_mul(dx, cdx), dw_mul(dy, cdy)), ir_dr);
    const DW c = dw_add(dw_add(dw_mul(dx, dx), dw_mul(dy, dy)), nir2);
    const float Ab = ax * dw_abs_h(cdx) + ay * dw_abs_h(cdy) + dw_abs_h(ir_dr);
    const float Ac = ax * ax + ay * ay + dw_abs_h(nir2);
    const float eb = Ab * kFastErr + kFastFloor, ec = Ac * kFastErr + kFastFloor;
    const float adr = dw_abs_h(dr), amin = dw_abs_h(min_dr);
    // t * dr >= min_dr, decided over the interval of t (half-width et)
    auto accept = [&](DW t, float et, int &verdict) -> bool {
        const DW p = dw_mul(t, dr);
        const float ep = et * adr + (fabsf(p.h) + amin) * kFastErr + kFastFloor;
        const DW diff = dw_sub(p, min_dr);
        if (!(fabsf(diff.h) * 0.99999f > ep)) return false;
        verdict = diff.h > 0.0f ? 1 : 0;
        return true;
    };
    if (a_zero) {
        if (!(fabsf(b.h) * 0.99999f > 2.0f * eb)) return 0;  // b == 0 undecided (or b too small to divide by)
        const DW t = dw_div(DW{0.5f * c.h, 0.5f * c.l}, b);
        const float at = fabsf(t.h);
        const float et = (0.5f * ec + at * eb) / (fabsf(b.h) - eb) * 1.01f + at * kFastErr + kFastFloor;
        int ok;
        if (!accept(t, et, ok)) return 0;
        if (!ok) {
            out = -1.0f;
            return 1;
        }
        return dw_round(t, et, true, out) ? 1 : 0;
    }
    const DW disc = dw_add(dw_mul(b, b), dw_mul(a, dw_neg(c)));
    const float ed = (Ab * Ab + dw_abs_h(a) * Ac) * kFastErr + kFastFloor;
    if (!(fabsf(disc.h) * 0.99999f > ed)) return 0;  // discr >= 0 undecided
    if (disc.h < 0.0f) {
        out = -1.0f;
        return 1;
    }
    const DW sq = dw_sqrt(disc);
    const float esq = ed / __fsqrt_rn(disc.h - ed) + sq.h * kFastErr;
    const float ainv = dw_abs_h(inv_a);
    const float e_lin = (eb + esq + (fabsf(b.h) + sq.h) * kFastErr) * ainv * 1.01f;
    const DW t0 = dw_mul(dw_add(b, sq), inv_a);
    const float e0 = e_lin + fabsf(t0.h) * kFastErr + kFastFloor;
    int ok;
    if (!accept(t0, e0, ok)) return 0;
    if (ok) return dw_round(t0, e0, true, out) ? 1 : 0;
    const DW t1 = dw_mul(dw_sub(b, sq), inv_a);
    const float e1 = e_lin + fabsf(t1.h) * kFastErr + kFastFloor;
    if (!accept(t1, e1, ok)) return 0;
    if (ok) return dw_round(t1, e1, true, out) ? 1 : 0;
    out = -1.0f;
    return 1;
}

// Double-word constants: the real pi / 2 and pi, the f64 2*pi z2d divides
// by (6.283185307179586) and its reciprocal, 1/3, and atan(k / 16) for
// k = 0..16 (each the float hi + lo split of the value).
__device__ __forceinline__ DW atan_k16(int k) {
    switch (k) {
        case 1: return DW{0x1.ff55bcp-5f, -0x1.1a6042p-30f};
        case 2: return DW{0x1.fd5baap-4f, -0x1.54f424p-30f};
        case 3: return DW{0x1.7b97b4p-3f, 0x1.79cb6p-28f};
        case 4: return DW{0x1.f5b76p-3f, -0x1.b4dfc8p-29f};
        case 5: return DW{0x1.362774p-2f, -0x1.1f0286p-27f};
        case 6: return DW{0x1.6f6194p-2f, 0x1.e4defp-30f};
        case 7: return DW{0x1.a64eecp-2f, 0x1.e611fep-29f};
        case 8: return DW{0x1.dac67p-2f, 0x1.586ed4p-28f};
        case 9: return DW{0x1.0657eap-1f, -0x1.6499e6p-26f};
        case 10: return DW{0x1.1e00bap-1f, 0x1.7bdfd6p-26f};
        case 11: return DW{0x1.345f02p-1f, -0x1.98e422p-28f};
        case 12: return DW{0x1.4978fap-1f, 0x1.934f7p-28f};
        case 13: return DW{0x1.5d5898p-1f, 0x1.c5a6c6p-27f};
        case 14: return DW{0x1.700a7cp-1f, 0x1.5e118cp-27f};
        case 15: return DW{0x1.819d0cp-1f, -0x1.1d4eb6p-26f};
        case 16: return DW{0x1.921fb6p-1f, -0x1.777a5cp-26f};
        default: return DW{0.0f, 0.0f};
    }
}
constexpr DW kDwPi2{0x1.921fb6p+0f, -0x1.777a5cp-25f};
constexpr DW kDwPi{0x1.921fb6p+1f, -0x1.777a5cp-24f};
constexpr DW kDwTwoPi{0x1.921fb6p+2f, -0x1.777a5cp-23f};
constexpr DW kDwInvTwoPi{0x1.45f306p-3f, 0x1.b93910p-28f};
constexpr DW kDwThird{0x1.555556p-2f, -0x1.555556p-27f};

// Conic.getOffset: @mod(atan2(dy, dx) - angle, 2 pi) / 2 pi.  atan2 by
// octant reduction, a table step atan(k/16) and the series of atan(w) for
// |w| <= 1/32 to w^9 (truncation below 2^-58).  The f64 code's error as a
// function of its inputs is bounded by |grad atan2| = 1 / r over the box of
// possible inputs; the box must stay off the branch cut (dy = 0, dx < 0)
// and off the origin, and v = atan2 - angle off the wrap points 0 and -2 pi.
__device__ __forceinline__ int fast_conic(const GradFast &F, bool has_tf, float fx, float fy, float &out) {
    DW px, py;
    float ax, ay;
    fast_point(F, has_tf, fx, fy, px, py, ax, ay);
    const DW dx = dw_sub(px, F.g0), dy = dw_sub(py, F.g1);
    const float ex = (ax + dw_abs_h(F.g0)) * kFastErrShort + kFastFloor;
    const float ey = (ay + dw_abs_h(F.g1)) * kFastErrShort + kFastFloor;
    // (|x.l| <= 2^-24 |x.h|: the 0.99999 factors cover the low words)
    const float r_lo = fmaxf(fabsf(dx.h) * 0.99999f - ex, fabsf(dy.h) * 0.99999f - ey);
    if (!(r_lo > 0.0f)) return 0;
    if (!(fabsf(dy.h) * 0.99999f > ey) && dx.h < ex) return 0;  // on or near the branch cut
    const DW X = dx.h < 0.0f ? dw_neg(dx) : dx, Y = dy.h < 0.0f ? dw_neg(dy) : dy;
    const bool swap = Y.h > X.h;
    const DW N = swap ? X : Y, D = swap ? Y : X;
    int k = __float2int_rn(__fdividef(N.h, D.h) * 16.0f);
    k = min(max(k, 0), 16);
    const float cst = (float)k * 0.0625f;
    const DW w = dw_div(dw_sub(N, dw_mul_f(D, cst)), dw_add(D, dw_mul_f(N, cst)));
    const DW s = dw_mul(w, w);
    const float sf = s.h;
    const float tail = sf * sf * (0.2f - sf * (0.142857149f - sf * 0.111111112f));  // w^4/5 - w^6/7 + w^8/9
    const DW poly = dw_add_f(dw_add_f(dw_neg(dw_mul(s, kDwThird)), 1.0f), tail);
    DW th = dw_add(atan_k16(k), dw_mul(w, poly));
    if (swap) th = dw_sub(kDwPi2, th);
    if (dx.h < 0.0f) th = dw_sub(kDwPi, th);
    if (dy.h < 0.0f) th = dw_neg(th);
    // atan2's own error: below 2^-43.5 for this evaluation (absolute, the
    // angle is at most pi), below 2^-51 for fdlibm's
    const float eth = 2.0f * (ex + ey) / r_lo + kFastErr;
    const DW v = dw_sub(th, F.k[0]);
    const float ev = eth + (fabsf(th.h) + dw_abs_h(F.k[0])) * kFastErrShort + kFastFloor;
    if (!(fabsf(v.h) * 0.99999f > ev)) return 0;  // at the wrap to 2 pi
    DW ang = v;
    if (v.h < 0.0f) {
        const DW u = dw_add(v, kDwTwoPi);
        if (!(fabsf(u.h) * 0.99999f > ev + 8.0f * kFastErrShort)) return 0;  // at -2 pi
        ang = u.h > 0.0f ? u : dw_add(u, kDwTwoPi);
    }
    const DW t = dw_mul(ang, kDwInvTwoPi);
    const float et = (ev + 16.0f * kFastErrShort) * 0.16f + fabsf(t.h) * kFastErrShort + kFastFloor;
    return dw_round(t, et, false, out) ? 1 : 0;
}

#endif  // __CUDACC__

}  // namespace z2dg
