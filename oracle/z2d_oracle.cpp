// z2d_oracle.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// A CPU restatement of z2d's painter.fill / SurfaceCompositor path, written
// from the reference's algorithm in its own evaluation order so that it can
// serve as the bit-exact parity oracle for the GPU kernels and as the timed
// CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg load it.  Every function cites the z2d file:line it follows
// (paths inside the z2d project).
//
// Build flags matter: -O2/-O3 -ffp-contract=off -fno-fast-math.  z2d's Zig
// code has strict IEEE semantics (no fused multiply-add), which this file
// must match operation for operation.
//
// Known divergence (documented, not observable on balanced paths): z2d sorts
// active edges with std.sort.pdqContext; for <= 24 active edges that is an
// insertion sort (restated exactly below).  For > 24 active edges this file
// uses a stable merge sort.  The two orders can only differ for edges whose
// rounded crossings tie, and the order of tied edges only changes output on
// scanlines whose crossings are unbalanced (open 2-point subpaths).
#include "../include/z2dgpu.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// ===================================================================
// Pixel formats and surfaces          src/pixel.zig, src/surface.zig
// ===================================================================

int fmt_bits(int f) {
    switch (f) {
        case Z2D_FORMAT_ALPHA8: return 8;
        case Z2D_FORMAT_ALPHA4: return 4;
        case Z2D_FORMAT_ALPHA2: return 2;
        case Z2D_FORMAT_ALPHA1: return 1;
        default: return 32;
    }
}
bool fmt_packed(int f) { return f >= Z2D_FORMAT_ALPHA4; }
bool fmt_has_color(int f) { return f <= Z2D_FORMAT_RGBA; }
bool fmt_has_alpha(int f) { return f == Z2D_FORMAT_ARGB || f == Z2D_FORMAT_RGBA || f >= Z2D_FORMAT_ALPHA8; }
uint8_t fmt_max(int f) {
    switch (f) {
        case Z2D_FORMAT_ALPHA4: return 15;
        case Z2D_FORMAT_ALPHA2: return 3;
        case Z2D_FORMAT_ALPHA1: return 1;
        default: return 255;
    }
}

// Alpha(T).scaleIntoIntAlpha / shlr (src/pixel.zig:582-626): value with
// `from` bits to value with `to` bits.
uint32_t scale_alpha(uint32_t v, int from, int to) {
    if (from == 1) return v * ((1u << to) - 1);          // :583
    if (v == 0) return 0;                                 // :591
    if (from == to) return v;                             // :593
    if (from > to) return v >> (from - to);               // :597-599
    switch (to - from) {                                  // :618-625
        case 2: case 4: return (v << (to - from)) + v;
        case 6: return (v << (to - from)) | (v << (to - 2 * from)) | (v << (to - 3 * from)) | v;
        default: return v;
    }
}

// mem.readPackedInt / writePackedInt, little endian (src/pixel.zig:664-677)
uint32_t packed_get(const uint8_t *buf, size_t idx, int bits) {
    size_t bit = idx * (size_t)bits;
    return (buf[bit >> 3] >> (bit & 7)) & ((1u << bits) - 1);
}
void packed_set(uint8_t *buf, size_t idx, int bits, uint32_t v) {
    size_t bit = idx * (size_t)bits;
    uint8_t mask = (uint8_t)(((1u << bits) - 1) << (bit & 7));
    buf[bit >> 3] = (uint8_t)((buf[bit >> 3] & ~mask) | ((v << (bit & 7)) & mask));
}

struct Sfc {
    int fmt, w, h;
    uint8_t *buf;
};

// A z2d pixel held in its own format (src/pixel.zig:101-110).
struct Px {
    int fmt;
    uint8_t r, g, b, a;
};

// RGBA16 lane (src/compositor.zig:664-703)
struct I16 {
    uint16_t r, g, b, a;
};

// Raw pixel at flat index i, in the surface's own format.
Px raw_get(const Sfc &s, size_t i) {
    Px p{s.fmt, 0, 0, 0, 0};
    if (fmt_packed(s.fmt)) {
        p.a = (uint8_t)packed_get(s.buf, i, fmt_bits(s.fmt));
        return p;
    }
    if (s.fmt == Z2D_FORMAT_ALPHA8) {
        p.a = s.buf[i];
        return p;
    }
    const uint8_t *q = s.buf + 4 * i;
    switch (s.fmt) {
        case Z2D_FORMAT_ARGB: p.b = q[0]; p.g = q[1]; p.r = q[2]; p.a = q[3]; break;
        case Z2D_FORMAT_XRGB: p.b = q[0]; p.g = q[1]; p.r = q[2]; p.a = 0; break;
        case Z2D_FORMAT_RGB: p.r = q[0]; p.g = q[1]; p.b = q[2]; p.a = 0; break;
        default: p.r = q[0]; p.g = q[1]; p.b = q[2]; p.a = q[3]; break;
    }
    return p;
}

// Raw store; the padding byte of XRGB/RGB is written as 0 (z2d's vector
// store writes 0 there; its scalar store leaves it undefined).
void raw_set(Sfc &s, size_t i, const Px &p) {
    if (fmt_packed(s.fmt)) {
        packed_set(s.buf, i, fmt_bits(s.fmt), p.a);
        return;
    }
    if (s.fmt == Z2D_FORMAT_ALPHA8) {
        s.buf[i] = p.a;
        return;
    }
    uint8_t *q = s.buf + 4 * i;
    switch (s.fmt) {
        case Z2D_FORMAT_ARGB: q[0] = p.b; q[1] = p.g; q[2] = p.r; q[3] = p.a; break;
        case Z2D_FORMAT_XRGB: q[0] = p.b; q[1] = p.g; q[2] = p.r; q[3] = 0; break;
        case Z2D_FORMAT_RGB: q[0] = p.r; q[1] = p.g; q[2] = p.b; q[3] = 0; break;
        default: q[0] = p.r; q[1] = p.g; q[2] = p.b; q[3] = p.a; break;
    }
}

// T.fromPixel(p): RGBA_T(T).fromPixel (src/pixel.zig:399-433) and
// Alpha(T).fromPixel (src/pixel.zig:569-577).
Px convert_px(const Px &p, int to) {
    if (p.fmt == to) return p;
    Px o{to, 0, 0, 0, 0};
    if (fmt_has_color(to)) {
        if (fmt_has_color(p.fmt)) {
            o.r = p.r; o.g = p.g; o.b = p.b;
            o.a = fmt_has_alpha(p.fmt) ? p.a : 255;
        } else {
            o.a = (uint8_t)scale_alpha(p.a, fmt_bits(p.fmt), 8);  // Alpha8.fromPixel(p).a
        }
        if (!fmt_has_alpha(to)) o.a = 0;
        return o;
    }
    // alpha target
    int tb = fmt_bits(to);
    if (p.fmt == Z2D_FORMAT_XRGB || p.fmt == Z2D_FORMAT_RGB) {
        o.a = fmt_max(to);
    } else {
        int fb = (p.fmt == Z2D_FORMAT_ARGB || p.fmt == Z2D_FORMAT_RGBA) ? 8 : fmt_bits(p.fmt);
        o.a = (uint8_t)scale_alpha(p.a, fb, tb);
    }
    return o;
}

// RGBA16.fromPixelT / RGBA16Vec.fromStride lane (src/compositor.zig:675-682,
// 718-747, 861-934): colorless formats give r=g=b=0, alphaless give a=255.
I16 to_i16(const Px &p) {
    I16 v{0, 0, 0, 0};
    if (fmt_has_color(p.fmt)) {
        v.r = p.r; v.g = p.g; v.b = p.b;
        v.a = fmt_has_alpha(p.fmt) ? p.a : 255;
    } else {
        v.a = (uint16_t)scale_alpha(p.a, fmt_bits(p.fmt), 8);
    }
    return v;
}

// RGBA16.toPixelT / RGBA16Vec.toStride lane (src/compositor.zig:688-698,
// 806-833): values are truncated to u8 (@intCast) and scaled down for
// sub-byte alpha.
Px from_i16(const I16 &v, int fmt) {
    Px p{fmt, 0, 0, 0, 0};
    if (fmt_has_color(fmt)) {
        p.r = (uint8_t)v.r; p.g = (uint8_t)v.g; p.b = (uint8_t)v.b;
        p.a = fmt_has_alpha(fmt) ? (uint8_t)v.a : 0;
    } else {
        p.a = (uint8_t)scale_alpha((uint8_t)v.a, 8, fmt_bits(fmt));
    }
    return p;
}

I16 load_i16(const Sfc &s, size_t i) { return to_i16(raw_get(s, i)); }
void store_i16(Sfc &s, size_t i, const I16 &v) { raw_set(s, i, from_i16(v, s.fmt)); }

Px px_from_abi(const z2d_pixel &p) { return Px{p.format, p.r, p.g, p.b, p.a}; }

// pixel.RGBA.fromPixel then RGBA16Vec.fromPixel (src/compositor.zig:708-716)
I16 i16_from_pixel(const Px &p) { return to_i16(convert_px(p, Z2D_FORMAT_RGBA)); }

// ===================================================================
// Integer operators                     src/compositor.zig:1158-1568
// ===================================================================
// u16 lanes; results wrap at 16 bits as z2d's u16 vectors do.

inline int32_t mul(int32_t a, int32_t b) { return (a * b) / 255; }        // :1525-1530
inline int32_t inv(int32_t a) { return 255 - a; }                          // :1543
inline int32_t invMul(int32_t a, int32_t b) { return mul(a, inv(b)); }     // :1555
inline int32_t rInvMul(int32_t a, int32_t b) { return mul(a, 255 + b); }  // :1561
inline uint16_t w16(int32_t v) { return (uint16_t)v; }

uint16_t overlay_ch(int32_t sca, int32_t dca, int32_t sa, int32_t da) {  // :1331-1394
    if (w16(dca * 2) <= da) return w16(mul(sca * 2, dca) + invMul(sca, da) + invMul(dca, sa));
    return w16(rInvMul(sca, da) + rInvMul(dca, sa) - mul(dca * 2, sca) - mul(da, sa));
}
uint16_t hardlight_ch(int32_t sca, int32_t dca, int32_t sa, int32_t da) {  // :1420-1491
    if (w16(sca * 2) <= sa) return w16(mul(sca * 2, dca) + invMul(sca, da) + invMul(dca, sa));
    return w16(rInvMul(sca, da) + rInvMul(dca, sa) - mul(sa, da) - mul(sca * 2, dca));
}

I16 int_op(int op, I16 d, I16 s) {
    I16 o{0, 0, 0, 0};
    const int32_t dr = d.r, dg = d.g, db = d.b, da = d.a;
    const int32_t sr = s.r, sg = s.g, sb = s.b, sa = s.a;
    const uint16_t a_union = w16(sa + da - mul(sa, da));
    switch (op) {
        case Z2D_OP_CLEAR: return o;
        case Z2D_OP_SRC: return s;
        case Z2D_OP_DST: return d;
        case Z2D_OP_SRC_OVER:
            o.r = w16(sr + invMul(dr, sa)); o.g = w16(sg + invMul(dg, sa));
            o.b = w16(sb + invMul(db, sa)); o.a = a_union; return o;
        case Z2D_OP_DST_OVER:
            o.r = w16(dr + invMul(sr, da)); o.g = w16(dg + invMul(sg, da));
            o.b = w16(db + invMul(sb, da)); o.a = a_union; return o;
        case Z2D_OP_SRC_IN:
            o.r = w16(mul(sr, da)); o.g = w16(mul(sg, da)); o.b = w16(mul(sb, da)); o.a = w16(mul(sa, da)); return o;
        case Z2D_OP_DST_IN:
            o.r = w16(mul(dr, sa)); o.g = w16(mul(dg, sa)); o.b = w16(mul(db, sa)); o.a = w16(mul(da, sa)); return o;
        case Z2D_OP_SRC_OUT:
            o.r = w16(invMul(sr, da)); o.g = w16(invMul(sg, da)); o.b = w16(invMul(sb, da)); o.a = w16(invMul(sa, da)); return o;
        case Z2D_OP_DST_OUT:
            o.r = w16(invMul(dr, sa)); o.g = w16(invMul(dg, sa)); o.b = w16(invMul(db, sa)); o.a = w16(invMul(da, sa)); return o;
        case Z2D_OP_SRC_ATOP:
            o.r = w16(mul(sr, da) + invMul(dr, sa)); o.g = w16(mul(sg, da) + invMul(dg, sa));
            o.b = w16(mul(sb, da) + invMul(db, sa)); o.a = (uint16_t)da; return o;
        case Z2D_OP_DST_ATOP:
            o.r = w16(mul(dr, sa) + invMul(sr, da)); o.g = w16(mul(dg, sa) + invMul(sg, da));
            o.b = w16(mul(db, sa) + invMul(sb, da)); o.a = (uint16_t)sa; return o;
        case Z2D_OP_XOR:
            o.r = w16(invMul(sr, da) + invMul(dr, sa)); o.g = w16(invMul(sg, da) + invMul(dg, sa));
            o.b = w16(invMul(sb, da) + invMul(db, sa)); o.a = w16(invMul(sa, da) + invMul(da, sa)); return o;
        case Z2D_OP_PLUS:
            o.r = w16(std::min(255, sr + dr)); o.g = w16(std::min(255, sg + dg));
            o.b = w16(std::min(255, sb + db)); o.a = w16(std::min(255, sa + da)); return o;
        case Z2D_OP_MULTIPLY:
            o.r = w16(mul(sr, dr) + invMul(sr, da) + invMul(dr, sa));
            o.g = w16(mul(sg, dg) + invMul(sg, da) + invMul(dg, sa));
            o.b = w16(mul(sb, db) + invMul(sb, da) + invMul(db, sa)); o.a = a_union; return o;
        case Z2D_OP_SCREEN:
            o.r = w16(sr + dr - mul(sr, dr)); o.g = w16(sg + dg - mul(sg, dg));
            o.b = w16(sb + db - mul(sb, db)); o.a = a_union; return o;
        case Z2D_OP_OVERLAY:
            o.r = overlay_ch(sr, dr, sa, da); o.g = overlay_ch(sg, dg, sa, da);
            o.b = overlay_ch(sb, db, sa, da); o.a = a_union; return o;
        case Z2D_OP_DARKEN:
            o.r = w16(std::min(mul(sr, da), mul(dr, sa)) + invMul(sr, da) + invMul(dr, sa));
            o.g = w16(std::min(mul(sg, da), mul(dg, sa)) + invMul(sg, da) + invMul(dg, sa));
            o.b = w16(std::min(mul(sb, da), mul(db, sa)) + invMul(sb, da) + invMul(db, sa));
            o.a = a_union; return o;
        case Z2D_OP_LIGHTEN:
            o.r = w16(std::max(mul(sr, da), mul(dr, sa)) + invMul(sr, da) + invMul(dr, sa));
            o.g = w16(std::max(mul(sg, da), mul(dg, sa)) + invMul(sg, da) + invMul(dg, sa));
            o.b = w16(std::max(mul(sb, da), mul(db, sa)) + invMul(sb, da) + invMul(db, sa));
            o.a = a_union; return o;
        case Z2D_OP_HARD_LIGHT:
            o.r = hardlight_ch(sr, dr, sa, da); o.g = hardlight_ch(sg, dg, sa, da);
            o.b = hardlight_ch(sb, db, sa, da); o.a = a_union; return o;
        case Z2D_OP_DIFFERENCE:
            o.r = w16(sr + dr - 2 * std::min(mul(sr, da), mul(dr, sa)));
            o.g = w16(sg + dg - 2 * std::min(mul(sg, da), mul(dg, sa)));
            o.b = w16(sb + db - 2 * std::min(mul(sb, da), mul(db, sa)));
            o.a = a_union; return o;
        case Z2D_OP_EXCLUSION:
            o.r = w16((mul(sr, da) + mul(dr, sa) - 2 * mul(sr, dr)) + invMul(sr, da) + invMul(dr, sa));
            o.g = w16((mul(sg, da) + mul(dg, sa) - 2 * mul(sg, dg)) + invMul(sg, da) + invMul(dg, sa));
            o.b = w16((mul(sb, da) + mul(db, sa) - 2 * mul(sb, db)) + invMul(sb, da) + invMul(db, sa));
            o.a = a_union; return o;
        default:  // color_dodge, color_burn, soft_light, hue, saturation, color, luminosity -> clear (:1179-1188)
            return o;
    }
}

bool requires_float(int op) {  // src/compositor.zig:165-177
    switch (op) {
        case Z2D_OP_COLOR_DODGE: case Z2D_OP_COLOR_BURN: case Z2D_OP_SOFT_LIGHT:
        case Z2D_OP_HUE: case Z2D_OP_SATURATION: case Z2D_OP_COLOR: case Z2D_OP_LUMINOSITY:
            return true;
        default: return false;
    }
}
bool is_bounded(int op) {  // src/compositor.zig:187-196
    return !(op == Z2D_OP_SRC_IN || op == Z2D_OP_DST_IN || op == Z2D_OP_SRC_OUT || op == Z2D_OP_DST_ATOP);
}

// ===================================================================
// Float operators (vector form)          src/compositor.zig:1571-2440
// ===================================================================
struct F4 {
    float r, g, b, a;
};

// Zig @min/@max on floats return the non-NaN operand, like fminf/fmaxf.
inline float fmin2(float a, float b) { return std::fmin(a, b); }
inline float fmax2(float a, float b) { return std::fmax(a, b); }
inline float fmin3(float a, float b, float c) { return fmin2(fmin2(a, b), c); }
inline float fmax3(float a, float b, float c) { return fmax2(fmax2(a, b), c); }

float f_overlay(float sca, float dca, float sa, float da) {  // :1751-1804
    if (2.0f * dca <= da) return 2.0f * sca * dca + sca * (1.0f - da) + dca * (1.0f - sa);
    return sca * (1.0f + da) + dca * (1.0f + sa) - 2.0f * dca * sca - da * sa;
}
float f_dodge(float sca, float dca, float sa, float da) {  // :1826-1902
    if (sca == sa && dca == 0.0f) return sca * (1.0f - da);
    if (sca == sa) return sa * da + sca * (1.0f - da) + dca * (1.0f - sa);
    return sa * da * fmin2(1.0f, dca / da * sa / (sa - sca)) + sca * (1.0f - da) + dca * (1.0f - sa);
}
float f_burn(float sca, float dca, float sa, float da) {  // :1904-1981
    // p0 is declared (sca, dca, da) but called with sa as its third argument
    // (:1915, :1932), so the first case tests dca == sa.
    if (sca == 0.0f && dca == sa) return sa * da + dca * (1.0f - sa);
    if (sca == 0.0f) return dca * (1.0f - sa);
    return sa * da * (1.0f - fmin2(1.0f, (1.0f - dca / da) * sa / sca)) + sca * (1.0f - da) + dca * (1.0f - sa);
}
float f_hardlight(float sca, float dca, float sa, float da) {  // :1983-2044
    if (2.0f * sca <= sa) return 2.0f * sca * dca + sca * (1.0f - da) + dca * (1.0f - sa);
    return sca * (1.0f + da) + dca * (1.0f + sa) - sa * da - 2.0f * sca * dca;
}
float f_softlight(float sca, float dca, float sa, float da) {  // :2046-2150
    if (da == 0.0f) return sca;
    if (2.0f * sca <= sa) {
        const float m = dca / da;
        return dca * (sa + (2.0f * sca - sa) * (1.0f - m)) + sca * (1.0f - da) + dca * (1.0f - sa);
    }
    if (4.0f * dca <= da) {
        const float m = dca / da;
        return dca * sa + da * (2.0f * sca - sa) * (4.0f * m * (4.0f * m + 1.0f) * (m - 1.0f) + 7.0f * m) +
               sca * (1.0f - da) + dca * (1.0f - sa);
    }
    const float m = dca / da;
    return da * (2.0f * sca - sa) * (std::sqrt(m) - m) + sca - sca * da + dca;
}

struct F3 {
    float r, g, b;
};
float ns_lum(F3 c) { return c.r * 0.3f + c.g * 0.59f + c.b * 0.11f; }  // :2263-2268
float ns_sat(F3 c) { return fmax3(c.r, c.g, c.b) - fmin3(c.r, c.g, c.b); }
F3 ns_set_lum(F3 c, float l) {  // :2365-2372
    const float d = l - ns_lum(c);
    return F3{c.r + d, c.g + d, c.b + d};
}
F3 ns_set_sat(F3 c, float s) {  // :2374-2420
    const float n = fmin3(c.r, c.g, c.b), x = fmax3(c.r, c.g, c.b), d = x - n;
    auto sc = [&](float v) { return d == 0.0f ? 0.0f : (v - n) * s / d; };
    return F3{sc(c.r), sc(c.g), sc(c.b)};
}
// clipColor, vector form (:2272-2307): the x > a case overrides the n < 0
// case when both hold (the scalar form would keep the n < 0 result).
F3 ns_clip(F3 c, float a) {
    const float l = ns_lum(c), n = fmin3(c.r, c.g, c.b), x = fmax3(c.r, c.g, c.b);
    auto ch = [&](float cv) {
        const float t_l_n = l - n, t_x_l = x - l;
        float r = cv;
        if (n < 0.0f) r = (t_l_n == 0.0f) ? 0.0f : l + ((cv - l) * l) / t_l_n;
        if (x > a) r = (t_x_l == 0.0f) ? 0.0f : l + ((cv - l) * (a - l)) / t_x_l;
        return r;
    };
    return F3{ch(c.r), ch(c.g), ch(c.b)};
}
F4 ns_out(F3 c, F4 d, F4 s) {  // toRGBA :2249-2257
    return F4{s.r * (1.0f - d.a) + d.r * (1.0f - s.a) + c.r, s.g * (1.0f - d.a) + d.g * (1.0f - s.a) + c.g,
              s.b * (1.0f - d.a) + d.b * (1.0f - s.a) + c.b, s.a + d.a - s.a * d.a};
}

F4 float_op(int op, F4 d, F4 s) {
    const float a_union = s.a + d.a - s.a * d.a;
    switch (op) {
        case Z2D_OP_CLEAR: return F4{0, 0, 0, 0};
        case Z2D_OP_SRC: return s;
        case Z2D_OP_DST: return d;
        case Z2D_OP_SRC_OVER:
            return F4{s.r + d.r * (1.0f - s.a), s.g + d.g * (1.0f - s.a), s.b + d.b * (1.0f - s.a), a_union};
        case Z2D_OP_DST_OVER:
            return F4{d.r + s.r * (1.0f - d.a), d.g + s.g * (1.0f - d.a), d.b + s.b * (1.0f - d.a), a_union};
        case Z2D_OP_SRC_IN: return F4{s.r * d.a, s.g * d.a, s.b * d.a, s.a * d.a};
        case Z2D_OP_DST_IN: return F4{d.r * s.a, d.g * s.a, d.b * s.a, s.a * d.a};
        case Z2D_OP_SRC_OUT:
            return F4{s.r * (1.0f - d.a), s.g * (1.0f - d.a), s.b * (1.0f - d.a), s.a * (1.0f - d.a)};
        case Z2D_OP_DST_OUT:
            return F4{d.r * (1.0f - s.a), d.g * (1.0f - s.a), d.b * (1.0f - s.a), d.a * (1.0f - s.a)};
        case Z2D_OP_SRC_ATOP:
            return F4{s.r * d.a + d.r * (1.0f - s.a), s.g * d.a + d.g * (1.0f - s.a), s.b * d.a + d.b * (1.0f - s.a), d.a};
        case Z2D_OP_DST_ATOP:
            return F4{d.r * s.a + s.r * (1.0f - d.a), d.g * s.a + s.g * (1.0f - d.a), d.b * s.a + s.b * (1.0f - d.a), s.a};
        case Z2D_OP_XOR:
            return F4{s.r * (1.0f - d.a) + d.r * (1.0f - s.a), s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      s.b * (1.0f - d.a) + d.b * (1.0f - s.a), s.a + d.a - 2.0f * s.a * d.a};
        case Z2D_OP_PLUS:
            return F4{fmin2(1.0f, s.r + d.r), fmin2(1.0f, s.g + d.g), fmin2(1.0f, s.b + d.b), fmin2(1.0f, s.a + d.a)};
        case Z2D_OP_MULTIPLY:
            return F4{s.r * d.r + s.r * (1.0f - d.a) + d.r * (1.0f - s.a), s.g * d.g + s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      s.b * d.b + s.b * (1.0f - d.a) + d.b * (1.0f - s.a), a_union};
        case Z2D_OP_SCREEN:
            return F4{s.r + d.r - s.r * d.r, s.g + d.g - s.g * d.g, s.b + d.b - s.b * d.b, a_union};
        case Z2D_OP_OVERLAY:
            return F4{f_overlay(s.r, d.r, s.a, d.a), f_overlay(s.g, d.g, s.a, d.a), f_overlay(s.b, d.b, s.a, d.a), a_union};
        case Z2D_OP_DARKEN:
            return F4{fmin2(s.r * d.a, d.r * s.a) + s.r * (1.0f - d.a) + d.r * (1.0f - s.a),
                      fmin2(s.g * d.a, d.g * s.a) + s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      fmin2(s.b * d.a, d.b * s.a) + s.b * (1.0f - d.a) + d.b * (1.0f - s.a), a_union};
        case Z2D_OP_LIGHTEN:
            return F4{fmax2(s.r * d.a, d.r * s.a) + s.r * (1.0f - d.a) + d.r * (1.0f - s.a),
                      fmax2(s.g * d.a, d.g * s.a) + s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      fmax2(s.b * d.a, d.b * s.a) + s.b * (1.0f - d.a) + d.b * (1.0f - s.a), a_union};
        case Z2D_OP_COLOR_DODGE:
            return F4{f_dodge(s.r, d.r, s.a, d.a), f_dodge(s.g, d.g, s.a, d.a), f_dodge(s.b, d.b, s.a, d.a), a_union};
        case Z2D_OP_COLOR_BURN:
            return F4{f_burn(s.r, d.r, s.a, d.a), f_burn(s.g, d.g, s.a, d.a), f_burn(s.b, d.b, s.a, d.a), a_union};
        case Z2D_OP_HARD_LIGHT:
            return F4{f_hardlight(s.r, d.r, s.a, d.a), f_hardlight(s.g, d.g, s.a, d.a), f_hardlight(s.b, d.b, s.a, d.a), a_union};
        case Z2D_OP_SOFT_LIGHT:
            return F4{f_softlight(s.r, d.r, s.a, d.a), f_softlight(s.g, d.g, s.a, d.a), f_softlight(s.b, d.b, s.a, d.a), a_union};
        case Z2D_OP_DIFFERENCE:
            return F4{s.r + d.r - 2.0f * fmin2(s.r * d.a, d.r * s.a), s.g + d.g - 2.0f * fmin2(s.g * d.a, d.g * s.a),
                      s.b + d.b - 2.0f * fmin2(s.b * d.a, d.b * s.a), a_union};
        case Z2D_OP_EXCLUSION:
            return F4{(s.r * d.a + d.r * s.a - 2.0f * s.r * d.r) + s.r * (1.0f - d.a) + d.r * (1.0f - s.a),
                      (s.g * d.a + d.g * s.a - 2.0f * s.g * d.g) + s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      (s.b * d.a + d.b * s.a - 2.0f * s.b * d.b) + s.b * (1.0f - d.a) + d.b * (1.0f - s.a), a_union};
        case Z2D_OP_HUE: {  // :2176-2183
            F3 c = F3{s.r * s.a, s.g * s.a, s.b * s.a};
            const F3 cd = F3{d.r, d.g, d.b};
            c = ns_set_sat(c, ns_sat(cd) * s.a);
            c = ns_set_lum(c, ns_lum(cd) * s.a);
            c = ns_clip(c, s.a * d.a);
            return ns_out(c, d, s);
        }
        case Z2D_OP_SATURATION: {  // :2185-2193
            F3 c = F3{d.r * s.a, d.g * s.a, d.b * s.a};
            const F3 cs = F3{s.r, s.g, s.b}, cd = F3{d.r, d.g, d.b};
            c = ns_set_sat(c, ns_sat(cs) * d.a);
            c = ns_set_lum(c, ns_lum(cd) * s.a);
            c = ns_clip(c, s.a * d.a);
            return ns_out(c, d, s);
        }
        case Z2D_OP_COLOR: {  // :2195-2201
            F3 c = F3{s.r * d.a, s.g * d.a, s.b * d.a};
            const F3 cd = F3{d.r, d.g, d.b};
            c = ns_set_lum(c, ns_lum(cd) * s.a);
            c = ns_clip(c, s.a * d.a);
            return ns_out(c, d, s);
        }
        case Z2D_OP_LUMINOSITY: {  // :2203-2209
            F3 c = F3{d.r * s.a, d.g * s.a, d.b * s.a};
            const F3 cs = F3{s.r, s.g, s.b};
            c = ns_set_lum(c, ns_lum(cs) * d.a);
            c = ns_clip(c, s.a * d.a);
            return ns_out(c, d, s);
        }
        default: return F4{0, 0, 0, 0};
    }
}

// decodeRGBAVecRaw / encodeRGBAVecRaw (src/internal/color_vector.zig:266-284)
F4 decode_raw(I16 v) { return F4{(float)v.r / 255.0f, (float)v.g / 255.0f, (float)v.b / 255.0f, (float)v.a / 255.0f}; }
uint16_t enc_ch(float x) {
    const float r = std::round(255.0f * x);
    if (!(r == r)) return 0;  // NaN: undefined in z2d; pinned to 0 here
    return (uint16_t)(int32_t)r;
}
I16 encode_raw(F4 v) { return I16{enc_ch(v.r), enc_ch(v.g), enc_ch(v.b), enc_ch(v.a)}; }

// ===================================================================
// Colors                  src/color.zig, src/internal/color_vector.zig
// ===================================================================
const float kGamma = 2.2f;             // src/color.zig:206-209
const float kInvGamma = 1.0f / 2.2f;

// -------------------------------------------------------------------
// The Zig standard-library math z2d calls, restated so that the oracle
// computes what z2d computes (not the host libm's correctly rounded
// results).  z2d is a freestanding Zig library (no libc is linked), so
// Zig's @exp / @log on f32 lower to compiler_rt's expf / logf, which are
// Zig ports of musl's expf.c / logf.c (themselves FreeBSD msun e_expf.c /
// e_logf.c); std.math.pow (lib/std/math/pow.zig) is Zig's port of Go's
// math.Pow; std.math.atan2 / atan (lib/std/math/atan2.zig, atan.zig) are
// ports of musl's atan2.c / atan.c (FreeBSD e_atan2.c / s_atan.c).
// Written from those published algorithms; every constant below was
// checked against its bit pattern, and expf / logf / atan against
// high-precision values (< 1 ulp).
// -------------------------------------------------------------------
uint32_t f32_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
float f32_from(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
uint32_t f64_hi(double d) {
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return (uint32_t)(u >> 32);
}
uint32_t f64_lo(double d) {
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return (uint32_t)u;
}

// std.math.scalbn / ldexp for f32: x * 2^n (exact while the result is
// normal; below that, rounded once by the final multiply).
float zscalbnf(float x, int n) {
    if (n > 127) {
        x *= f32_from(0x7F000000u);  // 2^127
        n -= 127;
        if (n > 127) {
            x *= f32_from(0x7F000000u);
            n -= 127;
            if (n > 127) n = 127;
        }
    } else if (n < -126) {
        x *= f32_from(0x0C800000u);  // 2^-102
        n += 102;
        if (n < -126) {
            x *= f32_from(0x0C800000u);
            n += 102;
            if (n < -126) n = -126;
        }
    }
    return x * f32_from((uint32_t)(0x7F + n) << 23);
}

// compiler_rt expf (musl src/math/expf.c, pre-2017 FreeBSD form):
// x = k*ln2 + r, exp(r) from a degree-2 rational approximation.
float zexpf(float x) {
    const float half[2] = {0.5f, -0.5f};
    const float ln2hi = f32_from(0x3F317200u), ln2lo = f32_from(0x35BFBE8Eu), invln2 = f32_from(0x3FB8AA3Bu);
    const float P1 = 11184783.0f / 67108864.0f;   //  0xaaaa8f * 2^-26
    const float P2 = -11883029.0f / 4294967296.0f;  // -0xb55215 * 2^-32
    uint32_t hx = f32_bits(x);
    const int sign = (int)(hx >> 31);
    hx &= 0x7FFFFFFFu;
    if (x != x) return x;
    if (hx >= 0x42AEAC50u) {                       // |x| >= 87.33655
        if (hx > 0x7F800000u) return x;            // NaN
        if (hx >= 0x42B17218u && !sign) return x * f32_from(0x7F000000u);  // overflow
        if (sign && hx >= 0x42CFF1B5u) return 0.0f;  // x <= -103.972084
    }
    int k;
    float hi, lo;
    if (hx > 0x3EB17218u) {                        // |x| > 0.5 ln2
        if (hx > 0x3F851592u) k = (int)(invln2 * x + half[sign]);  // |x| > 1.5 ln2
        else k = 1 - sign - sign;
        const float fk = (float)k;
        hi = x - fk * ln2hi;
        lo = fk * ln2lo;
        x = hi - lo;
    } else if (hx > 0x39000000u) {                 // |x| > 2^-14
        k = 0;
        hi = x;
        lo = 0.0f;
    } else {
        return 1.0f + x;
    }
    const float xx = x * x;
    const float c = x - xx * (P1 + xx * P2);
    const float y = 1.0f + (x * c / (2.0f - c) - lo + hi);
    return k == 0 ? y : zscalbnf(y, k);
}

// compiler_rt logf (musl src/math/logf.c, pre-2017 FreeBSD form): x
// reduced into [sqrt(2)/2, sqrt(2)], log(1+f) = f - hfsq + s*(hfsq+R).
float zlogf(float x) {
    const float ln2_hi = f32_from(0x3F317180u), ln2_lo = f32_from(0x3717F7D1u);
    const float Lg1 = 11184810.0f / 16777216.0f;  // 0xaaaaaa * 2^-24
    const float Lg2 = 13420051.0f / 33554432.0f;  // 0xccce13 * 2^-25
    const float Lg3 = 9562606.0f / 33554432.0f;   // 0x91e9ee * 2^-25
    const float Lg4 = 16293414.0f / 67108864.0f;  // 0xf89e26 * 2^-26
    uint32_t ix = f32_bits(x);
    int k = 0;
    if (ix < 0x00800000u || (ix >> 31)) {
        if ((ix << 1) == 0) return -INFINITY;
        if (ix >> 31) return NAN;
        k -= 25;                                   // subnormal: scale up
        x *= f32_from(0x4C000000u);                // 2^25
        ix = f32_bits(x);
    } else if (ix >= 0x7F800000u) {
        return x;
    } else if (ix == 0x3F800000u) {
        return 0.0f;
    }
    ix += 0x3F800000u - 0x3F3504F3u;
    k += (int)(ix >> 23) - 0x7F;
    ix = (ix & 0x007FFFFFu) + 0x3F3504F3u;
    x = f32_from(ix);
    const float f = x - 1.0f;
    const float s = f / (2.0f + f);
    const float z = s * s;
    const float w = z * z;
    const float t1 = w * (Lg2 + w * Lg4);
    const float t2 = z * (Lg1 + w * Lg3);
    const float R = t2 + t1;
    const float hfsq = 0.5f * f * f;
    const float dk = (float)k;
    return s * (hfsq + R) + dk * ln2_lo - hfsq + f + dk * ln2_hi;
}

// std.math.frexp for f32: x = m * 2^e with m in [0.5, 1).
float zfrexpf(float x, int *e) {
    uint32_t u = f32_bits(x);
    int ex = (int)((u >> 23) & 0xFF);
    if (ex == 0) {
        if ((u << 1) == 0) {
            *e = 0;
            return x;
        }
        x *= f32_from(0x5F800000u);  // 2^64
        u = f32_bits(x);
        ex = (int)((u >> 23) & 0xFF) - 64;
    } else if (ex == 0xFF) {
        *e = 0;
        return x;
    }
    *e = ex - 126;
    return f32_from((u & 0x807FFFFFu) | 0x3F000000u);
}

// std.math.pow(f32, x, y) (lib/std/math/pow.zig, Go's math.Pow): special
// cases, then x^y = exp(yf*log(x)) * x^yi with yf in (-0.5, 0.5] and x^yi
// by repeated squaring of frexp(x), scaled by 2^ae at the end.  z2d calls
// it with y = 2.2 and 1/2.2 (src/color.zig:336-351,
// src/internal/color_vector.zig:210-240).
bool zis_odd_int(float y) {
    if (std::fabs(y) >= 16777216.0f) return false;  // beyond 2^24 every float is even
    const float t = std::trunc(y);
    if (t != y) return false;
    return ((int64_t)t & 1) != 0;
}
float zpow(float x, float y) {
    if (y == 0.0f || x == 1.0f) return 1.0f;
    if (x != x || y != y) return NAN;
    if (y == 1.0f) return x;
    if (x == 0.0f) {
        if (y < 0.0f) return zis_odd_int(y) ? std::copysign(INFINITY, x) : INFINITY;
        return zis_odd_int(y) ? x : 0.0f;
    }
    if (std::isinf(y)) {
        if (x == -1.0f) return 1.0f;
        return ((std::fabs(x) < 1.0f) == (y > 0.0f)) ? 0.0f : INFINITY;
    }
    if (std::isinf(x)) {
        if (x < 0.0f) return zpow(1.0f / x, -y);  // pow(-0, -y)
        return y < 0.0f ? 0.0f : INFINITY;
    }
    if (y == 0.5f) return std::sqrt(x);
    if (y == -0.5f) return 1.0f / std::sqrt(x);
    float yi = std::trunc(std::fabs(y));
    float yf = std::fabs(y) - yi;
    if (yf != 0.0f && x < 0.0f) return NAN;
    if (yi >= 2147483648.0f) {
        if (x == -1.0f) return 1.0f;
        return ((std::fabs(x) < 1.0f) == (y > 0.0f)) ? 0.0f : INFINITY;
    }
    float a1 = 1.0f;
    int ae = 0;
    if (yf != 0.0f) {
        if (yf > 0.5f) {
            yf -= 1.0f;
            yi += 1.0f;
        }
        a1 = zexpf(yf * zlogf(x));
    }
    int xe;
    float x1 = zfrexpf(x, &xe);
    for (int32_t i = (int32_t)yi; i != 0; i >>= 1) {
        if (xe < -(1 << 9) || (1 << 9) < xe) {
            ae += xe;
            break;
        }
        if (i & 1) {
            a1 *= x1;
            ae += xe;
        }
        x1 *= x1;
        xe <<= 1;
        if (x1 < 0.5f) {
            x1 += x1;
            xe -= 1;
        }
    }
    if (y < 0.0f) {
        a1 = 1.0f / a1;
        ae = -ae;
    }
    return zscalbnf(a1, ae);
}

// std.math.atan for f64 (musl src/math/atan.c / FreeBSD s_atan.c):
// reduction to |x| < 7/16 around atan(0.5), atan(1), atan(1.5), atan(inf),
// then an odd polynomial of degree 23 split in two halves.
double zatan(double x) {
    static const double atanhi[4] = {4.63647609000806093515e-01, 7.85398163397448278999e-01,
                                     9.82793723247329054082e-01, 1.57079632679489655800e+00};
    static const double atanlo[4] = {2.26987774529616870924e-17, 3.06161699786838301793e-17,
                                     1.39033110312309984516e-17, 6.12323399573676603587e-17};
    static const double aT[11] = {3.33333333333329318027e-01, -1.99999999998764832476e-01,
                                  1.42857142725034663711e-01, -1.11111104054623557880e-01,
                                  9.09088713343650656196e-02, -7.69187620504482999495e-02,
                                  6.66107313738753120669e-02, -5.83357013379057348645e-02,
                                  4.97687799461593236017e-02, -3.65315727442169155270e-02,
                                  1.62858201153657823623e-02};
    uint32_t ix = f64_hi(x);
    const uint32_t sign = ix >> 31;
    ix &= 0x7FFFFFFFu;
    if (ix >= 0x44100000u) {                       // |x| >= 2^66
        if (x != x) return x;
        const double z = atanhi[3] + 0x1p-120;
        return sign ? -z : z;
    }
    int id;
    if (ix < 0x3FDC0000u) {                        // |x| < 0.4375
        if (ix < 0x3E400000u) return x;            // |x| < 2^-27
        id = -1;
    } else {
        x = std::fabs(x);
        if (ix < 0x3FF30000u) {                    // |x| < 1.1875
            if (ix < 0x3FE60000u) {                // 7/16 <= |x| < 11/16
                id = 0;
                x = (2.0 * x - 1.0) / (2.0 + x);
            } else {                               // 11/16 <= |x| < 19/16
                id = 1;
                x = (x - 1.0) / (x + 1.0);
            }
        } else if (ix < 0x40038000u) {             // |x| < 2.4375
            id = 2;
            x = (x - 1.5) / (1.0 + 1.5 * x);
        } else {                                   // 2.4375 <= |x| < 2^66
            id = 3;
            x = -1.0 / x;
        }
    }
    const double z = x * x;
    const double w = z * z;
    const double s1 = z * (aT[0] + w * (aT[2] + w * (aT[4] + w * (aT[6] + w * (aT[8] + w * aT[10])))));
    const double s2 = w * (aT[1] + w * (aT[3] + w * (aT[5] + w * (aT[7] + w * aT[9]))));
    if (id < 0) return x - x * (s1 + s2);
    const double r = atanhi[id] - ((x * (s1 + s2) - atanlo[id]) - x);
    return sign ? -r : r;
}

// std.math.atan2 for f64 (musl src/math/atan2.c / FreeBSD e_atan2.c); the
// conic gradient's angle (src/gradient.zig:739).
double zatan2(double y, double x) {
    const double pi = 3.1415926535897931160E+00, pi_lo = 1.2246467991473531772E-16;
    if (x != x || y != y) return x + y;
    uint32_t ix = f64_hi(x), iy = f64_hi(y);
    const uint32_t lx = f64_lo(x), ly = f64_lo(y);
    if (((ix - 0x3FF00000u) | lx) == 0) return zatan(y);  // x == 1.0
    const uint32_t m = ((iy >> 31) & 1u) | ((ix >> 30) & 2u);
    ix &= 0x7FFFFFFFu;
    iy &= 0x7FFFFFFFu;
    if ((iy | ly) == 0) {
        if (m <= 1) return y;
        return m == 2 ? pi : -pi;
    }
    if ((ix | lx) == 0) return (m & 1) ? -pi / 2 : pi / 2;
    if (ix == 0x7FF00000u) {
        if (iy == 0x7FF00000u) {
            switch (m) {
                case 0: return pi / 4;
                case 1: return -pi / 4;
                case 2: return 3 * pi / 4;
                default: return -3 * pi / 4;
            }
        }
        switch (m) {
            case 0: return 0.0;
            case 1: return -0.0;
            case 2: return pi;
            default: return -pi;
        }
    }
    if (ix + (64u << 20) < iy || iy == 0x7FF00000u) return (m & 1) ? -pi / 2 : pi / 2;
    double z;
    if ((m & 2) && iy + (64u << 20) < ix) z = 0.0;
    else z = zatan(std::fabs(y / x));
    switch (m) {
        case 0: return z;
        case 1: return -z;
        case 2: return pi - (z - pi_lo);
        default: return (z - pi_lo) - pi;
    }
}

// Zig @mod on floats: fmod, then shifted into [0, b) when the numerator is
// negative.
float zmodf(float a, float b) {
    const float r = std::fmod(a, b);
    return a < 0.0f ? std::fmod(r + b, b) : r;
}
double zmod(double a, double b) {
    const double r = std::fmod(a, b);
    return a < 0.0 ? std::fmod(r + b, b) : r;
}

struct RGBf {
    float r, g, b, a;
};
struct HSLf {
    float h, s, l, a;
};

RGBf hsl_to_rgb(HSLf c);

// LinearRGB.fromColor (src/color.zig:227-249); gamma of linear is 1, so
// applyGamma there is pow(x, 1) = x.
RGBf linear_from_color(const z2d_color &c) {
    RGBf o{c.c[0], c.c[1], c.c[2], c.c[3]};
    if (c.space == Z2D_COLOR_SRGB) {
        o.r = zpow(o.r, kGamma); o.g = zpow(o.g, kGamma); o.b = zpow(o.b, kGamma);
    } else if (c.space == Z2D_COLOR_HSL) {
        o = hsl_to_rgb(HSLf{c.c[0], c.c[1], c.c[2], c.c[3]});
    }
    return o;
}
// SRGB.fromColor (same lines, profile srgb)
RGBf srgb_from_color(const z2d_color &c) {
    if (c.space == Z2D_COLOR_SRGB) return RGBf{c.c[0], c.c[1], c.c[2], c.c[3]};
    RGBf lin = (c.space == Z2D_COLOR_HSL) ? hsl_to_rgb(HSLf{c.c[0], c.c[1], c.c[2], c.c[3]})
                                          : RGBf{c.c[0], c.c[1], c.c[2], c.c[3]};
    return RGBf{zpow(lin.r, kInvGamma), zpow(lin.g, kInvGamma), zpow(lin.b, kInvGamma), lin.a};
}
// HSL.fromRGB (src/color.zig:436-471)
HSLf hsl_from_rgb(RGBf s) {
    const float mx = fmax2(s.r, fmax2(s.g, s.b));
    const float mn = fmin2(s.r, fmin2(s.g, s.b));
    const float range = mx - mn;
    const float light = (mn + mx) / 2.0f;
    float sat = (light == 0.0f || light == 1.0f) ? 0.0f : (mx - light) / fmin2(light, 1.0f - light);
    float hue = 0.0f;
    if (range != 0.0f) {
        if (mx == s.r) hue = 60.0f * zmodf((s.g - s.b) / range, 6.0f);
        else if (mx == s.g) hue = 60.0f * ((s.b - s.r) / range + 2.0f);
        else if (mx == s.b) hue = 60.0f * ((s.r - s.g) / range + 4.0f);
    }
    if (sat < 0.0f) {
        hue += 180.0f;
        if (hue >= 360.0f) hue -= 360.0f;
        sat = std::fabs(sat);
    }
    return HSLf{hue, sat, light, s.a};
}
HSLf hsl_from_color(const z2d_color &c) {  // src/color.zig:422-427
    if (c.space == Z2D_COLOR_HSL) return HSLf{c.c[0], c.c[1], c.c[2], c.c[3]};
    return hsl_from_rgb(linear_from_color(c));
}
// HSL.toRGB / toRGBChannel (src/color.zig:474-493; vector form
// color_vector.zig:362-383 is the same arithmetic)
float hsl_ch(float n, float hue, float sat, float light) {
    const float k = std::fmod(n + hue / 30.0f, 12.0f);
    const float a = sat * fmin2(light, 1.0f - light);
    return light - a * fmax2(-1.0f, fmin3(k - 3.0f, 9.0f - k, 1.0f));
}
RGBf hsl_to_rgb(HSLf c) {
    float hue = std::fmod(c.h, 360.0f);
    if (hue < 0.0f) hue += 360.0f;
    return RGBf{hsl_ch(0.0f, hue, c.s, c.l), hsl_ch(8.0f, hue, c.s, c.l), hsl_ch(4.0f, hue, c.s, c.l), c.a};
}

inline float lerpf(float a, float b, float t) { return a + (b - a) * t; }  // color_vector.zig:462-468

// RGBVec.interpolateVec (color_vector.zig:307-321): premultiplied lerp,
// then demultiplied.
RGBf rgb_interp(RGBf a, RGBf b, float t) {
    const RGBf am{a.r * a.a, a.g * a.a, a.b * a.a, a.a};
    const RGBf bm{b.r * b.a, b.g * b.a, b.b * b.a, b.a};
    RGBf o{lerpf(am.r, bm.r, t), lerpf(am.g, bm.g, t), lerpf(am.b, bm.b, t), lerpf(am.a, bm.a, t)};
    if (o.a == 0.0f) return RGBf{0, 0, 0, o.a};
    return RGBf{o.r / o.a, o.g / o.a, o.b / o.a, o.a};
}
// HSL.interpolateVec (color_vector.zig:404-448)
HSLf hsl_interp(HSLf a, HSLf b, float t, int polar) {
    const HSLf am{a.h, a.s * a.a, a.l * a.a, a.a};
    const HSLf bm{b.h, b.s * b.a, b.l * b.a, b.a};
    float ah = am.h, bh = bm.h;
    switch (polar) {
        case Z2D_INTERP_HSL_SHORTER: {
            const bool gt = bh - ah > 180.0f, lt = bh - ah < -180.0f;
            if (gt) ah = ah + 360.0f;
            if (lt) bh = bh + 360.0f;
            break;
        }
        case Z2D_INTERP_HSL_LONGER: {
            const float delta = bh - ah;
            const bool c1 = (0.0f < delta) && (delta < 180.0f);
            const bool c2 = (-180.0f < delta) && (delta <= 0.0f);
            if (c1) ah = ah + 360.0f;
            if (c2) bh = bh + 360.0f;
            break;
        }
        case Z2D_INTERP_HSL_INCREASING:
            if (bh < ah) bh = bh + 360.0f;
            break;
        default:
            if (ah < bh) ah = ah + 360.0f;
            break;
    }
    const float h = am.h + (bh - ah) * t;  // lerpPolar(a_mul.h, a_mul_h, b_mul_h, t)
    HSLf o{zmodf(h, 360.0f), lerpf(am.s, bm.s, t), lerpf(am.l, bm.l, t), lerpf(am.a, bm.a, t)};
    if (o.a == 0.0f) return HSLf{o.h, 0.0f, 0.0f, o.a};
    return HSLf{o.h, o.s / o.a, o.l / o.a, o.a};
}

// premultiply in u16 lanes (src/internal/pixel_vector.zig:18-25)
I16 premul16(I16 v) {
    return I16{(uint16_t)((uint32_t)(uint16_t)(v.r * v.a) / 255u), (uint16_t)((uint32_t)(uint16_t)(v.g * v.a) / 255u),
               (uint16_t)((uint32_t)(uint16_t)(v.b * v.a) / 255u), v.a};
}
// LinearRGB.encodeRGBAVec (color_vector.zig:244-262)
I16 encode_linear(RGBf c) { return premul16(I16{enc_ch(c.r), enc_ch(c.g), enc_ch(c.b), enc_ch(c.a)}); }

// interpolateEncodeVec (color_vector.zig:62-86) for one lane
I16 interp_encode(int method, const z2d_color &c0, const z2d_color &c1, float t) {
    if (method == Z2D_INTERP_LINEAR_RGB) {  // RGBVec(linear).interpolateEncodeVec :324-342
        const RGBf a = linear_from_color(c0), b = linear_from_color(c1);
        const RGBf am{a.r * a.a, a.g * a.a, a.b * a.a, a.a};
        const RGBf bm{b.r * b.a, b.g * b.a, b.b * b.a, b.a};
        return I16{enc_ch(lerpf(am.r, bm.r, t)), enc_ch(lerpf(am.g, bm.g, t)), enc_ch(lerpf(am.b, bm.b, t)),
                   enc_ch(lerpf(am.a, bm.a, t))};
    }
    if (method == Z2D_INTERP_SRGB) {  // demultiply, removeGamma, round, premultiply
        const RGBf d = rgb_interp(srgb_from_color(c0), srgb_from_color(c1), t);
        return encode_linear(RGBf{zpow(d.r, kGamma), zpow(d.g, kGamma), zpow(d.b, kGamma), d.a});
    }
    const HSLf h = hsl_interp(hsl_from_color(c0), hsl_from_color(c1), t, method);
    return encode_linear(hsl_to_rgb(h));
}
// interpolateVec (color_vector.zig:30-58): linear, demultiplied
RGBf interp_linear(int method, const z2d_color &c0, const z2d_color &c1, float t) {
    if (method == Z2D_INTERP_LINEAR_RGB) return rgb_interp(linear_from_color(c0), linear_from_color(c1), t);
    if (method == Z2D_INTERP_SRGB) {
        const RGBf d = rgb_interp(srgb_from_color(c0), srgb_from_color(c1), t);
        return RGBf{zpow(d.r, kGamma), zpow(d.g, kGamma), zpow(d.b, kGamma), d.a};
    }
    return hsl_to_rgb(hsl_interp(hsl_from_color(c0), hsl_from_color(c1), t, method));
}

// ===================================================================
// Gradients                                          src/gradient.zig
// ===================================================================
struct Stop {
    float offset;
    z2d_color color;
    size_t idx;
};
struct Grad {
    int type, method;
    std::vector<Stop> stops;
    bool has_tf;
    double tf[6];
    double g[6];
    // radial pre-calcs (:401-438)
    double inner_r, outer_r, cdx, cdy, dr, min_dr, a, inv_a;
    double angle;
};

Grad make_grad(const z2d_gradient &src) {
    Grad gr{};
    gr.type = src.type;
    gr.method = src.method;
    for (int i = 0; i < 6; i++) {
        gr.g[i] = src.geom[i];
        gr.tf[i] = src.transform[i];
    }
    static const double ident[6] = {1, 0, 0, 1, 0, 0};
    gr.has_tf = false;
    for (int i = 0; i < 6; i++)
        if (!(src.transform[i] == ident[i])) gr.has_tf = true;  // Transformation.equal
    // Stop.List.addAssumeCapacity (:797-811): clamp, stable sort by
    // (offset, insertion index)
    for (int i = 0; i < src.n_stops; i++) {
        Stop s;
        s.offset = fmax2(0.0f, fmin2(src.stops[i].offset, 1.0f));
        s.color = src.stops[i].color;
        s.idx = (size_t)i;
        gr.stops.push_back(s);
    }
    std::stable_sort(gr.stops.begin(), gr.stops.end(), [](const Stop &a, const Stop &b) {
        if (a.offset == b.offset) return a.idx < b.idx;
        return a.offset < b.offset;
    });
    if (gr.type == Z2D_GRADIENT_RADIAL) {
        const double ir = std::fmax(0.0, src.geom[2]), orr = std::fmax(0.0, src.geom[5]);
        gr.inner_r = ir;
        gr.outer_r = orr;
        gr.cdx = src.geom[3] - src.geom[0];
        gr.cdy = src.geom[4] - src.geom[1];
        gr.dr = orr - ir;
        gr.min_dr = -ir;
        double a = 0;
        a += gr.cdx * gr.cdx;
        a += gr.cdy * gr.cdy;
        a += gr.dr * -gr.dr;
        gr.a = a;
        gr.inv_a = (a != 0) ? 1 / a : 0;
    } else if (gr.type == Z2D_GRADIENT_CONIC) {
        gr.angle = zmod(src.geom[2], M_PI * 2);  // Conic.initBuffer :675
    }
    return gr;
}

double clampd(double v, double lo, double hi) { return std::fmax(lo, std::fmin(v, hi)); }

// Gradient.getOffset (src/gradient.zig:239-243, 349-372, 605-648, 731-741)
float grad_offset(const Grad &gr, int32_t x, int32_t y) {
    if (gr.type == Z2D_GRADIENT_RADIAL && gr.inner_r == 0 && gr.outer_r == 0) return -1;
    double px = (double)x + 0.5, py = (double)y + 0.5;
    if (gr.has_tf) {  // Transformation.userToDevice (src/Transformation.zig:194-206)
        const double ix = px, iy = py;
        px = gr.tf[0] * ix + gr.tf[1] * iy;
        py = gr.tf[2] * ix + gr.tf[3] * iy;
        px += gr.tf[4];
        py += gr.tf[5];
    }
    if (gr.type == Z2D_GRADIENT_LINEAR) {
        const double dx = gr.g[2] - gr.g[0], dy = gr.g[3] - gr.g[1];
        double dist = 0;
        dist += dx * dx;
        dist += dy * dy;
        if (dist == 0) return -1;
        const double inv_dist = 1 / dist;
        const double spx = px - gr.g[0], spy = py - gr.g[1];
        double d = 0;
        d += dx * spx;
        d += dy * spy;
        return (float)clampd(d * inv_dist, 0, 1);
    }
    if (gr.type == Z2D_GRADIENT_RADIAL) {
        const double pdx = px - gr.g[0], pdy = py - gr.g[1];
        double b = 0;
        b += pdx * gr.cdx;
        b += pdy * gr.cdy;
        b += gr.inner_r * gr.dr;
        double c = 0;
        c += pdx * pdx;
        c += pdy * pdy;
        c += -gr.inner_r * gr.inner_r;
        if (gr.a == 0) {
            if (b == 0) return -1;
            const double t = 0.5 * c / b;
            if (t * gr.dr >= gr.min_dr) return (float)clampd(t, 0, 1);
            return -1;
        }
        double discr = 0;
        discr += b * b;
        discr += gr.a * -c;
        if (discr >= 0) {
            const double sq = std::sqrt(discr);
            const double t0 = (b + sq) * gr.inv_a;
            const double t1 = (b - sq) * gr.inv_a;
            if (t0 * gr.dr >= gr.min_dr) return (float)clampd(t0, 0, 1);
            if (t1 * gr.dr >= gr.min_dr) return (float)clampd(t1, 0, 1);
        }
        return -1;
    }
    const double dx = px - gr.g[0], dy = py - gr.g[1];
    const double ang = zmod(zatan2(dy, dx) - gr.angle, M_PI * 2);
    return (float)(ang / (M_PI * 2));
}

struct Search {
    z2d_color c0, c1;
    float offset;
};
// Stop.List.search (src/gradient.zig:832-897)
Search grad_search(const Grad &gr, float offset) {
    const z2d_color zero{Z2D_COLOR_LINEAR_RGB, {0, 0, 0, 0}};
    const size_t n = gr.stops.size();
    if (offset < 0 || n == 0) return Search{zero, zero, 0};
    const float o = fmin2(offset, 1.0f);
    size_t left = 0, right = n, mid = 0;
    while (left < right) {
        mid = left + (right - left) / 2;
        if (o >= gr.stops[mid].offset && (mid == n - 1 || o <= gr.stops[mid + 1].offset)) break;
        if (o < gr.stops[mid].offset) {
            right = mid;
            continue;
        }
        if (o > gr.stops[mid].offset) {
            left = mid + 1;
            continue;
        }
    }
    if (mid == n - 1) return Search{gr.stops[mid].color, gr.stops[mid].color, o - gr.stops[mid].offset};
    if (mid == 0 && o < gr.stops[mid].offset) return Search{gr.stops[mid].color, gr.stops[mid].color, o / gr.stops[mid].offset};
    const float start = gr.stops[mid].offset, end = gr.stops[mid + 1].offset;
    const float rl = end - start;
    const float ro = (rl != 0) ? (o - start) / rl : 0;
    return Search{gr.stops[mid].color, gr.stops[mid + 1].color, ro};
}

extern const uint16_t kBlueNoise[4096];

// mBayer8x8Vec / mBlueNoise64x64Vec lane (color_vector.zig:482-522)
float bayer(int32_t x, int32_t y) {
    const int32_t yy = y ^ x;
    const uint32_t m = (uint32_t)(((yy & 1) << 5) | ((x & 1) << 4) | ((yy & 2) << 2) | ((x & 2) << 1) |
                                  ((yy & 4) >> 1) | ((x & 4) >> 2));
    return (float)m * (2.0f / 128.0f) - (63.0f / 128.0f);
}
int32_t imod(int32_t a, int32_t b) {
    const int32_t r = a % b;
    return r < 0 ? r + b : r;
}
float blue_noise(int32_t x, int32_t y) {
    const int32_t idx = (imod(x, 64) << 6) | imod(y, 64);
    return (float)kBlueNoise[idx] * (2.0f / 8192.0f) - (4095.0f / 8192.0f);
}

// ===================================================================
// Sources for the stride compositor
// ===================================================================
struct Src {
    int kind;  // Z2D_PARAM_*
    Px px;
    Grad grad;
    bool has_grad;
    int dither_type, dither_source, dither_scale;
    z2d_color dither_color;
    Sfc sfc;
};

Src make_src_from_pattern(int kind, const z2d_pattern &p) {
    Src s{};
    s.kind = kind;
    s.px = px_from_abi(p.pixel);
    s.has_grad = false;
    if ((kind == Z2D_PARAM_GRADIENT || (kind == Z2D_PARAM_DITHER && p.dither_source == Z2D_DITHER_SRC_GRADIENT)) &&
        p.gradient) {
        s.grad = make_grad(*p.gradient);
        s.has_grad = true;
    }
    s.dither_type = p.dither_type;
    s.dither_source = p.dither_source;
    s.dither_scale = p.dither_scale;
    s.dither_color = p.dither_color;
    return s;
}

// color_vector.fromDitherVec lane (color_vector.zig:108-186)
RGBf dither_linear(const Src &s, int32_t x, int32_t y) {
    RGBf c{0, 0, 0, 0};
    if (s.dither_source == Z2D_DITHER_SRC_PIXEL) {
        // LinearRGB.decodeRGBA: integer demultiply, /255, gamma 1 (src/color.zig:261-269)
        I16 v = to_i16(convert_px(s.px, Z2D_FORMAT_RGBA));
        if (v.a == 0) v = I16{0, 0, 0, 0};
        else v = I16{(uint16_t)(v.r * 255 / v.a), (uint16_t)(v.g * 255 / v.a), (uint16_t)(v.b * 255 / v.a), v.a};
        c = RGBf{(float)(uint8_t)v.r / 255.0f, (float)(uint8_t)v.g / 255.0f, (float)(uint8_t)v.b / 255.0f,
                 (float)(uint8_t)v.a / 255.0f};
    } else if (s.dither_source == Z2D_DITHER_SRC_COLOR) {
        c = linear_from_color(s.dither_color);
    } else {
        const Search r = grad_search(s.grad, grad_offset(s.grad, x, y));
        c = interp_linear(s.grad.method, r.c0, r.c1, r.offset);
    }
    float m;
    switch (s.dither_type) {
        case Z2D_DITHER_BAYER: m = bayer(x, y); break;
        case Z2D_DITHER_BLUE_NOISE: m = blue_noise(x, y); break;
        default: return c;
    }
    const float scale = 1.0f / (float)((1 << s.dither_scale) - 1);
    auto ap = [&](float v) { return fmax2(0.0f, fmin2(v + m * scale, 1.0f)); };
    return RGBf{ap(c.r), ap(c.g), ap(c.b), ap(c.a)};
}

// Source lane at absolute position (x, y) in integer precision
// (RGBA16Vec.fromPixel/fromGradient/fromDither, src/compositor.zig:708-804).
I16 src_i16(const Src &s, int32_t x, int32_t y) {
    switch (s.kind) {
        case Z2D_PARAM_PIXEL: return i16_from_pixel(s.px);
        case Z2D_PARAM_GRADIENT: {
            const Search r = grad_search(s.grad, grad_offset(s.grad, x, y));
            return interp_encode(s.grad.method, r.c0, r.c1, r.offset);
        }
        case Z2D_PARAM_DITHER: return encode_linear(dither_linear(s, x, y));
        default: return I16{0, 0, 0, 0};
    }
}
// Float precision (RGBAFloat.Vector.fromPixel/fromGradient/fromDither,
// src/compositor.zig:1061-1131).  Gradient and dither lanes come out
// demultiplied (interpolateVec / fromDitherVec), pixels raw.
F4 src_f4(const Src &s, int32_t x, int32_t y) {
    switch (s.kind) {
        case Z2D_PARAM_PIXEL: return decode_raw(i16_from_pixel(s.px));
        case Z2D_PARAM_GRADIENT: {
            const Search r = grad_search(s.grad, grad_offset(s.grad, x, y));
            const RGBf c = interp_linear(s.grad.method, r.c0, r.c1, r.offset);
            return F4{c.r, c.g, c.b, c.a};
        }
        case Z2D_PARAM_DITHER: {
            const RGBf c = dither_linear(s, x, y);
            return F4{c.r, c.g, c.b, c.a};
        }
        default: return F4{0, 0, 0, 0};
    }
}

// ===================================================================
// Stride compositor                       src/compositor.zig:443-621
// ===================================================================
// One operation of a stride batch.  `stride_*` index a surface row.
struct SOp {
    int op;
    int dst_kind;  // Z2D_PARAM_NONE => the destination stride
    const Src *dst;
    size_t dst_off;  // flat index of the first pixel for SURFACE params
    int src_kind;
    const Src *src;
    size_t src_off;
};

// Runs ops over `len` pixels of `dst` starting at flat index `dst_start`;
// (x0, y) are the device coordinates of the first pixel (gradient/dither).
// Every lane of z2d's 16-wide vectors is independent, so the chunk/tail
// split of runPrecision (:562-620) does not change any pixel and is folded
// into one loop here.
void stride_run(Sfc &dst, size_t dst_start, size_t len, int32_t x0, int32_t y, const SOp *ops, int n_ops,
                int precision) {
    for (size_t i = 0; i < len; i++) {
        const int32_t x = x0 + (int32_t)i;
        if (precision == Z2D_PRECISION_INTEGER) {
            I16 d{}, s{};
            for (int k = 0; k < n_ops; k++) {
                const SOp &o = ops[k];
                if (o.src_kind == Z2D_PARAM_NONE) s = d;
                else if (o.src_kind == Z2D_PARAM_SURFACE) s = load_i16(o.src->sfc, o.src_off + i);
                else s = src_i16(*o.src, x, y);
                if (o.dst_kind == Z2D_PARAM_NONE) d = load_i16(dst, dst_start + i);
                else if (o.dst_kind == Z2D_PARAM_SURFACE) d = load_i16(o.dst->sfc, o.dst_off + i);
                else d = src_i16(*o.dst, x, y);
                d = int_op(o.op, d, s);
            }
            store_i16(dst, dst_start + i, d);
        } else {
            F4 d{}, s{};
            for (int k = 0; k < n_ops; k++) {
                const SOp &o = ops[k];
                if (o.src_kind == Z2D_PARAM_NONE) s = d;
                else if (o.src_kind == Z2D_PARAM_SURFACE) s = decode_raw(load_i16(o.src->sfc, o.src_off + i));
                else s = src_f4(*o.src, x, y);
                if (o.dst_kind == Z2D_PARAM_NONE) d = decode_raw(load_i16(dst, dst_start + i));
                else if (o.dst_kind == Z2D_PARAM_SURFACE) d = decode_raw(load_i16(o.dst->sfc, o.dst_off + i));
                else d = src_f4(*o.dst, x, y);
                d = float_op(o.op, d, s);
            }
            store_i16(dst, dst_start + i, encode_raw(d));
        }
    }
}

// ===================================================================
// Surface helpers                                    src/surface.zig
// ===================================================================
bool in_surface(const Sfc &s, int32_t x, int32_t y) { return !(x < 0 || y < 0 || x >= s.w || y >= s.h); }

// paintStride (src/surface.zig:537-544, 787-839)
void paint_stride(Sfc &s, int32_t x, int32_t y, size_t len, const Px &px) {
    if (!in_surface(s, x, y)) return;
    const Px v = convert_px(px, s.fmt);
    const size_t start = (size_t)s.w * (size_t)y + (size_t)x;
    for (size_t i = 0; i < len; i++) raw_set(s, start + i, v);
}
void clear_stride(Sfc &s, int32_t x, int32_t y, size_t len) {  // :323-325
    paint_stride(s, x, y, len, Px{Z2D_FORMAT_RGBA, 0, 0, 0, 0});
}
// compositeStride (src/surface.zig:557-581, 852-876)
void composite_stride(Sfc &s, int32_t x, int32_t y, size_t len, const Px &px, int op, uint8_t opacity) {
    if (!in_surface(s, x, y)) return;
    const size_t start = (size_t)s.w * (size_t)y + (size_t)x;
    I16 src = to_i16(convert_px(px, Z2D_FORMAT_RGBA));
    if (opacity < 255) src = int_op(Z2D_OP_DST_IN, src, I16{0, 0, 0, opacity});
    // runPixelT(RGBA, src, ...) stores src back as an RGBA pixel first
    src = to_i16(from_i16(src, Z2D_FORMAT_RGBA));
    for (size_t i = start; i < start + len; i++) store_i16(s, i, int_op(op, load_i16(s, i), src));
}

// ===================================================================
// Span compositing                     src/internal/raster/shared.zig
// ===================================================================
struct FillSrc {
    int kind;  // Z2D_PATTERN_*
    Src src;   // as a stride-compositor parameter
};

bool reduces_to_source(int op, const Px &px) {  // shared.zig:111-117
    if (op == Z2D_OP_SRC) return true;
    if (op == Z2D_OP_SRC_OVER) {
        switch (px.fmt) {  // Pixel.isOpaque (src/pixel.zig:133-141)
            case Z2D_FORMAT_XRGB: case Z2D_FORMAT_RGB: return true;
            default: return px.a == fmt_max(px.fmt);
        }
    }
    return false;
}

void composite_opaque(int op, Sfc &s, const FillSrc &pat, int32_t x, int32_t y, size_t len, int precision) {
    if (op == Z2D_OP_CLEAR) {  // shared.zig:9-46
        clear_stride(s, x, y, len);
    } else if (pat.kind == Z2D_PATTERN_PIXEL && reduces_to_source(op, pat.src.px)) {
        paint_stride(s, x, y, len, pat.src.px);
    } else {
        if (!in_surface(s, x, y) || len == 0) return;
        SOp o{op, Z2D_PARAM_NONE, nullptr, 0, pat.src.kind, &pat.src, 0};
        stride_run(s, (size_t)s.w * y + x, len, x, y, &o, 1, precision);
    }
}

void composite_opacity(int op, Sfc &s, const FillSrc &pat, int32_t x, int32_t y, size_t len, int precision,
                       uint8_t opacity) {
    if (op == Z2D_OP_CLEAR) {  // shared.zig:50-104
        clear_stride(s, x, y, len);
    } else if (pat.kind == Z2D_PATTERN_PIXEL && reduces_to_source(op, pat.src.px)) {
        composite_stride(s, x, y, len, pat.src.px, op, opacity);
    } else {
        if (!in_surface(s, x, y) || len == 0) return;
        Src mask{};
        mask.kind = Z2D_PARAM_PIXEL;
        mask.px = Px{Z2D_FORMAT_ALPHA8, 0, 0, 0, opacity};
        SOp o[2] = {{Z2D_OP_DST_IN, pat.src.kind, &pat.src, 0, Z2D_PARAM_PIXEL, &mask, 0},
                    {op, Z2D_PARAM_NONE, nullptr, 0, Z2D_PARAM_NONE, nullptr, 0}};
        stride_run(s, (size_t)s.w * y + x, len, x, y, o, 2, precision);
    }
}

// ===================================================================
// Tessellation                      src/internal/tess/*.zig
// ===================================================================
struct Pt {
    double x, y;
    bool operator==(const Pt &o) const { return x == o.x && y == o.y; }
    bool operator!=(const Pt &o) const { return !(*this == o); }
};
struct Edge {  // Polygon.Edge (Polygon.zig:18-47)
    double y0, y1, x_start, x_inc;
    int dir() const { return y0 < y1 ? -1 : 1; }
    double top() const { return y0 < y1 ? y0 : y1; }
    double bottom() const { return y0 < y1 ? y1 : y0; }
};
struct Poly {
    std::vector<Edge> edges;
    double scale = 1;
    double et = 0, eb = 0, el = 0, er = 0;

    void add_edge(Pt p0, Pt p1) {  // Polygon.addEdge (Polygon.zig:61-109)
        const Pt a{p0.x * scale, p0.y * scale}, b{p1.x * scale, p1.y * scale};
        Edge e;
        if (a.y < b.y) e = Edge{a.y, b.y, a.x, (b.x - a.x) / (b.y - a.y)};
        else if (a.y > b.y) e = Edge{a.y, b.y, b.x, (a.x - b.x) / (a.y - b.y)};
        else return;
        const double t = e.top(), bt = e.bottom();
        const double l = a.x < b.x ? a.x : b.x, r = a.x < b.x ? b.x : a.x;
        if (edges.empty()) {
            et = t; eb = bt; el = l; er = r;
        } else {
            if (t < et) et = t;
            if (bt > eb) eb = bt;
            if (l < el) el = l;
            if (r > er) er = r;
        }
        edges.push_back(e);
    }

    bool in_box(double sc, int32_t bw, int32_t bh) const {  // Polygon.inBox (Polygon.zig:142-201)
        if (er < 0.0 || eb < 0.0) return false;
        const int32_t sx = (int32_t)std::floor(el / sc), sy = (int32_t)std::floor(et / sc);
        const int32_t ex = (int32_t)std::ceil(er / sc), ey = (int32_t)std::ceil(eb / sc);
        const int32_t pw = ex - sx, ph = ey - sy;
        if (pw == 0 || ph == 0) return false;
        if (sx + pw < 0 || sy + ph < 0) return false;
        if (sx >= bw || sy >= bh) return false;
        return true;
    }
};

// PointBuffer(1, 3) (src/internal/tess/point_buffer.zig:14-60)
struct PointBuf {
    Pt items[3];
    size_t len = 0;
    void add(Pt p) {
        if (len < 3) items[len++] = p;
        else {
            items[1] = items[2];
            items[2] = p;
        }
    }
    Pt last() const { return items[len - 1]; }
    Pt first() const { return items[0]; }
};

struct Knots {
    Pt a, b, c, d;
};
// Spline.Knots.errorSq (Spline.zig:83-123)
double error_sq(const Knots &k) {
    double bx = k.b.x - k.a.x, by = k.b.y - k.a.y;
    double cx = k.c.x - k.a.x, cy = k.c.y - k.a.y;
    if (k.a.x != k.d.x || k.a.y != k.d.y) {
        const double dx = k.d.x - k.a.x, dy = k.d.y - k.a.y;
        const double dd = dx * dx + dy * dy;
        const double bd = bx * dx + by * dy;
        if (bd >= dd) {
            bx -= dx;
            by -= dy;
        } else {
            bx -= bd / dd * dx;
            by -= bd / dd * dy;
        }
        const double cd = cx * dx + cy * dy;
        if (cd >= dd) {
            cx -= dx;
            cy -= dy;
        } else {
            cx -= cd / dd * dx;
            cy -= cd / dd * dy;
        }
    }
    const double be = bx * bx + by * by, ce = cx * cx + cy * cy;
    return be > ce ? be : ce;
}
Pt lerp_half(Pt a, Pt b) { return Pt{a.x + ((b.x - a.x) / 2), a.y + ((b.y - a.y) / 2)}; }  // :158-165
// Knots.deCasteljau (:128-152): k becomes the first half, returns the second
Knots de_casteljau(Knots &k) {
    const Pt ab = lerp_half(k.a, k.b), bc = lerp_half(k.b, k.c), cd = lerp_half(k.c, k.d);
    const Pt abbc = lerp_half(ab, bc), bccd = lerp_half(bc, cd), fin = lerp_half(abbc, bccd);
    const Knots r{fin, bccd, cd, k.d};
    k.b = ab;
    k.c = abbc;
    k.d = fin;
    return r;
}

struct Plotter {
    Poly *poly;
    PointBuf *pts;
    void line_to(Pt p) {  // SplinePlotterCtx.line_to (fill_plotter.zig:104-118)
        const Pt last = pts->last();
        if (last != p) {
            poly->add_edge(last, p);
            pts->add(p);
        }
    }
};

void decompose_into(Plotter &pl, Knots &s1, Pt start, double tol) {  // Spline.zig:56-71
    if (error_sq(s1) < tol) {
        if (s1.a != start) pl.line_to(s1.a);
        return;
    }
    Knots s2 = de_casteljau(s1);
    decompose_into(pl, s1, start, tol);
    decompose_into(pl, s2, start, tol);
}
void decompose(Plotter &pl, Pt a, Pt b, Pt c, Pt d, double tol) {  // Spline.zig:37-53
    if (a == b && c == d) {
        pl.line_to(d);
        return;
    }
    Knots s1{a, b, c, d};
    decompose_into(pl, s1, a, tol * tol);
    pl.line_to(d);
}

// fill_plotter.plot (fill_plotter.zig:21-97)
int plot(const z2d_node *nodes, size_t n, double scale, double tol, Poly &poly) {
    poly.scale = scale;
    PointBuf pts;
    Plotter pl{&poly, &pts};
    for (size_t i = 0; i < n; i++) {
        const z2d_node &nd = nodes[i];
        switch (nd.tag) {
            case Z2D_MOVE_TO:
                if (i == n - 1) return Z2D_OK;
                pts.len = 0;
                pts.add(Pt{nd.p[0], nd.p[1]});
                break;
            case Z2D_LINE_TO: {
                if (pts.len == 0) return Z2D_ERR_INVALID_STATE;
                const Pt p{nd.p[0], nd.p[1]};
                if (pts.last() != p) {
                    poly.add_edge(pts.last(), p);
                    pts.add(p);
                }
                break;
            }
            case Z2D_CURVE_TO:
                if (pts.len == 0) return Z2D_ERR_INVALID_STATE;
                decompose(pl, pts.last(), Pt{nd.p[0], nd.p[1]}, Pt{nd.p[2], nd.p[3]}, Pt{nd.p[4], nd.p[5]}, tol);
                break;
            case Z2D_CLOSE_PATH:
                if (pts.len >= 3) {
                    if (pts.last() == pts.first()) continue;
                    poly.add_edge(pts.last(), pts.first());
                    pts.add(pts.first());
                }
                break;
            default: return Z2D_ERR_INVALID_ARGUMENT;
        }
    }
    return Z2D_OK;
}

// PathNode.isClosedNodeSet (path_nodes.zig:23-36)
bool is_closed(const z2d_node *nodes, size_t n) {
    if (n == 0) return false;
    bool closed = false;
    for (size_t i = 0; i < n; i++) {
        switch (nodes[i].tag) {
            case Z2D_MOVE_TO:
                if (!closed && i != 0) return closed;
                break;
            case Z2D_CLOSE_PATH: closed = true; break;
            default: closed = false; break;
        }
    }
    return closed;
}

// ===================================================================
// Working edge set                      Polygon.zig:203-354
// ===================================================================
struct WES {
    Poly *poly;
    size_t n_active = 0;
    std::vector<int32_t> xv;

    explicit WES(Poly *p) : poly(p), xv(p->edges.size()) {}

    std::vector<int32_t> breakpoints() const {  // :232-273
        std::vector<int32_t> r;
        auto ins = [&](int32_t v) {
            auto it = std::lower_bound(r.begin(), r.end(), v);
            if (it == r.end() || *it != v) r.insert(it, v);
        };
        for (const Edge &e : poly->edges) {
            ins((int32_t)std::round(e.top()));
            ins((int32_t)std::round(e.bottom()));
        }
        return r;
    }
    void rescan(int32_t line_y) {  // :275-300
        if (poly->edges.empty()) return;
        const double mid = (double)line_y + 0.5;
        size_t to = 0;
        auto &E = poly->edges;
        for (size_t from = 0; from < E.size(); from++) {
            if (E[from].top() < mid && E[from].bottom() >= mid) {
                if (from != to) std::swap(E[to], E[from]);
                to++;
            }
        }
        n_active = to;
    }
    void inc(int32_t y) {  // :302-307
        const double ym = (double)y + 0.5;
        for (size_t i = 0; i < n_active; i++) {
            const Edge &e = poly->edges[i];
            xv[i] = (int32_t)std::round(e.x_start + (e.x_inc * (ym - e.top())));
        }
    }
    void sort() {  // :309-324 (std.sort.pdqContext; see the note at the top)
        auto &E = poly->edges;
        const size_t n = n_active;
        if (n <= 24) {  // std.sort.insertionContext
            for (size_t i = 1; i < n; i++)
                for (size_t j = i; j > 0 && xv[j] < xv[j - 1]; j--) {
                    std::swap(E[j], E[j - 1]);
                    std::swap(xv[j], xv[j - 1]);
                }
            return;
        }
        std::vector<size_t> order(n);
        for (size_t i = 0; i < n; i++) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return xv[a] < xv[b]; });
        std::vector<Edge> e2(n);
        std::vector<int32_t> x2(n);
        for (size_t i = 0; i < n; i++) {
            e2[i] = E[order[i]];
            x2[i] = xv[order[i]];
        }
        for (size_t i = 0; i < n; i++) {
            E[i] = e2[i];
            xv[i] = x2[i];
        }
    }
    size_t filter(int rule) {  // :326-353; returns the filtered length (values in xv)
        if (rule == Z2D_FILL_EVEN_ODD) return n_active;
        int32_t wn = 0;
        size_t to = 0;
        for (size_t from = 0; from < n_active; from++) {
            xv[to] = xv[from];
            if (wn == 0) {
                wn += poly->edges[from].dir();
                to++;
            } else {
                wn += poly->edges[from].dir();
                if (wn == 0) to++;
            }
        }
        return to;
    }
};

size_t seek_breakpoint(const std::vector<int32_t> &bps, int32_t start, bool &found) {
    for (size_t i = 0; i < bps.size(); i++)
        if (bps[i] >= start) {
            found = true;
            return i == 0 ? 0 : i - 1;
        }
    found = false;
    return 0;
}

// ===================================================================
// Sparse coverage buffer        src/internal/raster/sparse_coverage.zig
// ===================================================================
struct SparseCov {
    std::vector<uint8_t> values;
    std::vector<uint32_t> lengths;
    uint32_t len = 0, capacity;

    explicit SparseCov(uint32_t cap) : values(cap), lengths(cap), capacity(cap) { lengths[0] = 0; }
    void reset() {
        len = 0;
        lengths[0] = 0;
    }
    void put(uint32_t x, uint8_t v, uint32_t l) {
        values[x] = v;
        lengths[x] = l;
    }
    void split_inner(uint32_t x, uint32_t l) {  // :168-184
        uint32_t idx = x, rem = l;
        while (true) {
            const uint8_t cv = values[idx];
            const uint32_t cl = lengths[idx];
            if (rem < cl) {
                put(idx, cv, rem);
                put(idx + rem, cv, cl - rem);
                break;
            } else if (rem == cl) {
                break;
            }
            rem -= cl;
            idx += cl;
        }
    }
    void extend(uint32_t x, uint32_t l) {  // :125-166
        if (l == 0) return;
        if (x == len) {
            put(x, 0, l);
            len = x + l;
            return;
        }
        if (x > len) {
            put(len, 0, x - len);
            put(x, 0, l);
            len = x + l;
            return;
        }
        split_inner(0, x);
        const uint32_t span_len = x + l;
        if (span_len > len) {
            put(len, 0, span_len - len);
            len = span_len;
        }
        split_inner(x, l);
    }
    void add_span(uint32_t x, uint8_t v, uint32_t l) {  // :92-102
        extend(x, l);
        uint32_t cur = x;
        const uint32_t end = x + l;
        while (cur < end) {
            values[cur] = (uint8_t)(values[cur] + v);
            cur += lengths[cur];
        }
    }
    void add_single(uint32_t x, uint8_t v) {  // :104-109
        extend(x, 1);
        values[x] = (uint8_t)(values[x] + v);
    }
};

// multisample.addSpan (multisample.zig:239-279)
void msaa_add_span(SparseCov &cb, uint32_t x, uint32_t len) {
    const uint32_t sc = 4;
    if (len == 0) return;
    const uint32_t sx = x / sc, so = x - sx * sc;
    if (so == 0 && len >= sc) {
        const uint32_t front = len / sc;
        cb.add_span(sx, sc, front);
        const uint32_t endc = std::min(sc, len - front * sc);
        if (endc > 0) cb.add_single(sx + front, (uint8_t)endc);
    } else {
        const uint32_t startc = std::min(sc, std::min(len, sc - so));
        cb.add_single(sx, (uint8_t)startc);
        const uint32_t after = len - startc;
        const uint32_t mid = after / sc;
        if (mid > 0) cb.add_span(sx + 1, sc, mid);
        const uint32_t endc = std::min(sc, after - mid * sc);
        if (endc > 0) cb.add_single(sx + 1 + mid, (uint8_t)endc);
    }
}

int32_t clampi(int32_t v, int32_t lo, int32_t hi) { return std::max(lo, std::min(v, hi)); }

// ===================================================================
// Rasterisers                          src/internal/raster/*.zig
// ===================================================================
// multisample.run (multisample.zig:22-229)
void run_msaa(Sfc &s, const FillSrc &pat, Poly &poly, int rule, int op, int precision) {
    const int32_t scale = 4, cov_full = 16, alpha_scale = 256 / 16;
    const int32_t sw = s.w, sh = s.h;
    const int prec = requires_float(op) ? Z2D_PRECISION_FLOAT : precision;
    if (!poly.in_box(scale, sw, sh)) return;
    const int32_t start_y = clampi((int32_t)std::floor(poly.et / scale), 0, sh - 1);
    const int32_t end_y = clampi((int32_t)std::ceil(poly.eb / scale), start_y, sh - 1);
    const int32_t start_x = clampi((int32_t)std::floor(poly.el / scale), 0, sw - 1);
    const int32_t end_x = clampi((int32_t)std::ceil(poly.er / scale), start_x, sw);
    const int32_t draw_w = end_x - start_x;
    SparseCov cb((uint32_t)std::max(0, draw_w));
    const int32_t sx_scaled = start_x * scale, dw_scaled = draw_w * scale;
    if (!is_bounded(op)) {  // :96-110, including the sfc_width loop bound and x=0 right clear
        for (int32_t y = 0; y < start_y; y++) clear_stride(s, 0, y, (size_t)sw);
        for (int32_t y = end_y + 1; y < sw; y++) clear_stride(s, 0, y, (size_t)sw);
        for (int32_t y = start_y; y <= end_y; y++) {
            if (start_x > 0) clear_stride(s, 0, y, (size_t)start_x);
            if (end_x < sw) clear_stride(s, 0, y, (size_t)(sw - end_x));
        }
    }
    WES wes(&poly);
    const std::vector<int32_t> bps = wes.breakpoints();
    bool found;
    size_t bpi = seek_breakpoint(bps, start_y, found);
    if (!found) return;
    for (int32_t y = start_y; y <= end_y; y++) {
        const int32_t ys = y * scale;
        for (int32_t off = 0; off < 4; off++) {
            const int32_t yss = ys + off;
            if (yss >= bps[bpi]) {
                wes.rescan(yss);
                if (bpi < bps.size() - 1) bpi++;
            }
            wes.inc(yss);
            wes.sort();
            const size_t fl = wes.filter(rule);
            int32_t x_min = 0;
            for (size_t p = 0; p < fl / 2; p++) {
                const int32_t sxp = std::max(x_min, wes.xv[2 * p] - sx_scaled);
                if (sxp >= dw_scaled) break;
                const int32_t exp_ = clampi(wes.xv[2 * p + 1] - sx_scaled, sxp, dw_scaled);
                const int32_t fill_len = exp_ - sxp;
                if (fill_len > 0) msaa_add_span(cb, (uint32_t)std::max(0, sxp), (uint32_t)std::max(0, fill_len));
                x_min = exp_;
            }
        }
        const uint32_t cmax = std::min(cb.len, cb.capacity);
        uint32_t cx = 0;
        while (cx < cmax) {
            const int32_t x = (int32_t)cx + start_x;
            const uint8_t raw_v = cb.values[cx];
            const uint32_t raw_l = cb.lengths[cx];
            const uint8_t cv = (uint8_t)std::min<int32_t>(raw_v, cov_full);
            const uint32_t cl = std::min<uint32_t>(raw_l, (uint32_t)std::max(0, sw - x));
            if (cv == cov_full) {
                composite_opaque(op, s, pat, x, y, cl, prec);
            } else if (cv != 0) {
                composite_opacity(op, s, pat, x, y, cl, prec, (uint8_t)clampi(cv * alpha_scale - 1, 0, 255));
            }
            cx += cl;
            if (cl == 0) break;  // guard: z2d would loop forever on a zero-length run
        }
        cb.reset();
    }
}

// direct.run (direct.zig:14-127)
void run_direct(Sfc &s, const FillSrc &pat, Poly &poly, int rule, int op, int precision) {
    const int32_t sw = s.w, sh = s.h;
    const int prec = requires_float(op) ? Z2D_PRECISION_FLOAT : precision;
    const bool bounded = is_bounded(op);
    if (!poly.in_box(1.0, sw, sh)) return;
    const int32_t psy = bounded ? (int32_t)std::floor(poly.et) : 0;
    const int32_t pey = bounded ? (int32_t)std::ceil(poly.eb) : sh - 1;
    const int32_t start_y = clampi(psy, 0, sh - 1);
    const int32_t end_y = clampi(pey, start_y, sh - 1);
    WES wes(&poly);
    const std::vector<int32_t> bps = wes.breakpoints();
    bool found;
    size_t bpi = seek_breakpoint(bps, start_y, found);
    if (!found) return;
    for (int32_t y = start_y; y <= end_y; y++) {
        if (y >= bps[bpi]) {
            wes.rescan(y);
            if (bpi < bps.size() - 1) bpi++;
        }
        wes.inc(y);
        wes.sort();
        const size_t fl = wes.filter(rule);
        if (!bounded && fl == 0) {
            clear_stride(s, 0, y, (size_t)sw);
            continue;
        }
        for (size_t p = 0; p < fl / 2; p++) {
            const int32_t sx = std::max(0, wes.xv[2 * p]);
            if (sx >= sw) break;
            const int32_t ex = clampi(wes.xv[2 * p + 1], sx, sw);
            const int32_t fill_len = ex - sx, end_clear = sw - ex;
            if (!bounded && sx > 0) clear_stride(s, 0, y, (size_t)sx);
            if (fill_len > 0) composite_opaque(op, s, pat, sx, y, (size_t)fill_len, prec);
            if (!bounded && end_clear > 0) clear_stride(s, ex, y, (size_t)end_clear);
        }
    }
}

void surface_composite(Sfc &dst, int32_t dst_x, int32_t dst_y, int n, const SOp *ops_in, int precision,
                       int src0_kind, const Sfc *src0_sfc);

// supersample.run (supersample.zig:17-185) and the downsample it uses
// (src/surface.zig:447-469, 687-709; pixel.zig:435-464, 633-646)
void run_ssaa(Sfc &s, const FillSrc &pat, Poly &poly, int rule, int op, int precision) {
    const double scale = 4;
    const int32_t is = 4;
    if (!poly.in_box(scale, s.w, s.h)) return;
    const bool bounded = is_bounded(op);
    const int32_t x0 = bounded ? (int32_t)std::floor(poly.el / scale) : 0;
    const int32_t y0 = bounded ? (int32_t)std::floor(poly.et / scale) : 0;
    const int32_t x1 = bounded ? (int32_t)std::ceil(poly.er / scale) : s.w;
    const int32_t y1 = bounded ? (int32_t)std::ceil(poly.eb / scale) : s.h;
    const int32_t tw = s.w * is, th = s.h * is;
    const int32_t bx0 = clampi(x0 * is, 0, tw - 1), by0 = clampi(y0 * is, 0, th - 1);
    const int32_t bx1 = clampi(x1 * is, bx0, tw - 1), by1 = clampi(y1 * is, by0, th - 1);
    const int32_t mw = (bx1 + 1) - bx0, mh = (by1 + 1) - by0;
    const int mfmt = (s.fmt >= Z2D_FORMAT_ALPHA4) ? s.fmt : Z2D_FORMAT_ALPHA8;
    const int bits = fmt_bits(mfmt);
    std::vector<uint8_t> mbuf(((size_t)mw * mh * bits + 7) / 8, 0);
    Sfc m{mfmt, mw, mh, mbuf.data()};
    const Px opq{mfmt, 0, 0, 0, fmt_max(mfmt)};
    {
        WES wes(&poly);
        const std::vector<int32_t> bps = wes.breakpoints();
        bool found;
        size_t bpi = seek_breakpoint(bps, by0, found);
        if (!found) return;
        for (int32_t y = 0; y < mh; y++) {
            const int32_t dy = y + by0;
            if (dy >= bps[bpi]) {
                wes.rescan(dy);
                if (bpi < bps.size() - 1) bpi++;
            }
            wes.inc(dy);
            wes.sort();
            const size_t fl = wes.filter(rule);
            for (size_t p = 0; p < fl / 2; p++) {
                const int32_t sx = std::max(0, wes.xv[2 * p] - bx0);
                if (sx >= mw) break;
                const int32_t ex = clampi(wes.xv[2 * p + 1] - bx0, sx, mw);
                if (ex - sx > 0) paint_stride(m, sx, y, (size_t)(ex - sx), opq);
            }
        }
    }
    // downsampleBuffer: skipped entirely when the mask is smaller than 4x4
    if (!(m.w < is || m.h < is)) {
        const int32_t h = m.h / is, w = m.w / is;
        for (int32_t y = 0; y < h; y++)
            for (int32_t x = 0; x < w; x++) {
                uint32_t sum = 0;
                for (int32_t i = 0; i < is; i++)
                    for (int32_t j = 0; j < is; j++) sum += raw_get(m, (size_t)(y * is + i) * m.w + (x * is + j)).a;
                raw_set(m, (size_t)y * w + x, Px{mfmt, 0, 0, 0, (uint8_t)(sum / 16)});
            }
        m.w = w;
        m.h = h;
    }
    Src mask_src{};
    mask_src.kind = Z2D_PARAM_SURFACE;
    mask_src.sfc = m;
    SOp ops[2] = {{Z2D_OP_DST_IN, pat.src.kind, &pat.src, 0, Z2D_PARAM_SURFACE, &mask_src, 0},
                  {op, Z2D_PARAM_NONE, nullptr, 0, Z2D_PARAM_NONE, nullptr, 0}};
    surface_composite(s, std::max(0, x0), std::max(0, y0), 2, ops, precision, Z2D_PARAM_SURFACE, &m);
}

// SurfaceCompositor.run (src/compositor.zig:302-440).  ops[k].src_off /
// dst_off are recomputed per row for SURFACE params.
void surface_composite(Sfc &dst, int32_t dst_x, int32_t dst_y, int n, const SOp *ops_in, int precision,
                       int src0_kind, const Sfc *src0_sfc) {
    if (n == 0) return;
    if (dst_x >= dst.w || dst_y >= dst.h) return;
    int prec = precision;
    for (int k = 0; k < n; k++)
        if (requires_float(ops_in[k].op)) prec = Z2D_PRECISION_FLOAT;
    int32_t sw, sh;
    if (src0_kind == Z2D_PARAM_NONE) return;
    if (src0_kind == Z2D_PARAM_SURFACE) {
        sw = src0_sfc->w;
        sh = src0_sfc->h;
    } else {
        if (dst_x != 0 || dst_y != 0) return;
        sw = dst.w;
        sh = dst.h;
    }
    const int32_t ssx = dst_x < 0 ? -dst_x : 0, ssy = dst_y < 0 ? -dst_y : 0;
    const int32_t width = (sw + dst_x > dst.w) ? dst.w - dst_x : sw;
    const int32_t height = (sh + dst_y > dst.h) ? dst.h - dst_y : sh;
    if (ssx >= width || ssy >= height) return;
    const int32_t scan_hi = std::max(ssy, height);
    const int32_t dsx = ssx + dst_x;
    const size_t line_w = (size_t)std::max(0, width - ssx);
    std::vector<SOp> ops(ops_in, ops_in + n);
    for (int32_t sy = ssy; sy < scan_hi; sy++) {
        const int32_t dy = sy + dst_y;
        if (!in_surface(dst, dsx, dy)) continue;  // getStride gives an empty stride
        bool skip = false;
        for (int k = 0; k < n; k++) {
            if (ops[k].dst_kind == Z2D_PARAM_SURFACE) {
                const Sfc &o = ops[k].dst->sfc;
                if (!in_surface(o, dsx, dy)) skip = true;  // stride shorter than dst: UB in z2d
                ops[k].dst_off = (size_t)o.w * dy + dsx;
            }
            if (ops[k].src_kind == Z2D_PARAM_SURFACE) {
                const Sfc &o = ops[k].src->sfc;
                if (!in_surface(o, ssx, sy)) skip = true;
                ops[k].src_off = (size_t)o.w * sy + ssx;
            }
        }
        if (skip) continue;
        stride_run(dst, (size_t)dst.w * dy + dsx, line_w, dsx, dy, ops.data(), n, prec);
    }
}

Sfc sfc_from_abi(const z2d_surface *s) { return Sfc{s->format, s->width, s->height, (uint8_t *)s->data}; }

bool pixel_premultiplied(const z2d_pixel &p) {  // canDemultiply (src/pixel.zig:504-514)
    if (p.format != Z2D_FORMAT_ARGB && p.format != Z2D_FORMAT_RGBA) return true;
    if (p.a == 0) return true;
    const int ch[3] = {p.r, p.g, p.b};
    for (int c : ch)
        if (c * 255 / p.a > 255) return false;
    return true;
}

}  // namespace

// blue-noise thresholds, shared with the GPU build as a data table
namespace {
const uint16_t kBlueNoise[4096] = {
#include "../z2d_gb300/csrc/blue_noise_64x64.inc"
};
}  // namespace

// ===================================================================
// Exported oracle entry points
// ===================================================================

extern "C" {

__attribute__((visibility("default"))) size_t z2doracle_surface_bytes(int32_t format, int32_t w, int32_t h) {
    return ((size_t)w * (size_t)h * (size_t)fmt_bits(format) + 7) / 8;
}

// painter.fill (src/painter.zig:66-143) on a host surface.
__attribute__((visibility("default"))) int z2doracle_fill(z2d_surface *surface, const z2d_pattern *pattern,
                                                          const z2d_node *nodes, size_t n_nodes,
                                                          const z2d_fill_opts *opts) {
    if (!surface || !pattern || !opts || (n_nodes && !nodes)) return Z2D_ERR_INVALID_ARGUMENT;
    if (surface->width < 1 || surface->height < 1) return Z2D_ERR_INVALID_DIMENSIONS;
    if (pattern->kind == Z2D_PATTERN_PIXEL && !pixel_premultiplied(pattern->pixel))
        return Z2D_ERR_PIXEL_NOT_PREMULTIPLIED;
    if (n_nodes == 0) return Z2D_OK;
    if (!is_closed(nodes, n_nodes)) return Z2D_ERR_PATH_NOT_CLOSED;
    Sfc s = sfc_from_abi(surface);
    const int aa = (s.fmt == Z2D_FORMAT_ALPHA1) ? Z2D_AA_NONE : opts->anti_aliasing;
    const double scale = (aa == Z2D_AA_NONE) ? 1.0 : 4.0;
    Poly poly;
    const int rc = plot(nodes, n_nodes, scale, std::fmax(opts->tolerance, 0.001), poly);
    if (rc != Z2D_OK) return rc;
    FillSrc pat;
    pat.kind = pattern->kind;
    const int pk = pattern->kind == Z2D_PATTERN_PIXEL      ? Z2D_PARAM_PIXEL
                   : pattern->kind == Z2D_PATTERN_GRADIENT ? Z2D_PARAM_GRADIENT
                                                           : Z2D_PARAM_DITHER;
    pat.src = make_src_from_pattern(pk, *pattern);
    // Polygon.inBox panics on non-finite extents; report that as InvalidState.
    if (!poly.edges.empty() &&
        !(std::isfinite(poly.el) && std::isfinite(poly.et) && std::isfinite(poly.er) && std::isfinite(poly.eb)))
        return Z2D_ERR_INVALID_STATE;
    if (poly.edges.empty()) {
        // inBox on the zero extents of an empty polygon returns false
        return Z2D_OK;
    }
    switch (aa) {
        case Z2D_AA_NONE: run_direct(s, pat, poly, opts->fill_rule, opts->op, opts->precision); break;
        case Z2D_AA_SUPERSAMPLE_4X: run_ssaa(s, pat, poly, opts->fill_rule, opts->op, opts->precision); break;
        default: run_msaa(s, pat, poly, opts->fill_rule, opts->op, opts->precision); break;
    }
    return Z2D_OK;
}

// SurfaceCompositor.run (src/compositor.zig:302-440) on host surfaces.
__attribute__((visibility("default"))) int z2doracle_composite(z2d_surface *dst, int32_t dst_x, int32_t dst_y,
                                                               int32_t n_ops, const z2d_operation *ops,
                                                               int32_t precision) {
    if (!dst || (n_ops && !ops) || n_ops < 0 || n_ops > 8) return Z2D_ERR_INVALID_ARGUMENT;
    Sfc d = sfc_from_abi(dst);
    std::vector<Src> srcs(2 * (size_t)n_ops);
    std::vector<SOp> sops((size_t)n_ops);
    for (int k = 0; k < n_ops; k++) {
        const z2d_operation &o = ops[k];
        Src &ds = srcs[2 * k], &ss = srcs[2 * k + 1];
        auto fill = [](Src &dst_src, const z2d_param &p) {
            if (p.kind == Z2D_PARAM_SURFACE) {
                dst_src = Src{};
                dst_src.kind = Z2D_PARAM_SURFACE;
                dst_src.sfc = sfc_from_abi(p.surface);
            } else if (p.kind != Z2D_PARAM_NONE) {
                dst_src = make_src_from_pattern(p.kind, p.pattern);
            } else {
                dst_src = Src{};
                dst_src.kind = Z2D_PARAM_NONE;
            }
        };
        fill(ds, o.dst);
        fill(ss, o.src);
        sops[k] = SOp{o.op, o.dst.kind, &ds, 0, o.src.kind, &ss, 0};
    }
    if (n_ops == 0) return Z2D_OK;
    const Sfc *s0 = ops[0].src.kind == Z2D_PARAM_SURFACE ? &srcs[1].sfc : nullptr;
    surface_composite(d, dst_x, dst_y, n_ops, sops.data(), precision, ops[0].src.kind, s0);
    return Z2D_OK;
}

// compositor.runPixel (src/compositor.zig:626-643): one pixel through one
// operator, result in dst's format.
__attribute__((visibility("default"))) z2d_pixel z2doracle_run_pixel(int32_t precision, z2d_pixel dst, z2d_pixel src,
                                                                     int32_t op) {
    const Px d = px_from_abi(dst), s = px_from_abi(src);
    I16 r;
    if (precision == Z2D_PRECISION_INTEGER) {
        r = int_op(op, i16_from_pixel(d), i16_from_pixel(s));
    } else {
        r = encode_raw(float_op(op, decode_raw(i16_from_pixel(d)), decode_raw(i16_from_pixel(s))));
    }
    const Px o = convert_px(Px{Z2D_FORMAT_RGBA, (uint8_t)r.r, (uint8_t)r.g, (uint8_t)r.b, (uint8_t)r.a}, d.fmt);
    return z2d_pixel{o.fmt, o.r, o.g, o.b, o.a};
}

// Pixel.fromColor (src/pixel.zig:119-121): LinearRGB.fromColor then
// encodeRGBA (removeGamma of linear = identity, round, integer premultiply).
__attribute__((visibility("default"))) z2d_pixel z2doracle_pixel_from_color(z2d_color c) {
    const RGBf l = linear_from_color(c);
    auto rd = [](float v) { return (uint16_t)(int32_t)std::round(255.0f * v); };
    I16 v{rd(l.r), rd(l.g), rd(l.b), rd(l.a)};
    v = I16{(uint16_t)(v.r * v.a / 255), (uint16_t)(v.g * v.a / 255), (uint16_t)(v.b * v.a / 255), v.a};
    return z2d_pixel{Z2D_FORMAT_RGBA, (uint8_t)v.r, (uint8_t)v.g, (uint8_t)v.b, (uint8_t)v.a};
}

// Gradient.getOffset (src/gradient.zig:239-243).
// std.math.pow(f32) as restated above (pinned to z2d's gamma KATs).
__attribute__((visibility("default"))) float z2doracle_pow_f32(float x, float y) { return zpow(x, y); }
// std.math.atan2(f64) as restated above.
__attribute__((visibility("default"))) double z2doracle_atan2(double y, double x) { return zatan2(y, x); }

__attribute__((visibility("default"))) float z2doracle_gradient_offset(const z2d_gradient *g, int32_t x, int32_t y) {
    const Grad gr = make_grad(*g);
    return grad_offset(gr, x, y);
}

// The offsets of a w x h block of pixels starting at (x0, y0), row-major.
__attribute__((visibility("default"))) void z2doracle_gradient_offsets(const z2d_gradient *g, int32_t x0, int32_t y0,
                                                                       int32_t w, int32_t h, float *out) {
    const Grad gr = make_grad(*g);
    for (int32_t j = 0; j < h; j++)
        for (int32_t i = 0; i < w; i++) out[(size_t)j * (size_t)w + (size_t)i] = grad_offset(gr, x0 + i, y0 + j);
}

// Edge list of fill_plotter.plot (fill_plotter.zig:21-97): writes up to
// `cap` edges as (y0, y1, x_start, x_inc) and the extents
// (top, bottom, left, right); returns the edge count or a negative status.
__attribute__((visibility("default"))) int64_t z2doracle_plot(const z2d_node *nodes, size_t n, double scale,
                                                              double tolerance, double *edges_out, size_t cap,
                                                              double *extents_out) {
    Poly poly;
    const int rc = plot(nodes, n, scale, tolerance, poly);
    if (rc != Z2D_OK) return -(int64_t)rc;
    for (size_t i = 0; i < poly.edges.size() && i < cap; i++) {
        edges_out[4 * i + 0] = poly.edges[i].y0;
        edges_out[4 * i + 1] = poly.edges[i].y1;
        edges_out[4 * i + 2] = poly.edges[i].x_start;
        edges_out[4 * i + 3] = poly.edges[i].x_inc;
    }
    if (extents_out) {
        extents_out[0] = poly.et;
        extents_out[1] = poly.eb;
        extents_out[2] = poly.el;
        extents_out[3] = poly.er;
    }
    return (int64_t)poly.edges.size();
}

// multisample.addSpan on a fresh coverage buffer of `capacity` pixels,
// followed by more spans; dumps (value, run length) at every run start into
// out[2*i], out[2*i+1] for i < cap.  Returns the buffer length.
__attribute__((visibility("default"))) uint32_t z2doracle_msaa_spans(uint32_t capacity, const uint32_t *spans,
                                                                     size_t n_spans, uint32_t *out, size_t cap) {
    SparseCov cb(capacity);
    for (size_t i = 0; i < n_spans; i++) msaa_add_span(cb, spans[2 * i], spans[2 * i + 1]);
    for (size_t i = 0; i < cb.len && i < cap; i++) {
        out[2 * i] = cb.values[i];
        out[2 * i + 1] = cb.lengths[i];
    }
    return cb.len;
}

// Dither.getPixel-equivalent through the compositor's vector path for one
// lane: fromDitherVecEncode (color_vector.zig:90-104).
__attribute__((visibility("default"))) z2d_pixel z2doracle_dither_pixel(const z2d_pattern *p, int32_t x, int32_t y) {
    const Src s = make_src_from_pattern(Z2D_PARAM_DITHER, *p);
    const I16 v = src_i16(s, x, y);
    return z2d_pixel{Z2D_FORMAT_RGBA, (uint8_t)v.r, (uint8_t)v.g, (uint8_t)v.b, (uint8_t)v.a};
}

// Gradient pixel through the compositor's integer vector path for one lane.
__attribute__((visibility("default"))) z2d_pixel z2doracle_gradient_pixel(const z2d_gradient *g, int32_t x,
                                                                          int32_t y) {
    Src s{};
    s.kind = Z2D_PARAM_GRADIENT;
    s.grad = make_grad(*g);
    const I16 v = src_i16(s, x, y);
    return z2d_pixel{Z2D_FORMAT_RGBA, (uint8_t)v.r, (uint8_t)v.g, (uint8_t)v.b, (uint8_t)v.a};
}

// ===================================================================
// Hairlines                         src/internal/raster/hairline.zig
// ===================================================================
struct Hair {
    Sfc &s;
    const FillSrc &pat;
    int op, prec;
    bool aa_none;
};
static void hair_opaque(Hair &h, int32_t x, int32_t y, size_t len) { composite_opaque(h.op, h.s, h.pat, x, y, len, h.prec); }
static void hair_opacity(Hair &h, int32_t x, int32_t y, uint8_t o) {
    composite_opacity(h.op, h.s, h.pat, x, y, 1, h.prec, o);
}
static void delta_step(int32_t a, int32_t b, int32_t &d, int32_t &st) {  // hairline.zig:373-379
    const int32_t c = b - a;
    if (c < 0) {
        d = -c;
        st = -1;
    } else {
        d = c;
        st = 1;
    }
}
static uint16_t err_inc(int32_t a, int32_t b) {  // hairline.zig:386-394
    if (a == b) return 0xFFFF;
    return (uint16_t)(((uint32_t)a << 16) / (uint32_t)b);
}
static void draw_horizontal(Hair &h, int32_t x0, int32_t x1, int32_t y) {  // hairline.zig:126-142
    const int32_t sx = clampi(std::min(x0, x1), 0, h.s.w - 1), ex = clampi(std::max(x0, x1), 0, h.s.w - 1);
    const int32_t len = ex - sx + 1;
    if (len > 0) hair_opaque(h, sx, y, (size_t)len);
}
static void draw_vertical(Hair &h, int32_t x, int32_t y0, int32_t y1) {  // hairline.zig:144-161
    const int32_t sy = clampi(std::min(y0, y1), 0, h.s.h - 1), ey = clampi(std::max(y0, y1), 0, h.s.h - 1);
    for (int32_t y = sy; y <= ey; y++) hair_opaque(h, x, y, 1);
}
static void draw_bres_horizontal(Hair &h, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {  // hairline.zig:163-199
    if (x0 > x1) return draw_bres_horizontal(h, x1, y1, x0, y0);
    const int32_t dx = x1 - x0;
    int32_t dy, sy;
    delta_step(y0, y1, dy, sy);
    int32_t x = x0, y = y0, d = 2 * dy - dx;
    const int32_t d_inc = 2 * dy, d_dec = 2 * dx;
    for (; x <= x1; x++) {
        hair_opaque(h, x, y, 1);
        if (d > 0) {
            y += sy;
            d -= d_dec;
        }
        d += d_inc;
    }
}
static void draw_bres_vertical(Hair &h, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {  // hairline.zig:201-231
    if (y0 > y1) return draw_bres_vertical(h, x1, y1, x0, y0);
    const int32_t dy = y1 - y0;
    int32_t dx, sx;
    delta_step(x0, x1, dx, sx);
    int32_t x = x0, y = y0, d = 2 * dx - dy;
    const int32_t d_inc = 2 * dx, d_dec = 2 * dy;
    for (; y <= y1; y++) {
        hair_opaque(h, x, y, 1);
        if (d > 0) {
            x += sx;
            d -= d_dec;
        }
        d += d_inc;
    }
}
static void draw_wu_horizontal(Hair &h, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {  // hairline.zig:233-309
    if (x0 > x1) return draw_wu_horizontal(h, x1, y1, x0, y0);
    const int32_t dx = x1 - x0;
    int32_t dy, sy;
    delta_step(y0, y1, dy, sy);
    int32_t x = x0, y = y0;
    uint16_t err = 0;
    const uint16_t inc = err_inc(dy, dx);
    hair_opaque(h, x, y, 1);
    for (x += 1; x < x1; x++) {
        const uint16_t prev = err;
        err = (uint16_t)(err + inc);
        if (err < prev) y += sy;  // overflow
        const uint8_t comp = (uint8_t)(err >> 8);
        hair_opacity(h, x, y, (uint8_t)(comp ^ 0xFF));
        hair_opacity(h, x, y + sy, comp);
    }
    hair_opaque(h, x1, y1, 1);
}
static void draw_wu_vertical(Hair &h, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {  // hairline.zig:311-365
    if (y0 > y1) return draw_wu_vertical(h, x1, y1, x0, y0);
    const int32_t dy = y1 - y0;
    int32_t dx, sx;
    delta_step(x0, x1, dx, sx);
    int32_t x = x0, y = y0;
    uint16_t err = 0;
    const uint16_t inc = err_inc(dx, dy);
    hair_opaque(h, x, y, 1);
    for (y += 1; y < y1; y++) {
        const uint16_t prev = err;
        err = (uint16_t)(err + inc);
        if (err < prev) x += sx;
        const uint8_t comp = (uint8_t)(err >> 8);
        hair_opacity(h, x, y, (uint8_t)(comp ^ 0xFF));
        hair_opacity(h, x + sx, y, comp);
    }
    hair_opaque(h, x1, y1, 1);
}
static void draw_line(Hair &h, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {  // hairline.zig:89-124
    // inBox (hairline.zig:396-406)
    if ((x0 < 0 || x0 >= h.s.w) && (x1 < 0 || x1 >= h.s.w)) return;
    if ((y0 < 0 || y0 >= h.s.h) && (y1 < 0 || y1 >= h.s.h)) return;
    const int32_t dx = std::abs(x1 - x0), dy = std::abs(y1 - y0);
    if (dx == 0) draw_vertical(h, x0, y0, y1);
    else if (dy == 0) draw_horizontal(h, x0, x1, y0);
    else if (dx < dy) h.aa_none ? draw_bres_vertical(h, x0, y0, x1, y1) : draw_wu_vertical(h, x0, y0, x1, y1);
    else h.aa_none ? draw_bres_horizontal(h, x0, y0, x1, y1) : draw_wu_horizontal(h, x0, y0, x1, y1);
}

// hairline_rasterizer.run (hairline.zig:29-81) on polylines given as points
// (polyline_plotter's contours): line_ends[k] is one past polyline k's last
// point.  `anti_aliasing` is the stroke's own option (Bresenham for none,
// Wu otherwise).
__attribute__((visibility("default"))) int z2doracle_hairline(z2d_surface *surface, const z2d_pattern *pattern,
                                                              const double *points, const uint64_t *line_ends,
                                                              size_t n_lines, int32_t op, int32_t precision,
                                                              int32_t anti_aliasing) {
    if (!surface || !pattern || (n_lines && (!points || !line_ends))) return Z2D_ERR_INVALID_ARGUMENT;
    if (surface->width < 1 || surface->height < 1) return Z2D_ERR_INVALID_DIMENSIONS;
    if (pattern->kind == Z2D_PATTERN_PIXEL && !pixel_premultiplied(pattern->pixel))
        return Z2D_ERR_PIXEL_NOT_PREMULTIPLIED;
    Sfc s = sfc_from_abi(surface);
    FillSrc pat;
    pat.kind = pattern->kind;
    const int pk = pattern->kind == Z2D_PATTERN_PIXEL      ? Z2D_PARAM_PIXEL
                   : pattern->kind == Z2D_PATTERN_GRADIENT ? Z2D_PARAM_GRADIENT
                                                           : Z2D_PARAM_DITHER;
    pat.src = make_src_from_pattern(pk, *pattern);
    Hair h{s, pat, op, requires_float(op) ? Z2D_PRECISION_FLOAT : precision, anti_aliasing == Z2D_AA_NONE};
    uint64_t start = 0;
    for (size_t k = 0; k < n_lines; k++) {
        const uint64_t end = line_ends[k];
        auto X = [&](uint64_t i) { return (int32_t)std::round(points[2 * i]); };
        auto Y = [&](uint64_t i) { return (int32_t)std::round(points[2 * i + 1]); };
        if (end == start + 1) hair_opaque(h, X(start), Y(start), 1);
        for (uint64_t i = start; end > start + 1 && i + 1 < end; i++) draw_line(h, X(i), Y(i), X(i + 1), Y(i + 1));
        start = end;
    }
    return Z2D_OK;
}

// ===================================================================
// PNG scanlines                     src/export_png.zig:153-372
// ===================================================================
// The unfiltered image data writeToPNGFile compresses: per row a 0 filter
// byte, then the row's pixels as writePNGIDATStream encodes them.
// `profile`: -1 none, 0 linear, 1 sRGB (gamma applied by encodeRGBAVec).
// Writes at most `cap` bytes to `out`; returns the full size in *len.
__attribute__((visibility("default"))) int z2doracle_png_scanlines(const z2d_surface *surface, int32_t profile,
                                                                   uint8_t *out, size_t cap, size_t *len) {
    if (!surface || !len) return Z2D_ERR_INVALID_ARGUMENT;
    if (surface->width < 1 || surface->height < 1) return Z2D_ERR_INVALID_DIMENSIONS;
    const Sfc s = sfc_from_abi(surface);
    const bool wide = s.fmt == Z2D_FORMAT_RGBA || s.fmt == Z2D_FORMAT_ARGB || s.fmt == Z2D_FORMAT_RGB ||
                      s.fmt == Z2D_FORMAT_XRGB;
    const bool alpha = s.fmt == Z2D_FORMAT_RGBA || s.fmt == Z2D_FORMAT_ARGB;
    const size_t bits = wide ? (alpha ? 32 : 24) : (size_t)fmt_bits(s.fmt);
    const size_t row_bytes = 1 + ((size_t)s.w * bits + 7) / 8;
    *len = row_bytes * (size_t)s.h;
    std::vector<uint8_t> row(row_bytes);
    for (int32_t y = 0; y < s.h; y++) {
        std::fill(row.begin(), row.end(), 0);
        for (int32_t x = 0; x < s.w; x++) {
            const Px p = raw_get(s, (size_t)s.w * y + x);
            if (wide) {  // encodeRGBAVec
                uint32_t r = p.r, g = p.g, b = p.b, a = alpha ? p.a : 255;
                if (alpha) {  // RGBA16.demultiply
                    r = a == 0 ? 0 : r * 255 / std::max(1u, a);
                    g = a == 0 ? 0 : g * 255 / std::max(1u, a);
                    b = a == 0 ? 0 : b * 255 / std::max(1u, a);
                }
                if (profile == 1) {  // decodeRGBAVecRaw, applyGammaVec, encodeRGBAVecRaw
                    auto enc = [](uint32_t c, bool gamma) {
                        float v = (float)c / 255.0f;
                        if (gamma) v = zpow(v, kInvGamma);
                        return (uint32_t)std::round(255.0f * v);
                    };
                    r = enc(r, true);
                    g = enc(g, true);
                    b = enc(b, true);
                    a = enc(a, false);
                }
                uint8_t *o = row.data() + 1 + (size_t)x * (alpha ? 4 : 3);
                o[0] = (uint8_t)r;
                o[1] = (uint8_t)g;
                o[2] = (uint8_t)b;
                if (alpha) o[3] = (uint8_t)a;
            } else if (s.fmt == Z2D_FORMAT_ALPHA8) {
                row[1 + (size_t)x] = p.a;
            } else {  // most significant bits first
                const int nb = fmt_bits(s.fmt), per = 8 / nb;
                row[1 + (size_t)x / per] |= (uint8_t)(p.a << (8 - nb - (x % per) * nb));
            }
        }
        const size_t at = row_bytes * (size_t)y;
        if (out && at < cap) memcpy(out + at, row.data(), std::min(row_bytes, cap - at));
    }
    return Z2D_OK;
}

// The rasterisers of painter.fill / painter.stroke on a polygon given as
// closed contours of already-scaled points (Polygon.addEdgesFromContour,
// Polygon.zig:115-139, with the polygon's own scale of 1), as
// painter.stroke hands its stroke polygon over (painter.zig:306-341).
// contour_ends[k] is one past contour k's last point.
__attribute__((visibility("default"))) int z2doracle_fill_contours(z2d_surface *surface, const z2d_pattern *pattern,
                                                                   const double *points, const uint64_t *contour_ends,
                                                                   size_t n_contours, const z2d_fill_opts *opts) {
    if (!surface || !pattern || !opts || (n_contours && (!points || !contour_ends))) return Z2D_ERR_INVALID_ARGUMENT;
    if (surface->width < 1 || surface->height < 1) return Z2D_ERR_INVALID_DIMENSIONS;
    if (pattern->kind == Z2D_PATTERN_PIXEL && !pixel_premultiplied(pattern->pixel))
        return Z2D_ERR_PIXEL_NOT_PREMULTIPLIED;
    Sfc s = sfc_from_abi(surface);
    const int aa = (s.fmt == Z2D_FORMAT_ALPHA1) ? Z2D_AA_NONE : opts->anti_aliasing;
    Poly poly;
    uint64_t start = 0;
    for (size_t k = 0; k < n_contours; k++) {
        const uint64_t end = contour_ends[k];
        for (uint64_t i = start; i + 1 < end; i++)
            poly.add_edge(Pt{points[2 * i], points[2 * i + 1]}, Pt{points[2 * i + 2], points[2 * i + 3]});
        if (end > start)
            poly.add_edge(Pt{points[2 * (end - 1)], points[2 * (end - 1) + 1]}, Pt{points[2 * start], points[2 * start + 1]});
        start = end;
    }
    FillSrc pat;
    pat.kind = pattern->kind;
    const int pk = pattern->kind == Z2D_PATTERN_PIXEL      ? Z2D_PARAM_PIXEL
                   : pattern->kind == Z2D_PATTERN_GRADIENT ? Z2D_PARAM_GRADIENT
                                                           : Z2D_PARAM_DITHER;
    pat.src = make_src_from_pattern(pk, *pattern);
    if (poly.edges.empty()) return Z2D_OK;
    if (!(std::isfinite(poly.el) && std::isfinite(poly.et) && std::isfinite(poly.er) && std::isfinite(poly.eb)))
        return Z2D_ERR_INVALID_STATE;
    switch (aa) {
        case Z2D_AA_NONE: run_direct(s, pat, poly, opts->fill_rule, opts->op, opts->precision); break;
        case Z2D_AA_SUPERSAMPLE_4X: run_ssaa(s, pat, poly, opts->fill_rule, opts->op, opts->precision); break;
        default: run_msaa(s, pat, poly, opts->fill_rule, opts->op, opts->precision); break;
    }
    return Z2D_OK;
}

}  // extern "C"
