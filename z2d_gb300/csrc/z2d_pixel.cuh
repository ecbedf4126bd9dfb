// z2d_pixel.cuh -- device-side pixel formats, operators, colors, gradients
// and dither for the GB300 fill/composite path.
//
// Everything here reproduces z2d's per-pixel arithmetic exactly (the file
// is compiled with --fmad=false and IEEE division/sqrt, so every float and
// double operation rounds like z2d's strict-IEEE Zig code).  Cited lines are
// in the z2d project.
#pragma once
#include <stdint.h>

#include "../../include/z2dgpu.h"
#include "grad_fast.cuh"
#include "zig_math.cuh"

#define Z2D_HD __host__ __device__ __forceinline__
#define Z2D_D __device__ __forceinline__

namespace z2dg {

constexpr int kMaxStops = 32;

// ---------------------------------------------------------------- formats
Z2D_HD int fmt_bits(int f) {
    return f == Z2D_FORMAT_ALPHA8 ? 8 : f == Z2D_FORMAT_ALPHA4 ? 4 : f == Z2D_FORMAT_ALPHA2 ? 2 : f == Z2D_FORMAT_ALPHA1 ? 1 : 32;
}
Z2D_HD bool fmt_packed(int f) { return f >= Z2D_FORMAT_ALPHA4; }
Z2D_HD bool fmt_has_color(int f) { return f <= Z2D_FORMAT_RGBA; }
Z2D_HD bool fmt_has_alpha(int f) { return f == Z2D_FORMAT_ARGB || f == Z2D_FORMAT_RGBA || f >= Z2D_FORMAT_ALPHA8; }
Z2D_HD uint32_t fmt_max(int f) {
    return f == Z2D_FORMAT_ALPHA4 ? 15u : f == Z2D_FORMAT_ALPHA2 ? 3u : f == Z2D_FORMAT_ALPHA1 ? 1u : 255u;
}

// Alpha(T).scaleIntoIntAlpha / shlr (src/pixel.zig:582-626)
Z2D_HD uint32_t scale_alpha(uint32_t v, int from, int to) {
    if (from == 1) return v * ((1u << to) - 1u);
    if (v == 0) return 0;
    if (from == to) return v;
    if (from > to) return v >> (from - to);
    const int d = to - from;
    if (d == 2 || d == 4) return (v << d) + v;
    return (v << d) | (v << (to - 2 * from)) | (v << (to - 3 * from)) | v;
}

// RGBA16 lane (src/compositor.zig:664-703); u16 semantics kept in u32.
struct I16 {
    uint32_t r, g, b, a;
};
struct F4 {
    float r, g, b, a;
};

// A pixel of a given format held as 4 bytes (src/pixel.zig:101-110).
struct Px {
    int fmt;
    uint32_t r, g, b, a;
};

// T.fromPixel (src/pixel.zig:399-433, 569-577)
Z2D_HD Px convert_px(Px p, int to) {
    if (p.fmt == to) return p;
    Px o{to, 0, 0, 0, 0};
    if (fmt_has_color(to)) {
        if (fmt_has_color(p.fmt)) {
            o.r = p.r; o.g = p.g; o.b = p.b;
            o.a = fmt_has_alpha(p.fmt) ? p.a : 255u;
        } else {
            o.a = scale_alpha(p.a, fmt_bits(p.fmt), 8);
        }
        if (!fmt_has_alpha(to)) o.a = 0;
        return o;
    }
    if (p.fmt == Z2D_FORMAT_XRGB || p.fmt == Z2D_FORMAT_RGB) {
        o.a = fmt_max(to);
    } else {
        const int fb = (p.fmt == Z2D_FORMAT_ARGB || p.fmt == Z2D_FORMAT_RGBA) ? 8 : fmt_bits(p.fmt);
        o.a = scale_alpha(p.a, fb, fmt_bits(to));
    }
    return o;
}

// RGBA16.fromPixelT / fromStride lane (src/compositor.zig:675-682, 718-747)
Z2D_HD I16 to_i16(Px p) {
    if (fmt_has_color(p.fmt)) return I16{p.r, p.g, p.b, fmt_has_alpha(p.fmt) ? p.a : 255u};
    return I16{0, 0, 0, scale_alpha(p.a, fmt_bits(p.fmt), 8)};
}
// RGBA16.toPixelT / toStride lane (src/compositor.zig:688-698, 806-833)
Z2D_HD Px from_i16(I16 v, int fmt) {
    Px p{fmt, 0, 0, 0, 0};
    if (fmt_has_color(fmt)) {
        p.r = v.r & 0xFFu; p.g = v.g & 0xFFu; p.b = v.b & 0xFFu;
        p.a = fmt_has_alpha(fmt) ? (v.a & 0xFFu) : 0u;
    } else {
        p.a = scale_alpha(v.a & 0xFFu, 8, fmt_bits(fmt));
    }
    return p;
}
Z2D_HD I16 i16_from_pixel(Px p) { return to_i16(convert_px(p, Z2D_FORMAT_RGBA)); }

// 32-bit word <-> pixel for the 4-byte formats (byte order in memory)
Z2D_HD I16 word_to_i16(uint32_t w, int fmt) {
    const uint32_t b0 = w & 0xFFu, b1 = (w >> 8) & 0xFFu, b2 = (w >> 16) & 0xFFu, b3 = w >> 24;
    switch (fmt) {
        case Z2D_FORMAT_ARGB: return I16{b2, b1, b0, b3};
        case Z2D_FORMAT_XRGB: return I16{b2, b1, b0, 255u};
        case Z2D_FORMAT_RGB: return I16{b0, b1, b2, 255u};
        default: return I16{b0, b1, b2, b3};
    }
}
Z2D_HD uint32_t i16_to_word(I16 v, int fmt) {
    const uint32_t r = v.r & 0xFFu, g = v.g & 0xFFu, b = v.b & 0xFFu, a = v.a & 0xFFu;
    switch (fmt) {
        case Z2D_FORMAT_ARGB: return b | (g << 8) | (r << 16) | (a << 24);
        case Z2D_FORMAT_XRGB: return b | (g << 8) | (r << 16);
        case Z2D_FORMAT_RGB: return r | (g << 8) | (b << 16);
        default: return r | (g << 8) | (b << 16) | (a << 24);
    }
}
Z2D_HD uint32_t px_to_word(Px p) { return i16_to_word(I16{p.r, p.g, p.b, p.a}, p.fmt); }

// Byte order of a source word for word_src_over on a 4-byte format: the
// colour bytes in the surface's order, alpha in byte 3.
Z2D_HD int word_order(int fmt) {
    return (fmt == Z2D_FORMAT_ARGB || fmt == Z2D_FORMAT_XRGB) ? Z2D_FORMAT_ARGB : Z2D_FORMAT_RGBA;
}

// floor(t / 255) in both 16-bit lanes of t, each lane at most 255 * 255:
// on [0, 65025], floor(t / 255) == (t + floor(t / 256) + 1) >> 8, and no
// lane carries into the other.
Z2D_HD uint32_t div255x2(uint32_t t) {
    return ((t + ((t >> 8) & 0x00FF00FFu) + 0x00010001u) >> 8) & 0x00FF00FFu;
}

// IntegerOps.srcOver (src/compositor.zig:1223-1230) of source word L over
// destination word w of a 4-byte format, two channels per 32-bit operation:
//   c = w16(s_c + d_c * (255 - s_a) / 255),  a = w16(s_a + d_a - s_a * d_a / 255)
// stored as their low bytes.  L is in word_order(fmt) with the source alpha
// in byte 3; without an alpha channel (XRGB, RGB) byte 3 is written as 0.
Z2D_HD uint32_t word_src_over(uint32_t w, uint32_t L, bool has_alpha) {
    const uint32_t ra = L >> 24, inv = 255u - ra;
    const uint32_t e = div255x2((w & 0x00FF00FFu) * inv) + (L & 0x00FF00FFu);
    const uint32_t o = div255x2(((w >> 8) & 0x00FF00FFu) * inv) + ((L >> 8) & 0x00FF00FFu);
    uint32_t out = (e & 0x00FF00FFu) | ((o & 0xFFu) << 8);
    if (has_alpha) {
        const uint32_t da = w >> 24;
        out |= ((ra + da - (ra * da) / 255u) & 0xFFu) << 24;
    }
    return out;
}

// Surface access by flat pixel index (w*y+x).  Packed formats are LSB
// first (src/pixel.zig:664-677).
struct DevSurface {
    uint8_t *data;
    int32_t fmt, w, h;
};

Z2D_D I16 load_px(const DevSurface &s, size_t i) {
    if (s.fmt <= Z2D_FORMAT_RGBA) return word_to_i16(reinterpret_cast<const uint32_t *>(s.data)[i], s.fmt);
    if (s.fmt == Z2D_FORMAT_ALPHA8) return I16{0, 0, 0, s.data[i]};
    const int bits = fmt_bits(s.fmt);
    const size_t bit = i * (size_t)bits;
    const uint32_t v = (s.data[bit >> 3] >> (bit & 7)) & ((1u << bits) - 1u);
    return I16{0, 0, 0, scale_alpha(v, bits, 8)};
}
// Packed stores use word atomics so that threads owning different pixels of
// one byte never race.
Z2D_D void store_raw_packed(const DevSurface &s, size_t i, uint32_t v) {
    const int bits = fmt_bits(s.fmt);
    const size_t bit = i * (size_t)bits;
    uint32_t *word = reinterpret_cast<uint32_t *>(s.data + ((bit >> 3) & ~(size_t)3));
    const uint32_t sh = (uint32_t)(bit & 31);
    const uint32_t mask = ((1u << bits) - 1u) << sh;
    atomicAnd(word, ~mask);
    atomicOr(word, (v << sh) & mask);
}
Z2D_D void store_px(const DevSurface &s, size_t i, I16 v) {
    if (s.fmt <= Z2D_FORMAT_RGBA) {
        reinterpret_cast<uint32_t *>(s.data)[i] = i16_to_word(v, s.fmt);
    } else if (s.fmt == Z2D_FORMAT_ALPHA8) {
        s.data[i] = (uint8_t)v.a;
    } else {
        store_raw_packed(s, i, scale_alpha(v.a & 0xFFu, 8, fmt_bits(s.fmt)));
    }
}
// Store of a pixel already converted to the surface format (paintStride).
Z2D_D void store_converted(const DevSurface &s, size_t i, Px p) {
    if (s.fmt <= Z2D_FORMAT_RGBA) reinterpret_cast<uint32_t *>(s.data)[i] = px_to_word(p);
    else if (s.fmt == Z2D_FORMAT_ALPHA8) s.data[i] = (uint8_t)p.a;
    else store_raw_packed(s, i, p.a);
}

// ---------------------------------------------------- integer operators
// src/compositor.zig:1158-1568.  u16 results wrap.
Z2D_HD int32_t imul(int32_t a, int32_t b) { return (a * b) / 255; }
Z2D_HD int32_t invMul(int32_t a, int32_t b) { return imul(a, 255 - b); }
Z2D_HD int32_t rInvMul(int32_t a, int32_t b) { return imul(a, 255 + b); }
Z2D_HD uint32_t w16(int32_t v) { return (uint32_t)v & 0xFFFFu; }
Z2D_HD int32_t imin(int32_t a, int32_t b) { return a < b ? a : b; }
Z2D_HD int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }

Z2D_HD uint32_t overlay_ch(int32_t sca, int32_t dca, int32_t sa, int32_t da) {
    if ((int32_t)w16(dca * 2) <= da) return w16(imul(sca * 2, dca) + invMul(sca, da) + invMul(dca, sa));
    return w16(rInvMul(sca, da) + rInvMul(dca, sa) - imul(dca * 2, sca) - imul(da, sa));
}
Z2D_HD uint32_t hardlight_ch(int32_t sca, int32_t dca, int32_t sa, int32_t da) {
    if ((int32_t)w16(sca * 2) <= sa) return w16(imul(sca * 2, dca) + invMul(sca, da) + invMul(dca, sa));
    return w16(rInvMul(sca, da) + rInvMul(dca, sa) - imul(sa, da) - imul(sca * 2, dca));
}

Z2D_HD I16 int_op(int op, I16 d, I16 s) {
    const int32_t dr = d.r, dg = d.g, db = d.b, da = d.a, sr = s.r, sg = s.g, sb = s.b, sa = s.a;
    const uint32_t au = w16(sa + da - imul(sa, da));
    switch (op) {
        case Z2D_OP_CLEAR: return I16{0, 0, 0, 0};
        case Z2D_OP_SRC: return s;
        case Z2D_OP_DST: return d;
        case Z2D_OP_SRC_OVER: return I16{w16(sr + invMul(dr, sa)), w16(sg + invMul(dg, sa)), w16(sb + invMul(db, sa)), au};
        case Z2D_OP_DST_OVER: return I16{w16(dr + invMul(sr, da)), w16(dg + invMul(sg, da)), w16(db + invMul(sb, da)), au};
        case Z2D_OP_SRC_IN: return I16{w16(imul(sr, da)), w16(imul(sg, da)), w16(imul(sb, da)), w16(imul(sa, da))};
        case Z2D_OP_DST_IN: return I16{w16(imul(dr, sa)), w16(imul(dg, sa)), w16(imul(db, sa)), w16(imul(da, sa))};
        case Z2D_OP_SRC_OUT: return I16{w16(invMul(sr, da)), w16(invMul(sg, da)), w16(invMul(sb, da)), w16(invMul(sa, da))};
        case Z2D_OP_DST_OUT: return I16{w16(invMul(dr, sa)), w16(invMul(dg, sa)), w16(invMul(db, sa)), w16(invMul(da, sa))};
        case Z2D_OP_SRC_ATOP:
            return I16{w16(imul(sr, da) + invMul(dr, sa)), w16(imul(sg, da) + invMul(dg, sa)), w16(imul(sb, da) + invMul(db, sa)), (uint32_t)da};
        case Z2D_OP_DST_ATOP:
            return I16{w16(imul(dr, sa) + invMul(sr, da)), w16(imul(dg, sa) + invMul(sg, da)), w16(imul(db, sa) + invMul(sb, da)), (uint32_t)sa};
        case Z2D_OP_XOR:
            return I16{w16(invMul(sr, da) + invMul(dr, sa)), w16(invMul(sg, da) + invMul(dg, sa)),
                       w16(invMul(sb, da) + invMul(db, sa)), w16(invMul(sa, da) + invMul(da, sa))};
        case Z2D_OP_PLUS: return I16{w16(imin(255, sr + dr)), w16(imin(255, sg + dg)), w16(imin(255, sb + db)), w16(imin(255, sa + da))};
        case Z2D_OP_MULTIPLY:
            return I16{w16(imul(sr, dr) + invMul(sr, da) + invMul(dr, sa)), w16(imul(sg, dg) + invMul(sg, da) + invMul(dg, sa)),
                       w16(imul(sb, db) + invMul(sb, da) + invMul(db, sa)), au};
        case Z2D_OP_SCREEN: return I16{w16(sr + dr - imul(sr, dr)), w16(sg + dg - imul(sg, dg)), w16(sb + db - imul(sb, db)), au};
        case Z2D_OP_OVERLAY: return I16{overlay_ch(sr, dr, sa, da), overlay_ch(sg, dg, sa, da), overlay_ch(sb, db, sa, da), au};
        case Z2D_OP_DARKEN:
            return I16{w16(imin(imul(sr, da), imul(dr, sa)) + invMul(sr, da) + invMul(dr, sa)),
                       w16(imin(imul(sg, da), imul(dg, sa)) + invMul(sg, da) + invMul(dg, sa)),
                       w16(imin(imul(sb, da), imul(db, sa)) + invMul(sb, da) + invMul(db, sa)), au};
        case Z2D_OP_LIGHTEN:
            return I16{w16(imax(imul(sr, da), imul(dr, sa)) + invMul(sr, da) + invMul(dr, sa)),
                       w16(imax(imul(sg, da), imul(dg, sa)) + invMul(sg, da) + invMul(dg, sa)),
                       w16(imax(imul(sb, da), imul(db, sa)) + invMul(sb, da) + invMul(db, sa)), au};
        case Z2D_OP_HARD_LIGHT: return I16{hardlight_ch(sr, dr, sa, da), hardlight_ch(sg, dg, sa, da), hardlight_ch(sb, db, sa, da), au};
        case Z2D_OP_DIFFERENCE:
            return I16{w16(sr + dr - 2 * imin(imul(sr, da), imul(dr, sa))), w16(sg + dg - 2 * imin(imul(sg, da), imul(dg, sa))),
                       w16(sb + db - 2 * imin(imul(sb, da), imul(db, sa))), au};
        case Z2D_OP_EXCLUSION:
            return I16{w16((imul(sr, da) + imul(dr, sa) - 2 * imul(sr, dr)) + invMul(sr, da) + invMul(dr, sa)),
                       w16((imul(sg, da) + imul(dg, sa) - 2 * imul(sg, dg)) + invMul(sg, da) + invMul(dg, sa)),
                       w16((imul(sb, da) + imul(db, sa) - 2 * imul(sb, db)) + invMul(sb, da) + invMul(db, sa)), au};
        default: return I16{0, 0, 0, 0};  // float-only operators run as clear (:1179-1188)
    }
}

Z2D_HD bool requires_float(int op) {
    return op == Z2D_OP_COLOR_DODGE || op == Z2D_OP_COLOR_BURN || op == Z2D_OP_SOFT_LIGHT || op == Z2D_OP_HUE ||
           op == Z2D_OP_SATURATION || op == Z2D_OP_COLOR || op == Z2D_OP_LUMINOSITY;
}
Z2D_HD bool is_bounded(int op) {
    return !(op == Z2D_OP_SRC_IN || op == Z2D_OP_DST_IN || op == Z2D_OP_SRC_OUT || op == Z2D_OP_DST_ATOP);
}

// ------------------------------------------------------ float operators
// src/compositor.zig:1571-2440, vector form.  fminf/fmaxf return the
// non-NaN operand like Zig's @min/@max.
Z2D_HD float fmin3(float a, float b, float c) { return fminf(fminf(a, b), c); }
Z2D_HD float fmax3(float a, float b, float c) { return fmaxf(fmaxf(a, b), c); }

Z2D_D float f_overlay(float sca, float dca, float sa, float da) {
    if (2.0f * dca <= da) return 2.0f * sca * dca + sca * (1.0f - da) + dca * (1.0f - sa);
    return sca * (1.0f + da) + dca * (1.0f + sa) - 2.0f * dca * sca - da * sa;
}
Z2D_D float f_dodge(float sca, float dca, float sa, float da) {
    if (sca == sa && dca == 0.0f) return sca * (1.0f - da);
    if (sca == sa) return sa * da + sca * (1.0f - da) + dca * (1.0f - sa);
    return sa * da * fminf(1.0f, dca / da * sa / (sa - sca)) + sca * (1.0f - da) + dca * (1.0f - sa);
}
Z2D_D float f_burn(float sca, float dca, float sa, float da) {
    // first case tests dca == sa: p0 is called with sa in its da slot (:1915)
    if (sca == 0.0f && dca == sa) return sa * da + dca * (1.0f - sa);
    if (sca == 0.0f) return dca * (1.0f - sa);
    return sa * da * (1.0f - fminf(1.0f, (1.0f - dca / da) * sa / sca)) + sca * (1.0f - da) + dca * (1.0f - sa);
}
Z2D_D float f_hardlight(float sca, float dca, float sa, float da) {
    if (2.0f * sca <= sa) return 2.0f * sca * dca + sca * (1.0f - da) + dca * (1.0f - sa);
    return sca * (1.0f + da) + dca * (1.0f + sa) - sa * da - 2.0f * sca * dca;
}
Z2D_D float f_softlight(float sca, float dca, float sa, float da) {
    if (da == 0.0f) return sca;
    const float m = dca / da;
    if (2.0f * sca <= sa) return dca * (sa + (2.0f * sca - sa) * (1.0f - m)) + sca * (1.0f - da) + dca * (1.0f - sa);
    if (4.0f * dca <= da)
        return dca * sa + da * (2.0f * sca - sa) * (4.0f * m * (4.0f * m + 1.0f) * (m - 1.0f) + 7.0f * m) + sca * (1.0f - da) +
               dca * (1.0f - sa);
    return da * (2.0f * sca - sa) * (sqrtf(m) - m) + sca - sca * da + dca;
}
struct F3 {
    float r, g, b;
};
Z2D_D float ns_lum(F3 c) { return c.r * 0.3f + c.g * 0.59f + c.b * 0.11f; }
Z2D_D float ns_sat(F3 c) { return fmax3(c.r, c.g, c.b) - fmin3(c.r, c.g, c.b); }
Z2D_D F3 ns_set_lum(F3 c, float l) {
    const float d = l - ns_lum(c);
    return F3{c.r + d, c.g + d, c.b + d};
}
Z2D_D float ns_sat_ch(float v, float n, float s, float d) { return d == 0.0f ? 0.0f : (v - n) * s / d; }
Z2D_D F3 ns_set_sat(F3 c, float s) {
    const float n = fmin3(c.r, c.g, c.b), x = fmax3(c.r, c.g, c.b), d = x - n;
    return F3{ns_sat_ch(c.r, n, s, d), ns_sat_ch(c.g, n, s, d), ns_sat_ch(c.b, n, s, d)};
}
Z2D_D float ns_clip_ch(float cv, float l, float n, float x, float a) {
    // vector clipColor (:2272-2307): the x > a case wins when both apply
    float r = cv;
    const float tln = l - n, txl = x - l;
    if (n < 0.0f) r = (tln == 0.0f) ? 0.0f : l + ((cv - l) * l) / tln;
    if (x > a) r = (txl == 0.0f) ? 0.0f : l + ((cv - l) * (a - l)) / txl;
    return r;
}
Z2D_D F3 ns_clip(F3 c, float a) {
    const float l = ns_lum(c), n = fmin3(c.r, c.g, c.b), x = fmax3(c.r, c.g, c.b);
    return F3{ns_clip_ch(c.r, l, n, x, a), ns_clip_ch(c.g, l, n, x, a), ns_clip_ch(c.b, l, n, x, a)};
}
Z2D_D F4 ns_out(F3 c, F4 d, F4 s) {
    return F4{s.r * (1.0f - d.a) + d.r * (1.0f - s.a) + c.r, s.g * (1.0f - d.a) + d.g * (1.0f - s.a) + c.g,
              s.b * (1.0f - d.a) + d.b * (1.0f - s.a) + c.b, s.a + d.a - s.a * d.a};
}

Z2D_D F4 float_op(int op, F4 d, F4 s) {
    const float au = s.a + d.a - s.a * d.a;
    switch (op) {
        case Z2D_OP_CLEAR: return F4{0.f, 0.f, 0.f, 0.f};
        case Z2D_OP_SRC: return s;
        case Z2D_OP_DST: return d;
        case Z2D_OP_SRC_OVER: return F4{s.r + d.r * (1.0f - s.a), s.g + d.g * (1.0f - s.a), s.b + d.b * (1.0f - s.a), au};
        case Z2D_OP_DST_OVER: return F4{d.r + s.r * (1.0f - d.a), d.g + s.g * (1.0f - d.a), d.b + s.b * (1.0f - d.a), au};
        case Z2D_OP_SRC_IN: return F4{s.r * d.a, s.g * d.a, s.b * d.a, s.a * d.a};
        case Z2D_OP_DST_IN: return F4{d.r * s.a, d.g * s.a, d.b * s.a, s.a * d.a};
        case Z2D_OP_SRC_OUT: return F4{s.r * (1.0f - d.a), s.g * (1.0f - d.a), s.b * (1.0f - d.a), s.a * (1.0f - d.a)};
        case Z2D_OP_DST_OUT: return F4{d.r * (1.0f - s.a), d.g * (1.0f - s.a), d.b * (1.0f - s.a), d.a * (1.0f - s.a)};
        case Z2D_OP_SRC_ATOP: return F4{s.r * d.a + d.r * (1.0f - s.a), s.g * d.a + d.g * (1.0f - s.a), s.b * d.a + d.b * (1.0f - s.a), d.a};
        case Z2D_OP_DST_ATOP: return F4{d.r * s.a + s.r * (1.0f - d.a), d.g * s.a + s.g * (1.0f - d.a), d.b * s.a + s.b * (1.0f - d.a), s.a};
        case Z2D_OP_XOR:
            return F4{s.r * (1.0f - d.a) + d.r * (1.0f - s.a), s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      s.b * (1.0f - d.a) + d.b * (1.0f - s.a), s.a + d.a - 2.0f * s.a * d.a};
        case Z2D_OP_PLUS: return F4{fminf(1.0f, s.r + d.r), fminf(1.0f, s.g + d.g), fminf(1.0f, s.b + d.b), fminf(1.0f, s.a + d.a)};
        case Z2D_OP_MULTIPLY:
            return F4{s.r * d.r + s.r * (1.0f - d.a) + d.r * (1.0f - s.a), s.g * d.g + s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      s.b * d.b + s.b * (1.0f - d.a) + d.b * (1.0f - s.a), au};
        case Z2D_OP_SCREEN: return F4{s.r + d.r - s.r * d.r, s.g + d.g - s.g * d.g, s.b + d.b - s.b * d.b, au};
        case Z2D_OP_OVERLAY: return F4{f_overlay(s.r, d.r, s.a, d.a), f_overlay(s.g, d.g, s.a, d.a), f_overlay(s.b, d.b, s.a, d.a), au};
        case Z2D_OP_DARKEN:
            return F4{fminf(s.r * d.a, d.r * s.a) + s.r * (1.0f - d.a) + d.r * (1.0f - s.a),
                      fminf(s.g * d.a, d.g * s.a) + s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      fminf(s.b * d.a, d.b * s.a) + s.b * (1.0f - d.a) + d.b * (1.0f - s.a), au};
        case Z2D_OP_LIGHTEN:
            return F4{fmaxf(s.r * d.a, d.r * s.a) + s.r * (1.0f - d.a) + d.r * (1.0f - s.a),
                      fmaxf(s.g * d.a, d.g * s.a) + s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      fmaxf(s.b * d.a, d.b * s.a) + s.b * (1.0f - d.a) + d.b * (1.0f - s.a), au};
        case Z2D_OP_COLOR_DODGE: return F4{f_dodge(s.r, d.r, s.a, d.a), f_dodge(s.g, d.g, s.a, d.a), f_dodge(s.b, d.b, s.a, d.a), au};
        case Z2D_OP_COLOR_BURN: return F4{f_burn(s.r, d.r, s.a, d.a), f_burn(s.g, d.g, s.a, d.a), f_burn(s.b, d.b, s.a, d.a), au};
        case Z2D_OP_HARD_LIGHT:
            return F4{f_hardlight(s.r, d.r, s.a, d.a), f_hardlight(s.g, d.g, s.a, d.a), f_hardlight(s.b, d.b, s.a, d.a), au};
        case Z2D_OP_SOFT_LIGHT:
            return F4{f_softlight(s.r, d.r, s.a, d.a), f_softlight(s.g, d.g, s.a, d.a), f_softlight(s.b, d.b, s.a, d.a), au};
        case Z2D_OP_DIFFERENCE:
            return F4{s.r + d.r - 2.0f * fminf(s.r * d.a, d.r * s.a), s.g + d.g - 2.0f * fminf(s.g * d.a, d.g * s.a),
                      s.b + d.b - 2.0f * fminf(s.b * d.a, d.b * s.a), au};
        case Z2D_OP_EXCLUSION:
            return F4{(s.r * d.a + d.r * s.a - 2.0f * s.r * d.r) + s.r * (1.0f - d.a) + d.r * (1.0f - s.a),
                      (s.g * d.a + d.g * s.a - 2.0f * s.g * d.g) + s.g * (1.0f - d.a) + d.g * (1.0f - s.a),
                      (s.b * d.a + d.b * s.a - 2.0f * s.b * d.b) + s.b * (1.0f - d.a) + d.b * (1.0f - s.a), au};
        case Z2D_OP_HUE: {
            F3 c{s.r * s.a, s.g * s.a, s.b * s.a};
            const F3 cd{d.r, d.g, d.b};
            c = ns_set_sat(c, ns_sat(cd) * s.a);
            c = ns_set_lum(c, ns_lum(cd) * s.a);
            return ns_out(ns_clip(c, s.a * d.a), d, s);
        }
        case Z2D_OP_SATURATION: {
            F3 c{d.r * s.a, d.g * s.a, d.b * s.a};
            const F3 cs{s.r, s.g, s.b}, cd{d.r, d.g, d.b};
            c = ns_set_sat(c, ns_sat(cs) * d.a);
            c = ns_set_lum(c, ns_lum(cd) * s.a);
            return ns_out(ns_clip(c, s.a * d.a), d, s);
        }
        case Z2D_OP_COLOR: {
            F3 c{s.r * d.a, s.g * d.a, s.b * d.a};
            const F3 cd{d.r, d.g, d.b};
            c = ns_set_lum(c, ns_lum(cd) * s.a);
            return ns_out(ns_clip(c, s.a * d.a), d, s);
        }
        case Z2D_OP_LUMINOSITY: {
            F3 c{d.r * s.a, d.g * s.a, d.b * s.a};
            const F3 cs{s.r, s.g, s.b};
            c = ns_set_lum(c, ns_lum(cs) * d.a);
            return ns_out(ns_clip(c, s.a * d.a), d, s);
        }
        default: return F4{0.f, 0.f, 0.f, 0.f};
    }
}

Z2D_D F4 decode_raw(I16 v) { return F4{(float)v.r / 255.0f, (float)v.g / 255.0f, (float)v.b / 255.0f, (float)v.a / 255.0f}; }
Z2D_D uint32_t enc_ch(float x) {
    const float r = roundf(255.0f * x);
    if (!(r == r)) return 0;
    return (uint32_t)(int32_t)r & 0xFFFFu;
}
Z2D_D I16 encode_raw(F4 v) { return I16{enc_ch(v.r), enc_ch(v.g), enc_ch(v.b), enc_ch(v.a)}; }

// ------------------------------------------------------------ colors
// std.math.pow(f32, x, y) as Zig computes it (zig_math.cuh)
Z2D_HD float zpow(float x, float y) { return zm::powf_(x, y); }
Z2D_HD float zmodf(float a, float b) {
    const float r = fmodf(a, b);
    return a < 0.0f ? fmodf(r + b, b) : r;
}
// fmod, exact: for b <= |a| < 2b the difference a -/+ b is exact (Sterbenz),
// so only operands of two or more periods reach the library fmod.
Z2D_D double fmod_exact(double a, double b) {
    const double m = fabs(a);
    if (m < b) return a;
    if (m < 2.0 * b) return a < 0.0 ? a + b : a - b;
    return fmod(a, b);
}
// Zig's @mod on f64 (fmod, moved into [0, b) for a negative numerator)
Z2D_D double zmod(double a, double b) {
    const double r = fmod_exact(a, b);
    return a < 0.0 ? fmod_exact(r + b, b) : r;
}

constexpr float kGamma = 2.2f;
#define Z2D_INV_GAMMA (1.0f / 2.2f)

struct RGBf {
    float r, g, b, a;
};
struct HSLf {
    float h, s, l, a;
};

Z2D_HD float hsl_ch(float n, float hue, float sat, float light) {
    const float k = fmodf(n + hue / 30.0f, 12.0f);
    const float a = sat * fminf(light, 1.0f - light);
    return light - a * fmaxf(-1.0f, fmin3(k - 3.0f, 9.0f - k, 1.0f));
}
Z2D_HD RGBf hsl_to_rgb(HSLf c) {
    float hue = fmodf(c.h, 360.0f);
    if (hue < 0.0f) hue += 360.0f;
    return RGBf{hsl_ch(0.0f, hue, c.s, c.l), hsl_ch(8.0f, hue, c.s, c.l), hsl_ch(4.0f, hue, c.s, c.l), c.a};
}
Z2D_HD RGBf linear_from_color(const z2d_color &c) {
    RGBf o{c.c[0], c.c[1], c.c[2], c.c[3]};
    if (c.space == Z2D_COLOR_SRGB) {
        o.r = zpow(o.r, kGamma); o.g = zpow(o.g, kGamma); o.b = zpow(o.b, kGamma);
    } else if (c.space == Z2D_COLOR_HSL) {
        o = hsl_to_rgb(HSLf{c.c[0], c.c[1], c.c[2], c.c[3]});
    }
    return o;
}
Z2D_HD RGBf srgb_from_color(const z2d_color &c) {
    if (c.space == Z2D_COLOR_SRGB) return RGBf{c.c[0], c.c[1], c.c[2], c.c[3]};
    const RGBf lin = (c.space == Z2D_COLOR_HSL) ? hsl_to_rgb(HSLf{c.c[0], c.c[1], c.c[2], c.c[3]}) : RGBf{c.c[0], c.c[1], c.c[2], c.c[3]};
    return RGBf{zpow(lin.r, Z2D_INV_GAMMA), zpow(lin.g, Z2D_INV_GAMMA), zpow(lin.b, Z2D_INV_GAMMA), lin.a};
}
Z2D_HD HSLf hsl_from_rgb(RGBf s) {
    const float mx = fmaxf(s.r, fmaxf(s.g, s.b)), mn = fminf(s.r, fminf(s.g, s.b));
    const float range = mx - mn, light = (mn + mx) / 2.0f;
    float sat = (light == 0.0f || light == 1.0f) ? 0.0f : (mx - light) / fminf(light, 1.0f - light);
    float hue = 0.0f;
    if (range != 0.0f) {
        if (mx == s.r) hue = 60.0f * zmodf((s.g - s.b) / range, 6.0f);
        else if (mx == s.g) hue = 60.0f * ((s.b - s.r) / range + 2.0f);
        else if (mx == s.b) hue = 60.0f * ((s.r - s.g) / range + 4.0f);
    }
    if (sat < 0.0f) {
        hue += 180.0f;
        if (hue >= 360.0f) hue -= 360.0f;
        sat = fabsf(sat);
    }
    return HSLf{hue, sat, light, s.a};
}
Z2D_HD HSLf hsl_from_color(const z2d_color &c) {
    if (c.space == Z2D_COLOR_HSL) return HSLf{c.c[0], c.c[1], c.c[2], c.c[3]};
    return hsl_from_rgb(linear_from_color(c));
}
Z2D_D float lerpf(float a, float b, float t) { return a + (b - a) * t; }
Z2D_D I16 premul16(I16 v) {
    return I16{((v.r * v.a) & 0xFFFFu) / 255u, ((v.g * v.a) & 0xFFFFu) / 255u, ((v.b * v.a) & 0xFFFFu) / 255u, v.a};
}
Z2D_D I16 encode_linear(RGBf c) { return premul16(I16{enc_ch(c.r), enc_ch(c.g), enc_ch(c.b), enc_ch(c.a)}); }


// --------------------------------------------------------- gradients
// Gradient prepared on the host: stops clamped and sorted
// (src/gradient.zig:797-811), radial pre-calcs (:401-438), conic angle
// normalised (:666-681).
// Per stop, its colour in the gradient's interpolation space, premultiplied
// by its alpha: LinearRGB (r*a, g*a, b*a, a) for linear_rgb, SRGB the same
// for srgb, HSL (h, s*a, l*a, a) for the hsl methods.  That is the first
// step of interpolateEncode / interpolate on each of the two stops
// (src/color.zig, src/internal/color_vector.zig); it depends on the stop
// only, so it is computed once on the host (same IEEE operations).
struct DevGradient {
    int32_t type, method, n_stops, has_tf;
    double g[6];
    double tf[6];
    double inner_r, outer_r, cdx, cdy, dr, min_dr, a, inv_a, angle;
    // Linear.getOffset's per-gradient terms (src/gradient.zig:355-359):
    // end - start and 1 / |end - start|^2; lin_zero: zero-length gradient
    double lin_dx, lin_dy, lin_inv;
    int32_t lin_zero, pad_;
    // the same offsets on double-word floats (grad_fast.cuh)
    GradFast fz;
    // Up to kMaxStops stops live inline.  A longer stop list (z2d's grows
    // without bound, src/gradient.zig:183-198) is a table in device memory
    // written with the descriptors (ext_off / ext_prep); `src` is the
    // caller's description it is built from, read on the host only.
    const float *ext_off;
    const RGBf *ext_prep;
    const z2d_gradient *src;
    float offsets[kMaxStops];
    RGBf prep[kMaxStops];
};

Z2D_D double clampd(double v, double lo, double hi) { return fmax(lo, fmin(v, hi)); }

// The f64 evaluation (the reference arithmetic).
Z2D_D float grad_offset_f64(const DevGradient &gr, int32_t x, int32_t y) {
    if (gr.type == Z2D_GRADIENT_RADIAL && gr.inner_r == 0.0 && gr.outer_r == 0.0) return -1.0f;
    double px = (double)x + 0.5, py = (double)y + 0.5;
    if (gr.has_tf) {
        const double ix = px, iy = py;
        px = gr.tf[0] * ix + gr.tf[1] * iy;
        py = gr.tf[2] * ix + gr.tf[3] * iy;
        px += gr.tf[4];
        py += gr.tf[5];
    }
    if (gr.type == Z2D_GRADIENT_LINEAR) {
        if (gr.lin_zero) return -1.0f;
        const double spx = px - gr.g[0], spy = py - gr.g[1];
        double d = 0.0;
        d += gr.lin_dx * spx;
        d += gr.lin_dy * spy;
        return (float)clampd(d * gr.lin_inv, 0.0, 1.0);
    }
    if (gr.type == Z2D_GRADIENT_RADIAL) {
        const double pdx = px - gr.g[0], pdy = py - gr.g[1];
        double b = 0.0;
        b += pdx * gr.cdx;
        b += pdy * gr.cdy;
        b += gr.inner_r * gr.dr;
        double c = 0.0;
        c += pdx * pdx;
        c += pdy * pdy;
        c += -gr.inner_r * gr.inner_r;
        if (gr.a == 0.0) {
            if (b == 0.0) return -1.0f;
            const double t = 0.5 * c / b;
            if (t * gr.dr >= gr.min_dr) return (float)clampd(t, 0.0, 1.0);
            return -1.0f;
        }
        double discr = 0.0;
        discr += b * b;
        discr += gr.a * -c;
        if (discr >= 0.0) {
            const double sq = sqrt(discr);
            const double t0 = (b + sq) * gr.inv_a, t1 = (b - sq) * gr.inv_a;
            if (t0 * gr.dr >= gr.min_dr) return (float)clampd(t0, 0.0, 1.0);
            if (t1 * gr.dr >= gr.min_dr) return (float)clampd(t1, 0.0, 1.0);
        }
        return -1.0f;
    }
    const double dx = px - gr.g[0], dy = py - gr.g[1];
    const double twopi = 6.283185307179586;
    const double ang = zmod(zm::atan2_(dy, dx) - gr.angle, twopi);
    return (float)(ang / twopi);
}

// Gradient.getOffset (src/gradient.zig:239-243, 349-372, 605-648, 731-741):
// the double-word evaluation when it decides the f32 result, else the f64
// code above (`slow` is set then).
Z2D_D float grad_offset_ex(const DevGradient &gr, int32_t x, int32_t y, bool &slow) {
    const int32_t mode = gr.fz.mode;
    if (mode == kFastVoid) return -1.0f;
    if (mode != kFastNone && (uint32_t)(x + (1 << 22)) < (1u << 23) && (uint32_t)(y + (1 << 22)) < (1u << 23)) {
        const float fx = (float)x + 0.5f, fy = (float)y + 0.5f;
        const bool tf = gr.has_tf != 0;
        float t = 0.0f;
        int done;
        if (mode == kFastLinear) done = fast_linear(gr.fz, tf, fx, fy, t);
        else if (mode == kFastConic) done = fast_conic(gr.fz, tf, fx, fy, t);
        else done = fast_radial(gr.fz, tf, mode == kFastRadialA0, fx, fy, t);
        if (done) return t;
    }
    slow = true;
    return grad_offset_f64(gr, x, y);
}
// Out of line: the kernels that composite every kind of source (the
// rasteriser among them) keep their registers for their own loops.
static __device__ __noinline__ float grad_offset(const DevGradient &gr, int32_t x, int32_t y) {
    bool slow = false;
    return grad_offset_ex(gr, x, y, slow);
}

struct Search {
    int i0, i1;  // stop indices, -1 for transparent
    float offset;
};
// Stop.List.search (src/gradient.zig:832-897)
Z2D_D Search grad_search(const DevGradient &gr, float offset) {
    const int n = gr.n_stops;
    if (offset < 0.0f || n == 0) return Search{-1, -1, 0.0f};
    const float *const offsets = n > kMaxStops ? gr.ext_off : gr.offsets;
    const float o = fminf(offset, 1.0f);
    int left = 0, right = n, mid = 0;
    while (left < right) {
        mid = left + (right - left) / 2;
        if (o >= offsets[mid] && (mid == n - 1 || o <= offsets[mid + 1])) break;
        if (o < offsets[mid]) {
            right = mid;
            continue;
        }
        if (o > offsets[mid]) {
            left = mid + 1;
            continue;
        }
    }
    if (mid == n - 1) return Search{mid, mid, o - offsets[mid]};
    if (mid == 0 && o < offsets[mid]) return Search{mid, mid, o / offsets[mid]};
    const float st = offsets[mid], en = offsets[mid + 1], rl = en - st;
    return Search{mid, mid + 1, (rl != 0.0f) ? (o - st) / rl : 0.0f};
}
// The prepared colour of stop i; i < 0 is the transparent result of an
// invalid offset, LinearRGB.init(0,0,0,0), which is zero in every space.
Z2D_D RGBf stop_prep(const DevGradient &gr, int i) {
    if (i < 0) return RGBf{0.f, 0.f, 0.f, 0.f};
    return gr.n_stops > kMaxStops ? gr.ext_prep[i] : gr.prep[i];
}

// The first step of the interpolation on a stop's colour (see DevGradient).
Z2D_HD RGBf prepare_stop(int method, const z2d_color &c) {
    if (method == Z2D_INTERP_LINEAR_RGB) {
        const RGBf a = linear_from_color(c);
        return RGBf{a.r * a.a, a.g * a.a, a.b * a.a, a.a};
    }
    if (method == Z2D_INTERP_SRGB) {
        const RGBf a = srgb_from_color(c);
        return RGBf{a.r * a.a, a.g * a.a, a.b * a.a, a.a};
    }
    const HSLf h = hsl_from_color(c);
    return RGBf{h.h, h.s * h.a, h.l * h.a, h.a};
}

// LinearRGB / SRGB interpolate from premultiplied stops: the lerp, then
// demultiply (src/color.zig:356-372).
Z2D_D RGBf rgb_lerp_demul(RGBf am, RGBf bm, float t) {
    const RGBf o{lerpf(am.r, bm.r, t), lerpf(am.g, bm.g, t), lerpf(am.b, bm.b, t), lerpf(am.a, bm.a, t)};
    if (o.a == 0.0f) return RGBf{0.f, 0.f, 0.f, o.a};
    return RGBf{o.r / o.a, o.g / o.a, o.b / o.a, o.a};
}
// HSL.interpolate from premultiplied stops (polar hue handling, then
// demultiply of saturation and lightness).
Z2D_D HSLf hsl_lerp_demul(RGBf am, RGBf bm, float t, int polar) {
    float ah = am.r, bh = bm.r;
    if (polar == Z2D_INTERP_HSL_SHORTER) {
        const bool gt = bh - ah > 180.0f, lt = bh - ah < -180.0f;
        if (gt) ah = ah + 360.0f;
        if (lt) bh = bh + 360.0f;
    } else if (polar == Z2D_INTERP_HSL_LONGER) {
        const float delta = bh - ah;
        const bool c1 = (0.0f < delta) && (delta < 180.0f), c2 = (-180.0f < delta) && (delta <= 0.0f);
        if (c1) ah = ah + 360.0f;
        if (c2) bh = bh + 360.0f;
    } else if (polar == Z2D_INTERP_HSL_INCREASING) {
        if (bh < ah) bh = bh + 360.0f;
    } else {
        if (ah < bh) ah = ah + 360.0f;
    }
    const float h = am.r + (bh - ah) * t;
    const HSLf o{zmodf(h, 360.0f), lerpf(am.g, bm.g, t), lerpf(am.b, bm.b, t), lerpf(am.a, bm.a, t)};
    if (o.a == 0.0f) return HSLf{o.h, 0.0f, 0.0f, o.a};
    return HSLf{o.h, o.s / o.a, o.l / o.a, o.a};
}
// interpolateEncode: the integer lanes of the interpolated colour.
Z2D_D I16 interp_encode_prep(int method, RGBf am, RGBf bm, float t) {
    if (method == Z2D_INTERP_LINEAR_RGB)
        return I16{enc_ch(lerpf(am.r, bm.r, t)), enc_ch(lerpf(am.g, bm.g, t)), enc_ch(lerpf(am.b, bm.b, t)),
                   enc_ch(lerpf(am.a, bm.a, t))};
    if (method == Z2D_INTERP_SRGB) {
        const RGBf d = rgb_lerp_demul(am, bm, t);
        return encode_linear(RGBf{zpow(d.r, kGamma), zpow(d.g, kGamma), zpow(d.b, kGamma), d.a});
    }
    return encode_linear(hsl_to_rgb(hsl_lerp_demul(am, bm, t, method)));
}
// interpolate: the linear colour (float precision, dither sources).
Z2D_D RGBf interp_linear_prep(int method, RGBf am, RGBf bm, float t) {
    if (method == Z2D_INTERP_LINEAR_RGB) return rgb_lerp_demul(am, bm, t);
    if (method == Z2D_INTERP_SRGB) {
        const RGBf d = rgb_lerp_demul(am, bm, t);
        return RGBf{zpow(d.r, kGamma), zpow(d.g, kGamma), zpow(d.b, kGamma), d.a};
    }
    return hsl_to_rgb(hsl_lerp_demul(am, bm, t, method));
}

// -------------------------------------------------------------- dither
// one copy per translation unit, so no relocatable device code is needed.
// Global memory read through the read-only cache, not __constant__: the
// lanes of a warp read 32 different entries, which the constant cache
// would serialise.
static __device__ const uint16_t g_blue_noise[4096] = {
#include "blue_noise_64x64.inc"
};

Z2D_D float bayer(int32_t x, int32_t y) {
    const int32_t yy = y ^ x;
    const uint32_t m = (uint32_t)(((yy & 1) << 5) | ((x & 1) << 4) | ((yy & 2) << 2) | ((x & 2) << 1) | ((yy & 4) >> 1) | ((x & 4) >> 2));
    return (float)m * (2.0f / 128.0f) - (63.0f / 128.0f);
}
Z2D_D float blue_noise(int32_t x, int32_t y) {
    int32_t xm = x % 64, ym = y % 64;
    if (xm < 0) xm += 64;
    if (ym < 0) ym += 64;
    return (float)__ldg(&g_blue_noise[(xm << 6) | ym]) * (2.0f / 8192.0f) - (4095.0f / 8192.0f);
}

// ---------------------------------------------------------- sources
enum : int32_t { SRC_NONE = 0, SRC_PIXEL = 1, SRC_GRADIENT = 2, SRC_DITHER = 3, SRC_SURFACE = 4 };

// A pattern/param prepared for the device.  Pixel sources carry their
// integer and float lanes ready to use.
struct DevSrc {
    int32_t kind;
    int32_t dither_type, dither_source, dither_scale;
    I16 pix;           // RGBA16Vec.fromPixel lanes (PIXEL); RGBA of the dither pixel
    F4 pixf;           // RGBAFloat.Vector.fromPixel lanes
    RGBf dither_base;  // linear color of a PIXEL/COLOR dither source
    Px px;             // the pixel in its own format (fast paths)
    DevSurface sfc;    // SURFACE
    const DevGradient *grad;
    int32_t grad_type, grad_method;  // the gradient's kind and method, for choosing a kernel on the host
};

Z2D_D RGBf dither_linear(const DevSrc &s, int32_t x, int32_t y) {
    RGBf c;
    if (s.dither_source == Z2D_DITHER_SRC_GRADIENT) {
        const Search r = grad_search(*s.grad, grad_offset(*s.grad, x, y));
        c = interp_linear_prep(s.grad->method, stop_prep(*s.grad, r.i0), stop_prep(*s.grad, r.i1), r.offset);
    } else {
        c = s.dither_base;
    }
    float m;
    if (s.dither_type == Z2D_DITHER_BAYER) m = bayer(x, y);
    else if (s.dither_type == Z2D_DITHER_BLUE_NOISE) m = blue_noise(x, y);
    else return c;
    const float scale = 1.0f / (float)((1 << s.dither_scale) - 1);
    return RGBf{fmaxf(0.0f, fminf(c.r + m * scale, 1.0f)), fmaxf(0.0f, fminf(c.g + m * scale, 1.0f)),
                fmaxf(0.0f, fminf(c.b + m * scale, 1.0f)), fmaxf(0.0f, fminf(c.a + m * scale, 1.0f))};
}

// Source lanes at device position (x, y); `idx` is the flat index used for
// SURFACE params.
Z2D_D I16 src_i16(const DevSrc &s, int32_t x, int32_t y, size_t idx) {
    switch (s.kind) {
        case SRC_PIXEL: return s.pix;
        case SRC_GRADIENT: {
            const Search r = grad_search(*s.grad, grad_offset(*s.grad, x, y));
            return interp_encode_prep(s.grad->method, stop_prep(*s.grad, r.i0), stop_prep(*s.grad, r.i1), r.offset);
        }
        case SRC_DITHER: return encode_linear(dither_linear(s, x, y));
        case SRC_SURFACE: return load_px(s.sfc, idx);
        default: return I16{0, 0, 0, 0};
    }
}
Z2D_D F4 src_f4(const DevSrc &s, int32_t x, int32_t y, size_t idx) {
    switch (s.kind) {
        case SRC_PIXEL: return s.pixf;
        case SRC_GRADIENT: {
            const Search r = grad_search(*s.grad, grad_offset(*s.grad, x, y));
            const RGBf c = interp_linear_prep(s.grad->method, stop_prep(*s.grad, r.i0), stop_prep(*s.grad, r.i1), r.offset);
            return F4{c.r, c.g, c.b, c.a};
        }
        case SRC_DITHER: {
            const RGBf c = dither_linear(s, x, y);
            return F4{c.r, c.g, c.b, c.a};
        }
        case SRC_SURFACE: return decode_raw(load_px(s.sfc, idx));
        default: return F4{0.f, 0.f, 0.f, 0.f};
    }
}

}  // namespace z2dg

namespace z2dg {
// Out-of-line entry points for the heavy per-pixel paths, so that kernels
// instantiated per format and precision do not each inline every source
// and operator (keeps code size and build time small).
static __device__ __noinline__ I16 src_i16_any(const DevSrc &s, int32_t x, int32_t y, size_t idx) { return src_i16(s, x, y, idx); }
static __device__ __noinline__ F4 src_f4_any(const DevSrc &s, int32_t x, int32_t y, size_t idx) { return src_f4(s, x, y, idx); }
static __device__ __noinline__ I16 int_op_any(int op, I16 d, I16 s) { return int_op(op, d, s); }
static __device__ __noinline__ F4 float_op_any(int op, F4 d, F4 s) { return float_op(op, d, s); }

// Source lanes with the pixel case inline.
__device__ __forceinline__ I16 src_i16_fast(const DevSrc &s, int32_t x, int32_t y, size_t idx) {
    if (s.kind == SRC_PIXEL) return s.pix;
    return src_i16_any(s, x, y, idx);
}
__device__ __forceinline__ F4 src_f4_fast(const DevSrc &s, int32_t x, int32_t y, size_t idx) {
    if (s.kind == SRC_PIXEL) return s.pixf;
    return src_f4_any(s, x, y, idx);
}
}  // namespace z2dg
