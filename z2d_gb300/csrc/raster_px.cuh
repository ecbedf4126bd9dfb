// raster_px.cuh -- one pixel of a fill or hairline composited onto a
// surface, and raw pixel access, shared by the rasteriser (fill.cu) and the
// hairline rasteriser (hairline.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fill.cuh"

namespace z2dg {

__device__ __forceinline__ I16 normalize(I16 v, int fmt) { return to_i16(from_i16(v, fmt)); }

// compositeOpacity (raster/shared.zig:50-104) of one pixel: the source
// (the pattern pixel through Surface.compositeStride when the operator
// reduces to it) taken through dst_in with `opacity`, then the operator.
static __device__ __forceinline__ I16 apply_opacity(const FillCmd &F, int fmt, int32_t x, int32_t y, uint32_t opacity,
                                                    I16 d) {
    if (F.op == Z2D_OP_CLEAR) return normalize(I16{0, 0, 0, 0}, fmt);
    if (F.reduces) {
        I16 s = F.px_rgba;
        if (opacity < 255) s = normalize(int_op(Z2D_OP_DST_IN, s, I16{0, 0, 0, opacity}), Z2D_FORMAT_RGBA);
        return normalize(int_op_any(F.op, d, s), fmt);
    }
    if (F.precision == Z2D_PRECISION_INTEGER) {
        const I16 r = int_op(Z2D_OP_DST_IN, src_i16_fast(F.src, x, y, 0), I16{0, 0, 0, opacity});
        return normalize(int_op_any(F.op, d, r), fmt);
    }
    const F4 r = float_op(Z2D_OP_DST_IN, src_f4_fast(F.src, x, y, 0), F4{0.f, 0.f, 0.f, (float)opacity / 255.0f});
    return normalize(encode_raw(float_op_any(F.op, decode_raw(d), r)), fmt);
}

// One pixel of a fill with coverage `cov` (1..full) on destination lanes d,
// following compositeOpaque / compositeOpacity (raster/shared.zig:9-104),
// Surface.paintStride and Surface.compositeStride (surface.zig:537-581).
// Out of line: every operator, precision and source kind is reachable from
// here, which keeps the rasteriser's hot loop small.
static __device__ __noinline__ I16 apply_fill(const FillCmd &F, int fmt, int32_t x, int32_t y, int cov, int full, I16 d) {
    if (F.op == Z2D_OP_CLEAR) return normalize(I16{0, 0, 0, 0}, fmt);
    if (cov >= full) {
        if (F.reduces) return to_i16(F.px_paint);
        if (F.precision == Z2D_PRECISION_INTEGER) return normalize(int_op_any(F.op, d, src_i16_fast(F.src, x, y, 0)), fmt);
        return normalize(encode_raw(float_op_any(F.op, decode_raw(d), src_f4_fast(F.src, x, y, 0))), fmt);
    }
    return apply_opacity(F, fmt, x, y, (uint32_t)min(max(cov * 16 - 1, 0), 255), d);
}

__device__ __forceinline__ I16 raw_to_i16(uint32_t raw, int fmt) {
    if (fmt <= Z2D_FORMAT_RGBA) return word_to_i16(raw, fmt);
    return I16{0, 0, 0, scale_alpha(raw, fmt_bits(fmt), 8)};
}
__device__ __forceinline__ uint32_t i16_to_raw(I16 v, int fmt) {
    if (fmt <= Z2D_FORMAT_RGBA) return i16_to_word(v, fmt);
    return scale_alpha(v.a & 0xFFu, 8, fmt_bits(fmt));
}
__device__ __forceinline__ uint32_t load_raw(const DevSurface &s, size_t i) {
    if (s.fmt <= Z2D_FORMAT_RGBA) return reinterpret_cast<const uint32_t *>(s.data)[i];
    if (s.fmt == Z2D_FORMAT_ALPHA8) return s.data[i];
    const int bits = fmt_bits(s.fmt);
    const size_t bit = i * (size_t)bits;
    return (s.data[bit >> 3] >> (bit & 7)) & ((1u << bits) - 1u);
}
__device__ __forceinline__ void store_raw(const DevSurface &s, size_t i, uint32_t v) {
    if (s.fmt <= Z2D_FORMAT_RGBA) reinterpret_cast<uint32_t *>(s.data)[i] = v;
    else if (s.fmt == Z2D_FORMAT_ALPHA8) s.data[i] = (uint8_t)v;
    else store_raw_packed(s, i, v);
}

}  // namespace z2dg
