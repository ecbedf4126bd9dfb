// composite.cu -- SurfaceCompositor.run on the GPU.
//
// Replaces z2d's per-row stride loop (src/compositor.zig:302-440, 540-621)
// with one launch over the whole destination region.  Two kernels:
//  * k_composite_flat: the region is the whole destination and every
//    surface parameter has the destination's width, so pixel i of the
//    destination pairs with pixel i of each parameter.  Each thread owns 16
//    bytes of destination (4 RGBA px, 16 alpha8 px, 32/64/128 packed px),
//    loaded and stored as one 16-byte vector; HBM bound.
//  * k_composite_region: any other region; one thread per destination
//    pixel (byte formats) or per destination byte (packed formats, so that
//    no two threads share a byte).
// Both evaluate the batch per pixel exactly like runPrecision's lanes.
#include <cuda_runtime.h>

#include "z2d_internal.h"

namespace z2dg {

// One pixel through the batch.  (x, y) are destination coordinates;
// flat indices of surface params are derived from them.
template <int PREC>
__device__ __forceinline__ I16 run_batch(const CompJob &J, int32_t x, int32_t y, I16 dpx) {
    if (PREC == Z2D_PRECISION_INTEGER) {
        I16 d = dpx, s = dpx;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            if (k >= J.n_ops) break;
            const CompOp &o = J.ops[k];
            if (o.src.kind == SRC_NONE) {
                s = d;
            } else {
                const size_t si = (size_t)o.src.sfc.w * (size_t)(y - J.dst_y) + (size_t)(x - J.dst_x);
                s = src_i16_fast(o.src, x, y, si);
            }
            if (o.dst.kind == SRC_NONE) {
                d = dpx;
            } else {
                const size_t di = (size_t)o.dst.sfc.w * (size_t)y + (size_t)x;
                d = src_i16_fast(o.dst, x, y, di);
            }
            d = int_op_any(o.op, d, s);
        }
        return d;
    } else {
        const F4 dpf = decode_raw(dpx);
        F4 d = dpf, s = dpf;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            if (k >= J.n_ops) break;
            const CompOp &o = J.ops[k];
            if (o.src.kind == SRC_NONE) {
                s = d;
            } else {
                const size_t si = (size_t)o.src.sfc.w * (size_t)(y - J.dst_y) + (size_t)(x - J.dst_x);
                s = src_f4_fast(o.src, x, y, si);
            }
            if (o.dst.kind == SRC_NONE) {
                d = dpf;
            } else {
                const size_t di = (size_t)o.dst.sfc.w * (size_t)y + (size_t)x;
                d = src_f4_fast(o.dst, x, y, di);
            }
            d = float_op_any(o.op, d, s);
        }
        return encode_raw(d);
    }
}

// Rows whose surface params do not cover the row are skipped (a shorter
// stride is undefined behaviour in z2d).
__device__ __forceinline__ bool row_ok(const CompJob &J, int32_t y) {
    for (int k = 0; k < J.n_ops; k++) {
        const CompOp &o = J.ops[k];
        if (o.dst.kind == SRC_SURFACE && (y >= o.dst.sfc.h || J.dsx >= o.dst.sfc.w)) return false;
        if (o.src.kind == SRC_SURFACE && (y - J.dst_y >= o.src.sfc.h || J.dsx - J.dst_x >= o.src.sfc.w)) return false;
    }
    return true;
}

// ---------------------------------------------------------------- flat
template <int FMT, int PREC>
__global__ void __launch_bounds__(256) k_composite_flat(const CompJob J, size_t n_chunks) {
    const int32_t W = J.dst.w;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n_chunks; c += (size_t)gridDim.x * blockDim.x) {
        uint4 *p = reinterpret_cast<uint4 *>(J.dst.data) + c;
        uint4 v = *p;
        uint32_t w[4] = {v.x, v.y, v.z, v.w};
        if constexpr (FMT <= Z2D_FORMAT_RGBA) {
            const size_t i0 = c * 4;
            // (x, y) of the chunk's first pixel, then stepped along the rows
            int32_t y = (int32_t)(i0 / (size_t)W), x = (int32_t)(i0 - (size_t)y * W);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                w[j] = i16_to_word(run_batch<PREC>(J, x, y, word_to_i16(w[j], FMT)), FMT);
                if (++x == W) {
                    x = 0;
                    y++;
                }
            }
        } else {
            constexpr int BITS = FMT == Z2D_FORMAT_ALPHA8 ? 8 : FMT == Z2D_FORMAT_ALPHA4 ? 4 : FMT == Z2D_FORMAT_ALPHA2 ? 2 : 1;
            constexpr int PER_WORD = 32 / BITS;
            constexpr uint32_t MASK = (1u << BITS) - 1u;
            const size_t i0 = c * 4 * PER_WORD;
            const size_t total = (size_t)W * (size_t)J.dst.h;
            int32_t y = (int32_t)(i0 / (size_t)W), x = (int32_t)(i0 - (size_t)y * W);
#pragma unroll 1
            for (int j = 0; j < 4; j++) {
                uint32_t out = w[j];
#pragma unroll 1
                for (int k = 0; k < PER_WORD; k++) {
                    const size_t i = i0 + (size_t)j * PER_WORD + k;
                    if (i >= total) break;
                    const int32_t px = x, py = y;
                    if (++x == W) {
                        x = 0;
                        y++;
                    }
                    const uint32_t raw = (w[j] >> (k * BITS)) & MASK;
                    const I16 r = run_batch<PREC>(J, px, py, I16{0, 0, 0, scale_alpha(raw, BITS, 8)});
                    const uint32_t nv = scale_alpha(r.a & 0xFFu, 8, BITS);
                    out = (out & ~(MASK << (k * BITS))) | (nv << (k * BITS));
                }
                w[j] = out;
            }
        }
        *p = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// -------------------------------------------------------------- region
template <int FMT, int PREC>
__global__ void __launch_bounds__(256) k_composite_region(const CompJob J, size_t n_units) {
    const int32_t W = J.dst.w;
    constexpr int BITS = FMT <= Z2D_FORMAT_RGBA ? 32 : FMT == Z2D_FORMAT_ALPHA8 ? 8 : FMT == Z2D_FORMAT_ALPHA4 ? 4 : FMT == Z2D_FORMAT_ALPHA2 ? 2 : 1;
    for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < n_units; u += (size_t)gridDim.x * blockDim.x) {
        if constexpr (BITS >= 8) {
            const int32_t row = (int32_t)(u / (size_t)J.line_w);
            const int32_t x = J.dsx + (int32_t)(u - (size_t)row * J.line_w);
            const int32_t y = J.y0 + row;
            if (!row_ok(J, y)) continue;
            const size_t i = (size_t)W * y + x;
            const I16 d = load_px(J.dst, i);
            store_px(J.dst, i, run_batch<PREC>(J, x, y, d));
        } else {
            // unit = one byte of the destination between the first and last
            // region pixel
            constexpr int PER = 8 / BITS;
            const size_t first = (size_t)W * J.y0 + J.dsx;
            const size_t byte = first / PER + u;
            uint32_t out = J.dst.data[byte];
            bool changed = false;
#pragma unroll 1
            for (int k = 0; k < PER; k++) {
                const size_t i = byte * PER + k;
                const int32_t y = (int32_t)(i / (size_t)W), x = (int32_t)(i - (size_t)y * W);
                if (y < J.y0 || y >= J.y1 || x < J.dsx || x >= J.dsx + J.line_w) continue;
                if (!row_ok(J, y)) continue;
                const uint32_t raw = (out >> (k * BITS)) & ((1u << BITS) - 1u);
                const I16 r = run_batch<PREC>(J, x, y, I16{0, 0, 0, scale_alpha(raw, BITS, 8)});
                const uint32_t nv = scale_alpha(r.a & 0xFFu, 8, BITS);
                out = (out & ~(((1u << BITS) - 1u) << (k * BITS))) | (nv << (k * BITS));
                changed = true;
            }
            if (changed) J.dst.data[byte] = (uint8_t)out;
        }
    }
}

template <int FMT, int PREC>
static void launch_one(Ctx &c, const CompJob &J, bool flat) {
    const int threads = 256;
    if (flat) {
        const size_t bytes = ((size_t)J.dst.w * J.dst.h * fmt_bits(FMT) + 7) / 8;
        const size_t n_chunks = bytes / 16;  // the caller guarantees a multiple of 16
        size_t blocks = (n_chunks + threads - 1) / threads;
        const size_t cap = (size_t)c.sm_count * 8;
        if (blocks > cap) blocks = cap;
        if (blocks == 0) return;
        k_composite_flat<FMT, PREC><<<(unsigned)blocks, threads, 0, c.stream>>>(J, n_chunks);
    } else {
        size_t n_units;
        if (fmt_bits(FMT) >= 8) {
            n_units = (size_t)(J.y1 - J.y0) * (size_t)J.line_w;
        } else {
            const int per = 8 / fmt_bits(FMT);
            const size_t first = (size_t)J.dst.w * J.y0 + J.dsx;
            const size_t last = (size_t)J.dst.w * (J.y1 - 1) + J.dsx + J.line_w - 1;
            n_units = last / per - first / per + 1;
        }
        size_t blocks = (n_units + threads - 1) / threads;
        const size_t cap = (size_t)c.sm_count * 16;
        if (blocks > cap) blocks = cap;
        if (blocks == 0) return;
        k_composite_region<FMT, PREC><<<(unsigned)blocks, threads, 0, c.stream>>>(J, n_units);
    }
    c.launches++;
}

template <int PREC>
static void launch_fmt(Ctx &c, const CompJob &J, bool flat) {
    switch (J.dst.fmt) {
        case Z2D_FORMAT_ARGB: launch_one<Z2D_FORMAT_ARGB, PREC>(c, J, flat); break;
        case Z2D_FORMAT_XRGB: launch_one<Z2D_FORMAT_XRGB, PREC>(c, J, flat); break;
        case Z2D_FORMAT_RGB: launch_one<Z2D_FORMAT_RGB, PREC>(c, J, flat); break;
        case Z2D_FORMAT_RGBA: launch_one<Z2D_FORMAT_RGBA, PREC>(c, J, flat); break;
        case Z2D_FORMAT_ALPHA8: launch_one<Z2D_FORMAT_ALPHA8, PREC>(c, J, flat); break;
        case Z2D_FORMAT_ALPHA4: launch_one<Z2D_FORMAT_ALPHA4, PREC>(c, J, flat); break;
        case Z2D_FORMAT_ALPHA2: launch_one<Z2D_FORMAT_ALPHA2, PREC>(c, J, flat); break;
        default: launch_one<Z2D_FORMAT_ALPHA1, PREC>(c, J, flat); break;
    }
}

int launch_composite(Ctx &c, const CompJob &J) {
    if (J.y1 <= J.y0 || J.line_w <= 0) return Z2D_OK;
    // The flat kernel applies when the region is the whole surface, the
    // surface is a whole number of 16-byte chunks and every surface param
    // has the destination's geometry.
    bool flat = J.dst_x == 0 && J.dst_y == 0 && J.dsx == 0 && J.y0 == 0 && J.y1 == J.dst.h && J.line_w == J.dst.w;
    const size_t bytes = ((size_t)J.dst.w * J.dst.h * fmt_bits(J.dst.fmt) + 7) / 8;
    if (bytes % 16 != 0 || (reinterpret_cast<uintptr_t>(J.dst.data) & 15) != 0) flat = false;
    for (int k = 0; k < J.n_ops && flat; k++) {
        const CompOp &o = J.ops[k];
        if (o.dst.kind == SRC_SURFACE && (o.dst.sfc.w != J.dst.w || o.dst.sfc.h < J.dst.h)) flat = false;
        if (o.src.kind == SRC_SURFACE && (o.src.sfc.w != J.dst.w || o.src.sfc.h < J.dst.h)) flat = false;
    }
    cudaEvent_t t0 = c.timer_begin(c.t_composite);
    if (try_mask_batch(c, J, flat) || try_mask_grad(c, J, flat)) {
    } else if (J.precision == Z2D_PRECISION_FLOAT) {
        launch_fmt<Z2D_PRECISION_FLOAT>(c, J, flat);
    } else {
        launch_fmt<Z2D_PRECISION_INTEGER>(c, J, flat);
    }
    c.timer_end(c.t_composite, t0);
    Z2D_CUDA(cudaGetLastError());
    return Z2D_OK;
}

}  // namespace z2dg
