// composite_grad.cu -- the compositor's mask batch with a gradient source.
//
// supersample.zig:171-184 / SurfaceCompositor.run (compositor.zig:302-440)
// with the batch [dst_in(dst = gradient or dithered gradient, src = alpha8
// mask), op] over a whole 4-byte-format surface, integer precision.  The
// generic composite kernel evaluates such a pixel through out-of-line
// calls and run-time dispatch on every level (source kind, gradient kind,
// interpolation method, operator); here the gradient kind, the
// interpolation space and the presence of a dither are template parameters
// and everything is inlined, so a pixel is the offset (grad_fast.cuh, f64
// only where its rounding is undecided), the stop search, the
// interpolation and the two operators.  Each thread owns 16-byte chunks of
// destination (4 pixels) and the matching 4 mask bytes; pixel coordinates
// advance with the grid stride instead of being divided out per chunk.
#include <cuda_runtime.h>

#include <atomic>

#include "z2d_internal.h"

namespace z2dg {

namespace {

constexpr int kGradThreads = 256;

enum : int { kLinRGB = 0, kSRGB = 1, kHSL = 2 };

// Out of line: the f64 offsets (taken for a pixel in thousands) and
// std.math.pow (three per sRGB pixel), so that each instantiation's loop
// stays small enough for the instruction cache.
__device__ __noinline__ float offset_f64_call(const DevGradient &g, int32_t x, int32_t y) {
    return grad_offset_f64(g, x, y);
}
__device__ __noinline__ float gamma_call(float x) { return zpow(x, kGamma); }

template <int KIND>
__device__ __forceinline__ float offset_inline(const DevGradient &g, int32_t x, int32_t y) {
    // the kind is known here, so only its evaluation is compiled in
    if ((uint32_t)(x + (1 << 22)) < (1u << 23) && (uint32_t)(y + (1 << 22)) < (1u << 23)) {
        const int32_t mode = g.fz.mode;
        if (mode == kFastVoid) return -1.0f;
        if (mode != kFastNone) {
            const float fx = (float)x + 0.5f, fy = (float)y + 0.5f;
            const bool tf = g.has_tf != 0;
            float t = 0.0f;
            int done;
            if constexpr (KIND == Z2D_GRADIENT_LINEAR) done = fast_linear(g.fz, tf, fx, fy, t);
            else if constexpr (KIND == Z2D_GRADIENT_CONIC) done = fast_conic(g.fz, tf, fx, fy, t);
            else done = fast_radial(g.fz, tf, mode == kFastRadialA0, fx, fy, t);
            if (done) return t;
        }
    }
    return offset_f64_call(g, x, y);
}

// The linear offset inline; the radial and conic evaluations (several
// times its code) out of line, one copy per kind.
template <int KIND>
__device__ __noinline__ float offset_call(const DevGradient &g, int32_t x, int32_t y) {
    return offset_inline<KIND>(g, x, y);
}
template <int KIND>
__device__ __forceinline__ float offset_of(const DevGradient &g, int32_t x, int32_t y) {
    if constexpr (KIND == Z2D_GRADIENT_LINEAR) return offset_inline<KIND>(g, x, y);
    else return offset_call<KIND>(g, x, y);
}
// HSL.interpolate + toLinearRGB, out of line (fmod and the hue cases)
__device__ __noinline__ RGBf hsl_call(RGBf a, RGBf b, float t, int method) {
    return hsl_to_rgb(hsl_lerp_demul(a, b, t, method));
}

// The source's colour lanes at (x, y): interpolateEncode, or the dithered
// linear colour encoded (Dither.getPixel)
template <int KIND, int METHOD, bool DITH>
__device__ __forceinline__ I16 grad_lanes(const DevSrc &s, const DevGradient &g, int32_t x, int32_t y) {
    const Search r = grad_search(g, offset_of<KIND>(g, x, y));
    const RGBf a = stop_prep(g, r.i0), b = stop_prep(g, r.i1);
    // (SRGB.interpolate then toLinearRGB, as interp_encode_prep /
    // interp_linear_prep do, with the gamma out of line)
    if constexpr (!DITH) {
        if constexpr (METHOD == kLinRGB) {
            return interp_encode_prep(Z2D_INTERP_LINEAR_RGB, a, b, r.offset);
        } else if constexpr (METHOD == kSRGB) {
            const RGBf d = rgb_lerp_demul(a, b, r.offset);
            return encode_linear(RGBf{gamma_call(d.r), gamma_call(d.g), gamma_call(d.b), d.a});
        } else {
            return encode_linear(hsl_call(a, b, r.offset, g.method));
        }
    } else {
        RGBf c;
        if constexpr (METHOD == kLinRGB) {
            c = rgb_lerp_demul(a, b, r.offset);
        } else if constexpr (METHOD == kSRGB) {
            const RGBf d = rgb_lerp_demul(a, b, r.offset);
            c = RGBf{gamma_call(d.r), gamma_call(d.g), gamma_call(d.b), d.a};
        } else {
            c = hsl_call(a, b, r.offset, g.method);
        }
        const float m = s.dither_type == Z2D_DITHER_BAYER ? bayer(x, y) : blue_noise(x, y);
        const float scale = 1.0f / (float)((1 << s.dither_scale) - 1);
        return encode_linear(RGBf{fmaxf(0.0f, fminf(c.r + m * scale, 1.0f)), fmaxf(0.0f, fminf(c.g + m * scale, 1.0f)),
                                  fmaxf(0.0f, fminf(c.b + m * scale, 1.0f)), fmaxf(0.0f, fminf(c.a + m * scale, 1.0f))});
    }
}

template <int KIND, int METHOD, bool DITH>
__global__ void __launch_bounds__(kGradThreads) k_mask_grad(uint8_t *__restrict__ dst, const uint8_t *__restrict__ mask,
                                                           int32_t W, size_t n_chunks, int32_t fmt, int32_t op,
                                                           const DevSrc src) {
    const DevGradient &g = *src.grad;
    const size_t first = (size_t)blockIdx.x * kGradThreads + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * kGradThreads;
    // (x, y) of the first pixel of this thread's first chunk, then advanced
    // by the stride (4 * stride pixels: q rows and r columns)
    const size_t p0 = first * 4, sp = stride * 4;
    int32_t y = (int32_t)(p0 / (size_t)W), x = (int32_t)(p0 - (size_t)y * W);
    const int32_t q = (int32_t)(sp / (size_t)W), rr = (int32_t)(sp - (size_t)q * W);
    for (size_t c = first; c < n_chunks; c += stride) {
        uint4 v = reinterpret_cast<const uint4 *>(dst)[c];
        const uint32_t mw = __ldcs(reinterpret_cast<const uint32_t *>(mask) + c);
        uint32_t w[4] = {v.x, v.y, v.z, v.w};
        int32_t px = x, py = y;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const I16 sl = grad_lanes<KIND, METHOD, DITH>(src, g, px, py);
            // IntegerOps.dstIn(d = source, s = mask), then the operator
            const I16 rl = int_op(Z2D_OP_DST_IN, sl, I16{0u, 0u, 0u, (mw >> (8 * j)) & 0xFFu});
            w[j] = i16_to_word(int_op_any(op, word_to_i16(w[j], fmt), rl), fmt);
            if (++px == W) {
                px = 0;
                py++;
            }
        }
        reinterpret_cast<uint4 *>(dst)[c] = make_uint4(w[0], w[1], w[2], w[3]);
        x += rr;
        y += q;
        if (x >= W) {
            x -= W;
            y++;
        }
    }
}

using GradKernel = void (*)(uint8_t *, const uint8_t *, int32_t, size_t, int32_t, int32_t, const DevSrc);

template <int KIND>
GradKernel pick_method(int method, bool dith) {
    if (method == Z2D_INTERP_LINEAR_RGB) return dith ? k_mask_grad<KIND, kLinRGB, true> : k_mask_grad<KIND, kLinRGB, false>;
    if (method == Z2D_INTERP_SRGB) return dith ? k_mask_grad<KIND, kSRGB, true> : k_mask_grad<KIND, kSRGB, false>;
    return dith ? k_mask_grad<KIND, kHSL, true> : k_mask_grad<KIND, kHSL, false>;
}

// Resident blocks per SM of each instantiation (3 kinds x 3 methods x
// dither or not), looked up once: the grid is sized to what fits at once,
// so that no block of the grid-stride loop waits for a second wave.
std::atomic<int> g_grad_occ[3][3][2];

}  // namespace

// The batch [dst_in(gradient source, alpha8 mask), op] on a whole 4-byte
// surface in integer precision; false when J has another shape.
bool try_mask_grad(Ctx &c, const CompJob &J, bool flat) {
    if (!flat || J.n_ops != 2 || J.precision != Z2D_PRECISION_INTEGER) return false;
    const CompOp &o0 = J.ops[0], &o1 = J.ops[1];
    if (o0.op != Z2D_OP_DST_IN || o0.src.kind != SRC_SURFACE || o1.dst.kind != SRC_NONE || o1.src.kind != SRC_NONE)
        return false;
    const DevSrc &s = o0.dst;
    bool dith = false;
    if (s.kind == SRC_DITHER) {
        if (s.dither_source != Z2D_DITHER_SRC_GRADIENT ||
            (s.dither_type != Z2D_DITHER_BAYER && s.dither_type != Z2D_DITHER_BLUE_NOISE))
            return false;
        dith = true;
    } else if (s.kind != SRC_GRADIENT) {
        return false;
    }
    if (!s.grad || J.dst.fmt > Z2D_FORMAT_RGBA || o1.op < 0 || o1.op >= Z2D_OP_COUNT) return false;
    if (o0.src.sfc.fmt != Z2D_FORMAT_ALPHA8 || o0.src.sfc.w != J.dst.w || o0.src.sfc.h < J.dst.h) return false;
    if ((reinterpret_cast<uintptr_t>(o0.src.sfc.data) & 3) != 0 || (reinterpret_cast<uintptr_t>(J.dst.data) & 15) != 0)
        return false;
    const size_t px = (size_t)J.dst.w * J.dst.h;
    if (px % 4 != 0) return false;
    const int kind = s.grad_type, method = s.grad_method;
    if (kind < Z2D_GRADIENT_LINEAR || kind > Z2D_GRADIENT_CONIC) return false;
    GradKernel k = kind == Z2D_GRADIENT_LINEAR   ? pick_method<Z2D_GRADIENT_LINEAR>(method, dith)
                   : kind == Z2D_GRADIENT_RADIAL ? pick_method<Z2D_GRADIENT_RADIAL>(method, dith)
                                                 : pick_method<Z2D_GRADIENT_CONIC>(method, dith);
    const int mslot = method == Z2D_INTERP_LINEAR_RGB ? 0 : method == Z2D_INTERP_SRGB ? 1 : 2;
    std::atomic<int> &slot = g_grad_occ[kind - Z2D_GRADIENT_LINEAR][mslot][dith ? 1 : 0];
    int occ = slot.load(std::memory_order_relaxed);
    if (occ <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kGradThreads, 0) != cudaSuccess || occ <= 0) occ = 1;
        slot.store(occ, std::memory_order_relaxed);
    }
    const size_t n_chunks = px / 4;
    size_t blocks = (n_chunks + kGradThreads - 1) / kGradThreads;
    const size_t cap = (size_t)c.sm_count * (size_t)occ;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) return true;
    k<<<(unsigned)blocks, kGradThreads, 0, c.stream>>>(J.dst.data, o0.src.sfc.data, J.dst.w, n_chunks, J.dst.fmt, o1.op,
                                                      s);
    c.launches++;
    return true;
}

}  // namespace z2dg
