// composite_mask.cu -- the mask batch of SurfaceCompositor.run.
//
// The batch [dst_in(dst = pixel source, src = alpha8 mask), op] over a
// whole surface is how z2d's painter composites a coverage mask onto its
// target (supersample.zig:171-184, compositor.zig:302-440).  Per pixel:
// r = pixel * mask / 255 (IntegerOps.dstIn), d = op(d, r).
//
// HBM bound: 4 B read + 4 B written + 1 B of mask per RGBA pixel.  Each
// thread issues kMaskUnroll independent 16-byte destination loads (and the
// matching mask loads) before it computes, so that enough bytes are in
// flight per SM to cover DRAM latency; the operator is a template
// parameter, so every kernel holds one operator's arithmetic and nothing
// else; dst_in(pixel, mask) comes from a 256-entry shared-memory table, and
// src_over on the 4-byte formats works on two channels per 32-bit word.
// The grid is sized from the kernel's occupancy on this device.
#include <cuda_runtime.h>

#include <atomic>
#include <utility>

#include "z2d_internal.h"

namespace z2dg {

constexpr int kMaskThreads = 256;
constexpr int kMaskUnroll = 4;  // 16-byte chunks in flight per thread

template <int FMT, int OP>
__global__ void __launch_bounds__(kMaskThreads) k_mask_op(uint8_t *__restrict__ dst, const uint8_t *__restrict__ mask,
                                                         size_t n_chunks, I16 spx) {
    constexpr bool WIDE = FMT <= Z2D_FORMAT_RGBA;  // 4 px per chunk; else 16 one-byte px
    constexpr bool HAS_ALPHA = FMT == Z2D_FORMAT_RGBA || FMT == Z2D_FORMAT_ARGB;
    constexpr int ORDER = (FMT == Z2D_FORMAT_ARGB || FMT == Z2D_FORMAT_XRGB) ? Z2D_FORMAT_ARGB : Z2D_FORMAT_RGBA;
    // r = dst_in(pixel, mask) depends on the mask byte only: one table entry
    // per mask value, in the destination's byte order (alpha in byte 3).
    __shared__ uint32_t lut[256];
    for (int i = threadIdx.x; i < 256; i += kMaskThreads) {
        const uint32_t m = (uint32_t)i;
        const I16 r{(spx.r * m) / 255u, (spx.g * m) / 255u, (spx.b * m) / 255u, (spx.a * m) / 255u};
        lut[i] = WIDE ? i16_to_word(r, ORDER) : r.a;
    }
    __syncthreads();
    const size_t tile = (size_t)kMaskThreads * kMaskUnroll;
    for (size_t base = (size_t)blockIdx.x * tile + threadIdx.x; base < n_chunks; base += (size_t)gridDim.x * tile) {
        uint4 v[kMaskUnroll];
        uint4 mv[kMaskUnroll];
#pragma unroll
        for (int k = 0; k < kMaskUnroll; k++) {
            const size_t c = base + (size_t)k * kMaskThreads;
            v[k] = make_uint4(0, 0, 0, 0);
            mv[k] = make_uint4(0, 0, 0, 0);
            if (c < n_chunks) {
                v[k] = reinterpret_cast<const uint4 *>(dst)[c];
                if constexpr (WIDE) mv[k].x = __ldcs(reinterpret_cast<const uint32_t *>(mask) + c);
                else mv[k] = __ldcs(reinterpret_cast<const uint4 *>(mask) + c);
            }
        }
#pragma unroll
        for (int k = 0; k < kMaskUnroll; k++) {
            const size_t c = base + (size_t)k * kMaskThreads;
            if (c >= n_chunks) break;
            uint32_t w[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
            if constexpr (WIDE && OP == Z2D_OP_SRC_OVER) {
                const uint32_t m4 = mv[k].x;
#pragma unroll
                for (int j = 0; j < 4; j++) w[j] = word_src_over(w[j], lut[(m4 >> (8 * j)) & 0xFFu], HAS_ALPHA);
            } else if constexpr (WIDE) {
                const uint32_t m4 = mv[k].x;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const I16 r = word_to_i16(lut[(m4 >> (8 * j)) & 0xFFu], ORDER);
                    w[j] = i16_to_word(int_op(OP, word_to_i16(w[j], FMT), r), FMT);
                }
            } else {
                const uint32_t mw[4] = {mv[k].x, mv[k].y, mv[k].z, mv[k].w};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    uint32_t out = 0;
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        const uint32_t da = (w[j] >> (8 * b)) & 0xFFu;
                        const I16 r{0u, 0u, 0u, lut[(mw[j] >> (8 * b)) & 0xFFu]};
                        out |= (int_op(OP, I16{0u, 0u, 0u, da}, r).a & 0xFFu) << (8 * b);
                    }
                    w[j] = out;
                }
            }
            reinterpret_cast<uint4 *>(dst)[c] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

using MaskKernel = void (*)(uint8_t *, const uint8_t *, size_t, I16);

template <int FMT, int... OPS>
static const MaskKernel *mask_table(std::integer_sequence<int, OPS...>) {
    static const MaskKernel table[] = {&k_mask_op<FMT, OPS>...};
    return table;
}

template <int FMT>
static MaskKernel mask_kernel(int op) {
    return mask_table<FMT>(std::make_integer_sequence<int, Z2D_OP_COUNT>{})[op];
}

// Resident blocks per SM of each kernel, looked up once.
static std::atomic<int> g_mask_occ[5][Z2D_OP_COUNT];

static int fmt_slot(int fmt) {
    switch (fmt) {
        case Z2D_FORMAT_ARGB: return 0;
        case Z2D_FORMAT_XRGB: return 1;
        case Z2D_FORMAT_RGB: return 2;
        case Z2D_FORMAT_RGBA: return 3;
        default: return 4;
    }
}

bool try_mask_batch(Ctx &c, const CompJob &J, bool flat) {
    if (!flat || J.n_ops != 2) return false;
    const CompOp &o0 = J.ops[0], &o1 = J.ops[1];
    if (o0.op != Z2D_OP_DST_IN || o0.dst.kind != SRC_PIXEL || o0.src.kind != SRC_SURFACE) return false;
    if (o0.src.sfc.fmt != Z2D_FORMAT_ALPHA8 || o0.src.sfc.w != J.dst.w || o0.src.sfc.h < J.dst.h) return false;
    if (o1.dst.kind != SRC_NONE || o1.src.kind != SRC_NONE) return false;
    if (o1.op < 0 || o1.op >= Z2D_OP_COUNT) return false;
    if ((reinterpret_cast<uintptr_t>(o0.src.sfc.data) & 15) != 0) return false;
    const size_t px = (size_t)J.dst.w * J.dst.h;
    // float precision and the packed formats (composite_fused.cu)
    if (J.precision == Z2D_PRECISION_FLOAT)
        return launch_mask_float(c, J.dst.data, J.dst.fmt, o0.src.sfc.data, px, o1.op, o0.dst.pixf);
    if (fmt_packed(J.dst.fmt)) return launch_mask_packed(c, J.dst.data, J.dst.fmt, o0.src.sfc.data, px, o1.op, o0.dst.pix);
    const int per = J.dst.fmt <= Z2D_FORMAT_RGBA ? 4 : 16;
    if (px % per != 0) return false;
    const size_t n_chunks = px / per;
    MaskKernel k;
    switch (J.dst.fmt) {
        case Z2D_FORMAT_ARGB: k = mask_kernel<Z2D_FORMAT_ARGB>(o1.op); break;
        case Z2D_FORMAT_XRGB: k = mask_kernel<Z2D_FORMAT_XRGB>(o1.op); break;
        case Z2D_FORMAT_RGB: k = mask_kernel<Z2D_FORMAT_RGB>(o1.op); break;
        case Z2D_FORMAT_RGBA: k = mask_kernel<Z2D_FORMAT_RGBA>(o1.op); break;
        default: k = mask_kernel<Z2D_FORMAT_ALPHA8>(o1.op); break;
    }
    std::atomic<int> &occ_slot = g_mask_occ[fmt_slot(J.dst.fmt)][o1.op];
    int occ = occ_slot.load(std::memory_order_relaxed);
    if (occ <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kMaskThreads, 0) != cudaSuccess || occ <= 0) occ = 4;
        occ_slot.store(occ, std::memory_order_relaxed);
    }
    const size_t tile = (size_t)kMaskThreads * kMaskUnroll;
    size_t blocks = (n_chunks + tile - 1) / tile;
    const size_t cap = (size_t)c.sm_count * (size_t)occ;
    if (blocks > cap) blocks = cap;
    if (blocks == 0) return true;
    const I16 s = o0.dst.pix;
    k<<<(unsigned)blocks, kMaskThreads, 0, c.stream>>>(J.dst.data, o0.src.sfc.data, n_chunks, s);
    c.launches++;
    return true;
}

}  // namespace z2dg
