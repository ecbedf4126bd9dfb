// composite_fused.cu -- the mask batch of SurfaceCompositor.run on the
// destinations and precisions the integer byte-format kernel
// (composite_mask.cu) does not take:
//
//  * k_mask_packed<FMT, OP>: integer precision on the packed alpha4 /
//    alpha2 / alpha1 formats.  Each item is 16 pixels: 16 mask bytes (one
//    16-byte vector) and the 16 * BITS destination bits that hold the same
//    pixels (8, 4 or 2 bytes, one aligned vector).  A warp therefore reads
//    512 contiguous mask bytes and 64-256 contiguous destination bytes per
//    load instruction: no shuffles or atomics are needed because every
//    destination word is owned by one lane.  The operator is a template
//    parameter; its result on one pixel depends on the mask byte and the
//    destination value only, so each CTA first tabulates it for every
//    pair (IntegerOps.dstIn on the pixel source's alpha, the operator on the
//    alpha lane after Alpha(T).scaleIntoIntAlpha, the scale back; z2d's
//    packed formats only carry alpha and the operators' alpha lanes read
//    alphas only), and every pixel becomes a table lookup.
//  * k_mask_float<FMT, OP>: float precision (StrideCompositor.runPrecision
//    with .float, compositor.zig:540-621) on the 4-byte formats and alpha8,
//    pixel source.  x / 255 for the 256 byte values comes from a shared
//    table filled with the same IEEE division (decodeRGBAVecRaw), the
//    operator is inlined as a template parameter.
//
// Both are HBM bound by design: each byte of destination and mask moves
// once, with several 16-byte loads in flight per thread before any compute.
#include <cuda_runtime.h>

#include <atomic>
#include <type_traits>
#include <utility>

#include "z2d_internal.h"

namespace z2dg {

constexpr int kFusedThreads = 256;
constexpr int kFusedUnroll = 4;

template <int BITS>
struct PackedUnit;
template <>
struct PackedUnit<4> {
    using T = uint2;
    static __device__ __forceinline__ uint64_t get(T v) { return (uint64_t)v.x | ((uint64_t)v.y << 32); }
    static __device__ __forceinline__ T put(uint64_t v) { return make_uint2((uint32_t)v, (uint32_t)(v >> 32)); }
};
template <>
struct PackedUnit<2> {
    using T = uint32_t;
    static __device__ __forceinline__ uint64_t get(T v) { return v; }
    static __device__ __forceinline__ T put(uint64_t v) { return (uint32_t)v; }
};
template <>
struct PackedUnit<1> {
    using T = uint16_t;
    static __device__ __forceinline__ uint64_t get(T v) { return v; }
    static __device__ __forceinline__ T put(uint64_t v) { return (uint16_t)v; }
};

// The packed kernels' result table.  With a pixel source the result of
// [dst_in(source, mask), op] on one packed pixel depends only on its mask
// byte m and its destination value v (2^BITS of them): the table holds it
// for all 256 x 2^BITS pairs, BITS bits each, at bit (m * 2^BITS + v) * BITS.
// Every CTA evaluates the table once with the operator's own arithmetic,
// then each pixel is one shared-memory lookup instead of the operator.  The
// table is kept in 32 copies interleaved by word (word w of copy l at
// w * 32 + l), and lane l reads copy l: every lane of a warp reads its own
// bank, so random mask bytes never conflict.
template <int BITS>
struct PackedTable {
    static constexpr int LOGB = BITS == 4 ? 2 : BITS == 2 ? 1 : 0;
    static constexpr int POS_M = BITS + LOGB;              // log2(2^BITS * BITS): bits per mask byte
    static constexpr int WORDS = (256 << POS_M) / 32;      // 512, 64, 16
    static constexpr size_t SMEM = (size_t)(WORDS * 32 + WORDS) * sizeof(uint32_t);
};

template <int FMT, int OP>
__global__ void __launch_bounds__(kFusedThreads) k_mask_packed(uint8_t *__restrict__ dst, const uint8_t *__restrict__ mask,
                                                               size_t n_items, uint32_t spa) {
    constexpr int BITS = FMT == Z2D_FORMAT_ALPHA4 ? 4 : FMT == Z2D_FORMAT_ALPHA2 ? 2 : 1;
    constexpr uint32_t MAXV = (1u << BITS) - 1u;
    using TB = PackedTable<BITS>;
    using U = PackedUnit<BITS>;
    using T = typename U::T;
    extern __shared__ uint32_t tab[];
    uint32_t *const words = tab + TB::WORDS * 32;
    for (int w = threadIdx.x; w < TB::WORDS; w += kFusedThreads) {
        uint32_t word = 0;
#pragma unroll 1
        for (int b = 0; b < 32; b += BITS) {
            const uint32_t pos = (uint32_t)w * 32u + (uint32_t)b;
            const uint32_t m = pos >> TB::POS_M, v = (pos >> TB::LOGB) & MAXV;
            const uint32_t ra = (spa * m) / 255u;  // IntegerOps.dstIn, alpha lane
            const I16 r = int_op(OP, I16{0u, 0u, 0u, scale_alpha(v, BITS, 8)}, I16{0u, 0u, 0u, ra});
            word |= scale_alpha(r.a & 0xFFu, 8, BITS) << b;
        }
        words[w] = word;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TB::WORDS * 32; i += kFusedThreads) tab[i] = words[i >> 5];
    __syncthreads();
    const uint32_t *const mine = tab + (threadIdx.x & 31u);
    T *const d = reinterpret_cast<T *>(dst);
    const uint4 *const m = reinterpret_cast<const uint4 *>(mask);
    const size_t tile = (size_t)kFusedThreads * kFusedUnroll;
    for (size_t base = (size_t)blockIdx.x * tile + threadIdx.x; base < n_items; base += (size_t)gridDim.x * tile) {
        T dv[kFusedUnroll];
        uint4 mv[kFusedUnroll];
#pragma unroll
        for (int k = 0; k < kFusedUnroll; k++) {
            const size_t it = base + (size_t)k * kFusedThreads;
            if (it < n_items) {
                dv[k] = d[it];
                mv[k] = __ldcs(m + it);
            }
        }
#pragma unroll
        for (int k = 0; k < kFusedUnroll; k++) {
            const size_t it = base + (size_t)k * kFusedThreads;
            if (it >= n_items) break;
            const uint64_t in = U::get(dv[k]);
            const uint32_t mw[4] = {mv[k].x, mv[k].y, mv[k].z, mv[k].w};
            uint64_t out = 0;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const uint32_t mb = (mw[j >> 2] >> (8 * (j & 3))) & 0xFFu;
                const uint32_t raw = (uint32_t)(in >> (j * BITS)) & MAXV;
                const uint32_t pos = (mb << TB::POS_M) | (raw << TB::LOGB);
                const uint32_t word = mine[pos & ~31u];
                out |= (uint64_t)((word >> (pos & 31u)) & MAXV) << (j * BITS);
            }
            d[it] = U::put(out);
        }
    }
}

template <int FMT, int OP>
__global__ void __launch_bounds__(kFusedThreads) k_mask_float(uint8_t *__restrict__ dst, const uint8_t *__restrict__ mask,
                                                              size_t n_chunks, F4 spf) {
    constexpr bool WIDE = FMT <= Z2D_FORMAT_RGBA;  // 4 px per 16-byte chunk; else 16 alpha8 px
    __shared__ float dec[256];  // decodeRGBAVecRaw: v / 255 in f32
    for (int i = threadIdx.x; i < 256; i += kFusedThreads) dec[i] = (float)i / 255.0f;
    __syncthreads();
    const size_t tile = (size_t)kFusedThreads * kFusedUnroll;
    for (size_t base = (size_t)blockIdx.x * tile + threadIdx.x; base < n_chunks; base += (size_t)gridDim.x * tile) {
        uint4 v[kFusedUnroll];
        uint4 mv[kFusedUnroll];
#pragma unroll
        for (int k = 0; k < kFusedUnroll; k++) {
            const size_t c = base + (size_t)k * kFusedThreads;
            v[k] = make_uint4(0, 0, 0, 0);
            mv[k] = make_uint4(0, 0, 0, 0);
            if (c < n_chunks) {
                v[k] = reinterpret_cast<const uint4 *>(dst)[c];
                if constexpr (WIDE) mv[k].x = __ldcs(reinterpret_cast<const uint32_t *>(mask) + c);
                else mv[k] = __ldcs(reinterpret_cast<const uint4 *>(mask) + c);
            }
        }
#pragma unroll
        for (int k = 0; k < kFusedUnroll; k++) {
            const size_t c = base + (size_t)k * kFusedThreads;
            if (c >= n_chunks) break;
            uint32_t w[4] = {v[k].x, v[k].y, v[k].z, v[k].w};
            if constexpr (WIDE) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const float ma = dec[(mv[k].x >> (8 * j)) & 0xFFu];
                    // FloatOps.dstIn(d = source, s = mask)
                    const F4 r{spf.r * ma, spf.g * ma, spf.b * ma, ma * spf.a};
                    const I16 dp = word_to_i16(w[j], FMT);
                    const F4 df{dec[dp.r], dec[dp.g], dec[dp.b], dec[dp.a]};
                    w[j] = i16_to_word(encode_raw(float_op(OP, df, r)), FMT);
                }
            } else {
                const uint32_t mw[4] = {mv[k].x, mv[k].y, mv[k].z, mv[k].w};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    uint32_t out = 0;
#pragma unroll
                    for (int b = 0; b < 4; b++) {
                        const float ma = dec[(mw[j] >> (8 * b)) & 0xFFu];
                        const F4 r{spf.r * ma, spf.g * ma, spf.b * ma, ma * spf.a};
                        const F4 df{0.0f, 0.0f, 0.0f, dec[(w[j] >> (8 * b)) & 0xFFu]};
                        out |= (encode_raw(float_op(OP, df, r)).a & 0xFFu) << (8 * b);
                    }
                    w[j] = out;
                }
            }
            reinterpret_cast<uint4 *>(dst)[c] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

using PackedKernel = void (*)(uint8_t *, const uint8_t *, size_t, uint32_t);
using FloatKernel = void (*)(uint8_t *, const uint8_t *, size_t, F4);

template <int FMT, int... OPS>
static const PackedKernel *packed_table(std::integer_sequence<int, OPS...>) {
    static const PackedKernel table[] = {&k_mask_packed<FMT, OPS>...};
    return table;
}
template <int FMT, int... OPS>
static const FloatKernel *float_table(std::integer_sequence<int, OPS...>) {
    static const FloatKernel table[] = {&k_mask_float<FMT, OPS>...};
    return table;
}

// Resident blocks per SM of each kernel, looked up once.
static std::atomic<int> g_packed_occ[3][Z2D_OP_COUNT];
static std::atomic<int> g_float_occ[5][Z2D_OP_COUNT];

template <class K>
static size_t grid_for(std::atomic<int> &slot, K k, const Ctx &c, size_t units, size_t smem = 0) {
    int occ = slot.load(std::memory_order_relaxed);
    if (occ <= 0) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kFusedThreads, smem) != cudaSuccess || occ <= 0) occ = 1;
        slot.store(occ, std::memory_order_relaxed);
    }
    const size_t tile = (size_t)kFusedThreads * kFusedUnroll;
    size_t blocks = (units + tile - 1) / tile;
    const size_t cap = (size_t)c.sm_count * (size_t)occ;
    return blocks > cap ? cap : blocks;
}

// Integer mask batch on alpha4 / alpha2 / alpha1 (the shape is checked by
// try_mask_batch).  Needs a whole number of 16-pixel items and a
// destination aligned to its per-item vector.
bool launch_mask_packed(Ctx &c, uint8_t *dst, int fmt, const uint8_t *mask, size_t px, int op, const I16 &spx) {
    if (px % 16 != 0) return false;
    const int bits = fmt_bits(fmt);
    if ((reinterpret_cast<uintptr_t>(dst) & (uintptr_t)(2 * bits - 1)) != 0) return false;
    const std::make_integer_sequence<int, Z2D_OP_COUNT> ops{};
    PackedKernel k;
    int slot;
    switch (fmt) {
        case Z2D_FORMAT_ALPHA4: k = packed_table<Z2D_FORMAT_ALPHA4>(ops)[op]; slot = 0; break;
        case Z2D_FORMAT_ALPHA2: k = packed_table<Z2D_FORMAT_ALPHA2>(ops)[op]; slot = 1; break;
        case Z2D_FORMAT_ALPHA1: k = packed_table<Z2D_FORMAT_ALPHA1>(ops)[op]; slot = 2; break;
        default: return false;
    }
    const size_t smem = bits == 4 ? PackedTable<4>::SMEM : bits == 2 ? PackedTable<2>::SMEM : PackedTable<1>::SMEM;
    const size_t n_items = px / 16;
    const size_t blocks = grid_for(g_packed_occ[slot][op], k, c, n_items, smem);
    if (blocks == 0) return true;
    k<<<(unsigned)blocks, kFusedThreads, smem, c.stream>>>(dst, mask, n_items, spx.a);
    c.launches++;
    return true;
}

// Float mask batch on the 4-byte formats and alpha8, pixel source.
bool launch_mask_float(Ctx &c, uint8_t *dst, int fmt, const uint8_t *mask, size_t px, int op, const F4 &spf) {
    const int per = fmt <= Z2D_FORMAT_RGBA ? 4 : 16;
    if (px % per != 0 || fmt > Z2D_FORMAT_ALPHA8) return false;
    const std::make_integer_sequence<int, Z2D_OP_COUNT> ops{};
    FloatKernel k;
    int slot;
    switch (fmt) {
        case Z2D_FORMAT_ARGB: k = float_table<Z2D_FORMAT_ARGB>(ops)[op]; slot = 0; break;
        case Z2D_FORMAT_XRGB: k = float_table<Z2D_FORMAT_XRGB>(ops)[op]; slot = 1; break;
        case Z2D_FORMAT_RGB: k = float_table<Z2D_FORMAT_RGB>(ops)[op]; slot = 2; break;
        case Z2D_FORMAT_RGBA: k = float_table<Z2D_FORMAT_RGBA>(ops)[op]; slot = 3; break;
        default: k = float_table<Z2D_FORMAT_ALPHA8>(ops)[op]; slot = 4; break;
    }
    const size_t n_chunks = px / per;
    const size_t blocks = grid_for(g_float_occ[slot][op], k, c, n_chunks);
    if (blocks == 0) return true;
    k<<<(unsigned)blocks, kFusedThreads, 0, c.stream>>>(dst, mask, n_chunks, spf);
    c.launches++;
    return true;
}

}  // namespace z2dg
