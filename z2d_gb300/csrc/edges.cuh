// edges.cuh -- Polygon.addEdge on the device and the ordered keys of the
// per-fill extents, shared by the fill flattener and the stroker.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "f64_int.cuh"
#include "fill.cuh"

namespace z2dg {

// Order-preserving map of finite doubles to u64 (for atomic min/max).
__device__ __forceinline__ unsigned long long dkey(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double dkey_inv(unsigned long long k) {
    unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    memcpy(&d, &b, 8);
    return d;
#endif
}

// The f64 operations of addEdge that have exact integer forms
// (f64_int.cuh), with the f64 instruction for the operands they decline.
__device__ __forceinline__ double scale_coord(double v, double s) {
    bool ok;
    const double r = f64_scale_pow2(v, s, ok);
    if (ok) return r;
    return f64_mul_hw(v, s);
}
__device__ __forceinline__ int32_t round_i32(double v) {
    bool ok;
    const int32_t r = f64_round_i32(v, ok);
    if (ok) return r;
    return f64_round_i32_hw(v);
}
__device__ __forceinline__ float to_f32(double v) {
    bool ok;
    const float r = f64_to_f32(v, ok);
    if (ok) return r;
    return f64_to_f32_hw(v);
}

__device__ __forceinline__ void add_edge(const FillCmd &F, DEdge *out, double x0, double y0, double x1, double y1,
                                         double &et, double &eb, double &el, double &er, bool &any) {
    // Polygon.addEdge (Polygon.zig:61-109)
    const double ax = scale_coord(x0, F.edge_scale), ay = scale_coord(y0, F.edge_scale);
    const double bx = scale_coord(x1, F.edge_scale), by = scale_coord(y1, F.edge_scale);
    DEdge e;
    const bool down = f64_lt(ay, by);
    if (down) {
        e.top = ay;
        e.x_start = ax;
        e.x_inc = f64_div_dev(bx - ax, by - ay);
        e.dir = -1;
        e.rb = round_i32(by);
    } else if (f64_lt(by, ay)) {
        e.top = by;
        e.x_start = bx;
        e.x_inc = f64_div_dev(ax - bx, ay - by);
        e.dir = 1;
        e.rb = round_i32(ay);
    } else {
        e.top = 0;
        e.x_start = 0;
        e.x_inc = 0;
        e.fxs = e.fxi = e.ftp = 0.0f;
        e.dir = 0;
        e.rt = 1;
        e.rb = 0;  // horizontal: never active
        *out = e;
        return;
    }
    e.rt = round_i32(e.top);
    e.fxs = to_f32(e.x_start);
    e.fxi = to_f32(e.x_inc);
    e.ftp = to_f32(e.top);
    const double bot = down ? by : ay;
    const bool lr = f64_lt(ax, bx);
    const double l = lr ? ax : bx, r = lr ? bx : ax;
    if (!any) {
        et = e.top; eb = bot; el = l; er = r;
        any = true;
    } else {
        if (f64_lt(e.top, et)) et = e.top;
        if (f64_lt(eb, bot)) eb = bot;
        if (f64_lt(l, el)) el = l;
        if (f64_lt(er, r)) er = r;
    }
    *out = e;
}

// Merges the lanes' edge extents into their fills' FillState: one set of
// atomics per warp when every lane that has edges draws the same fill, one
// per lane otherwise.  All 32 lanes must call it.
__device__ __forceinline__ void merge_extents(FillState *st, int32_t f, bool any, double et, double eb, double el,
                                              double er) {
    const unsigned all = 0xffffffffu;
    const unsigned am = __ballot_sync(all, any);
    if (!am) return;
    const int lead = __ffs(am) - 1;
    const int32_t f0 = __shfl_sync(all, f, lead);
    if (__all_sync(all, !any || f == f0)) {
        // reduced as ordered keys: integer minima and maxima (f64 min/max
        // instructions run on GB300's narrow f64 pipe)
        unsigned long long mt = any ? dkey(et) : ~0ull, mb = any ? dkey(eb) : 0ull;
        unsigned long long ml = any ? dkey(el) : ~0ull, mr = any ? dkey(er) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mt = min(mt, __shfl_xor_sync(all, mt, o));
            mb = max(mb, __shfl_xor_sync(all, mb, o));
            ml = min(ml, __shfl_xor_sync(all, ml, o));
            mr = max(mr, __shfl_xor_sync(all, mr, o));
        }
        if ((int)(threadIdx.x & 31) == lead) {
            FillState &S = st[f0];
            atomicMin(&S.ext[0], mt);
            atomicMax(&S.ext[1], mb);
            atomicMin(&S.ext[2], ml);
            atomicMax(&S.ext[3], mr);
            atomicOr(&S.has_edges, 1);
        }
    } else if (any) {
        FillState &S = st[f];
        atomicMin(&S.ext[0], dkey(et));
        atomicMax(&S.ext[1], dkey(eb));
        atomicMin(&S.ext[2], dkey(el));
        atomicMax(&S.ext[3], dkey(er));
        atomicOr(&S.has_edges, 1);
    }
}

}  // namespace z2dg
