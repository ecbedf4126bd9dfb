// edges.cuh -- Polygon.addEdge on the device and the ordered keys of the
// per-fill extents, shared by the fill flattener and the stroker.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

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

__device__ __forceinline__ void add_edge(const FillCmd &F, DEdge *out, double x0, double y0, double x1, double y1,
                                         double &et, double &eb, double &el, double &er, bool &any) {
    // Polygon.addEdge (Polygon.zig:61-109)
    const double ax = x0 * F.edge_scale, ay = y0 * F.edge_scale, bx = x1 * F.edge_scale, by = y1 * F.edge_scale;
    DEdge e;
    if (ay < by) {
        e.top = ay;
        e.x_start = ax;
        e.x_inc = (bx - ax) / (by - ay);
        e.dir = -1;
        e.rb = (int32_t)round(by);
    } else if (ay > by) {
        e.top = by;
        e.x_start = bx;
        e.x_inc = (ax - bx) / (ay - by);
        e.dir = 1;
        e.rb = (int32_t)round(ay);
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
    e.rt = (int32_t)round(e.top);
    e.fxs = (float)e.x_start;
    e.fxi = (float)e.x_inc;
    e.ftp = (float)e.top;
    const double bot = ay < by ? by : ay;
    const double l = ax < bx ? ax : bx, r = ax < bx ? bx : ax;
    if (!any) {
        et = e.top; eb = bot; el = l; er = r;
        any = true;
    } else {
        if (e.top < et) et = e.top;
        if (bot > eb) eb = bot;
        if (l < el) el = l;
        if (r > er) er = r;
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
        double mt = any ? et : 1e300, mb = any ? eb : -1e300, ml = any ? el : 1e300, mr = any ? er : -1e300;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mt = fmin(mt, __shfl_xor_sync(all, mt, o));
            mb = fmax(mb, __shfl_xor_sync(all, mb, o));
            ml = fmin(ml, __shfl_xor_sync(all, ml, o));
            mr = fmax(mr, __shfl_xor_sync(all, mr, o));
        }
        if ((int)(threadIdx.x & 31) == lead) {
            FillState &S = st[f0];
            atomicMin(&S.ext[0], dkey(mt));
            atomicMax(&S.ext[1], dkey(mb));
            atomicMin(&S.ext[2], dkey(ml));
            atomicMax(&S.ext[3], dkey(mr));
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
