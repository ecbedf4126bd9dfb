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

}  // namespace z2dg
