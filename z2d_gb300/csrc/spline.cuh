// spline.cuh -- Bezier subdivision of z2d's Spline.zig on the device,
// shared by the fill flattener (fill.cu) and the stroker (stroke_gpu.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "f64_int.cuh"
#include "fill.cuh"

namespace z2dg {

__host__ __device__ __forceinline__ bool pt_eq(double ax, double ay, double bx, double by) {
    return f64_eq(ax, bx) && f64_eq(ay, by);
}

struct Knots {
    double ax, ay, bx, by, cx, cy, dx, dy;
};

// Spline.Knots.errorSq (Spline.zig:83-123)
__device__ __forceinline__ double error_sq(const Knots &k) {
    double bx = k.bx - k.ax, by = k.by - k.ay, cx = k.cx - k.ax, cy = k.cy - k.ay;
    if (k.ax != k.dx || k.ay != k.dy) {
        const double dx = k.dx - k.ax, dy = k.dy - k.ay;
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
// f64 -> f32 by truncating the mantissa (relative error < 2^-23) with
// integer operations only, so that no FP64 instruction is spent on it.
// False outside f32's normal range (zero excepted).
__device__ __forceinline__ bool f32_trunc(double v, float &out) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const uint32_t hi = (uint32_t)(b >> 32);
    const uint32_t sign = hi & 0x80000000u;
    if ((b << 1) == 0ull) {
        out = __uint_as_float(sign);
        return true;
    }
    const int32_t fe = (int32_t)((hi >> 20) & 0x7FFu) - 1023 + 127;
    if (fe <= 0 || fe >= 255) return false;
    out = __uint_as_float(sign | ((uint32_t)fe << 23) | ((uint32_t)(b >> 29) & 0x7FFFFFu));
    return true;
}

// The decision errorSq(k) < tol2 of Spline.decomposeInto, taken in f32 when
// that is safe.  GB300 runs f64 at a small fraction of its f32 rate, and the
// error test is most of the subdivision's f64 work.  Every f32 quantity
// carries an absolute error bound built from first-order rounding analysis
// with slack: each input's own bound, each operation u (u = 2^-24),
// propagated through the projection and the squared norms.
// Returns 1 / 0 when the f32 value is farther than its bound from tol2 and,
// on the projection branches, from the branch condition; -1 otherwise (the
// caller then evaluates errorSq in f64).
__device__ __forceinline__ int error_sq_lt_f32_core(float bx, float by, float cx, float cy, float ebx, float eby,
                                                    float ecx, float ecy, bool proj, float dx, float dy, float edx,
                                                    float edy, float tol2f, float tol2e) {
    const float U = 5.9604644775390625e-8f;  // 2^-24
    if (proj) {
        const float dd = dx * dx + dy * dy;
        // the inputs' errors carried through the squares, then the roundings
        const float edd = 2.0f * fabsf(dx) * edx + edx * edx + 2.0f * fabsf(dy) * edy + edy * edy + 3.0f * U * dd;
#pragma unroll
        for (int i = 0; i < 2; i++) {
            float &px = i ? cx : bx, &py = i ? cy : by;
            float &epx = i ? ecx : ebx, &epy = i ? ecy : eby;
            const float t1 = px * dx, t2 = py * dy;
            const float pd = t1 + t2;
            const float epd = fabsf(dx) * epx + fabsf(px) * edx + epx * edx + fabsf(dy) * epy + fabsf(py) * edy +
                              epy * edy + 2.0f * U * (fabsf(t1) + fabsf(t2));
            const float diff = pd - dd;
            const float m = 1.125f * (epd + edd) + 2.0f * U * fabsf(diff) + 1e-30f;
            if (diff > m) {  // pd >= dd: subtract the whole chord
                const float nx = px - dx, ny = py - dy;
                epx = epx + edx + 2.0f * U * fabsf(nx);
                epy = epy + edy + 2.0f * U * fabsf(ny);
                px = nx;
                py = ny;
            } else if (diff < -m && dd > 0.0f) {  // subtract the projection onto the chord
                const float t = pd / dd;
                const float et = (epd + fabsf(t) * edd) / dd * 1.125f + 2.0f * U * fabsf(t) + 1e-30f;
                const float rx = t * dx, ry = t * dy;
                const float nx = px - rx, ny = py - ry;
                epx = epx + fabsf(dx) * et + fabsf(t) * edx + 2.0f * U * (fabsf(rx) + fabsf(nx));
                epy = epy + fabsf(dy) * et + fabsf(t) * edy + 2.0f * U * (fabsf(ry) + fabsf(ny));
                px = nx;
                py = ny;
            } else {
                return -1;
            }
        }
    }
    const float be = bx * bx + by * by, ce = cx * cx + cy * cy;
    const float ebe = 2.0f * fabsf(bx) * ebx + 2.0f * fabsf(by) * eby + ebx * ebx + eby * eby + 4.0f * U * be;
    const float ece = 2.0f * fabsf(cx) * ecx + 2.0f * fabsf(cy) * ecy + ecx * ecx + ecy * ecy + 4.0f * U * ce;
    const float e = be > ce ? be : ce;
    const float E = 1.25f * (ebe > ece ? ebe : ece) + 4.0f * U * e + 1e-30f + tol2e;
    if (!(E < 1e30f)) return -1;
    if (e + E < tol2f) return 1;
    if (e - E > tol2f) return 0;
    return -1;
}
// From the exact f64 differences b - a, c - a, d - a (truncation error < 2u
// of each).
__device__ __forceinline__ int error_sq_lt_f32(double bx64, double by64, double cx64, double cy64, bool proj,
                                               double dx64, double dy64, float tol2f, float tol2e) {
    const float U = 5.9604644775390625e-8f;  // 2^-24
    float bx, by, cx, cy, dx = 0.0f, dy = 0.0f;
    if (!f32_trunc(bx64, bx) || !f32_trunc(by64, by) || !f32_trunc(cx64, cx) || !f32_trunc(cy64, cy)) return -1;
    if (proj && (!f32_trunc(dx64, dx) || !f32_trunc(dy64, dy))) return -1;
    return error_sq_lt_f32_core(bx, by, cx, cy, 2.0f * U * fabsf(bx), 2.0f * U * fabsf(by), 2.0f * U * fabsf(cx),
                                2.0f * U * fabsf(cy), proj, dx, dy, 2.0f * U * fabsf(dx), 2.0f * U * fabsf(dy), tol2f,
                                tol2e);
}
// From the knots' coordinates, truncated to f32 (error < 2u of each) and
// subtracted in f32 (one more rounding): no f64 instruction at all, at the
// price of wider bounds (the coordinates' size instead of the differences').
__device__ __forceinline__ int error_sq_lt_f32_pts(double ax64, double ay64, double bx64, double by64, double cx64,
                                                   double cy64, double dx64, double dy64, bool proj, float tol2f,
                                                   float tol2e) {
    const float U = 5.9604644775390625e-8f;  // 2^-24
    float ax, ay, pbx, pby, pcx, pcy, pdx = 0.0f, pdy = 0.0f;
    if (!f32_trunc(ax64, ax) || !f32_trunc(ay64, ay) || !f32_trunc(bx64, pbx) || !f32_trunc(by64, pby) ||
        !f32_trunc(cx64, pcx) || !f32_trunc(cy64, pcy))
        return -1;
    if (proj && (!f32_trunc(dx64, pdx) || !f32_trunc(dy64, pdy))) return -1;
    const float bx = pbx - ax, by = pby - ay, cx = pcx - ax, cy = pcy - ay, dx = pdx - ax, dy = pdy - ay;
    const float eax = 2.0f * U * fabsf(ax), eay = 2.0f * U * fabsf(ay);
    return error_sq_lt_f32_core(bx, by, cx, cy, eax + 2.0f * U * fabsf(pbx) + U * fabsf(bx),
                                eay + 2.0f * U * fabsf(pby) + U * fabsf(by), eax + 2.0f * U * fabsf(pcx) + U * fabsf(cx),
                                eay + 2.0f * U * fabsf(pcy) + U * fabsf(cy), proj, dx, dy,
                                eax + 2.0f * U * fabsf(pdx) + U * fabsf(dx), eay + 2.0f * U * fabsf(pdy) + U * fabsf(dy),
                                tol2f, tol2e);
}

// The squared tolerance of a subdivision, in f64 and as a truncated f32
// with its error bound.
struct Tol {
    double d;
    float f, e;
    bool f_ok;
};
__device__ __forceinline__ Tol make_tol(double tol) {
    Tol t;
    t.d = tol * tol;  // decomposeInto's tolerance argument (Spline.zig:52)
    t.f = 0.0f;
    t.f_ok = f32_trunc(t.d, t.f);
    t.e = 4.0f * 5.9604644775390625e-8f * t.f;
    return t;
}

// errorSq(k) < t.d, exactly as the f64 comparison decides it.
// The rarely needed tests of below_tol, out of line so that the
// subdivision loops that inline below_tol stay small in the instruction
// cache.
static __device__ __noinline__ bool below_tol_slow(Knots k, Tol t, bool proj) {
    if (t.f_ok) {
        const int r = error_sq_lt_f32(k.bx - k.ax, k.by - k.ay, k.cx - k.ax, k.cy - k.ay, proj, k.dx - k.ax,
                                      k.dy - k.ay, t.f, t.e);
        if (r >= 0) return r != 0;
    }
    return error_sq(k) < t.d;
}

// Out of line, like the split: the subdivision loops stay small in the
// instruction cache and the curve kernels need 96 registers instead of
// 118-124 (flatten of the 2,000-path batch 0.68 -> 0.59 ms).
static __device__ __noinline__ bool below_tol(const Knots &k, const Tol &t) {
    const bool proj = !pt_eq(k.ax, k.ay, k.dx, k.dy);
    if (t.f_ok) {
        // from the coordinates first (no f64), then from the exact f64
        // differences, then errorSq itself
        const int r = error_sq_lt_f32_pts(k.ax, k.ay, k.bx, k.by, k.cx, k.cy, k.dx, k.dy, proj, t.f, t.e);
        if (r >= 0) return r != 0;
    }
    return below_tol_slow(k, t, proj);
}

// x / 2.  For normal x whose half is normal this only lowers the exponent,
// which integer operations do exactly (an f64 multiply is an expensive
// instruction on GB300); zeros, subnormals and non-finite values divide.
__device__ __forceinline__ double half_of(double x) {
    const long long b = __double_as_longlong(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    if (e > 1u && e < 0x7FFu) return __longlong_as_double(b - (1ll << 52));
    return x / 2;
}
// The f64 form, out of line so that it runs only on the lanes that need it.
static __device__ __noinline__ double lerp_half_f64(double a, double b) { return a + half_of(b - a); }
__device__ __forceinline__ double lerp_half(double a, double b) {
    bool done;
    const double r = lerp_half_int(a, b, done);
    if (done) return r;
    return lerp_half_f64(a, b);
}

// Knots.deCasteljau (Spline.zig:128-152): k becomes the first half, the
// second half is returned.  Out of line: one copy serves the frontier
// expansion and the depth-first walks (flatten of the 2,000-path batch
// 0.72 -> 0.68 ms against the inlined copies).
static __device__ __noinline__ Knots de_casteljau(Knots &k) {
    const double abx = lerp_half(k.ax, k.bx), aby = lerp_half(k.ay, k.by);
    const double bcx = lerp_half(k.bx, k.cx), bcy = lerp_half(k.by, k.cy);
    const double cdx = lerp_half(k.cx, k.dx), cdy = lerp_half(k.cy, k.dy);
    const double abbcx = lerp_half(abx, bcx), abbcy = lerp_half(aby, bcy);
    const double bccdx = lerp_half(bcx, cdx), bccdy = lerp_half(bcy, cdy);
    const double fx = lerp_half(abbcx, bccdx), fy = lerp_half(abbcy, bccdy);
    const Knots r{fx, fy, bccdx, bccdy, cdx, cdy, k.dx, k.dy};
    k.bx = abx; k.by = aby;
    k.cx = abbcx; k.cy = abbcy;
    k.dx = fx; k.dy = fy;
    return r;
}

// Depth-first subdivision (Spline.decomposeInto, Spline.zig:56-71) with an
// explicit stack.  Calls emit(x, y) for every lineTo the reference issues,
// including the final lineTo(d).  Returns false if the stack would overflow
// (coordinates are bounded, so this does not happen for valid input).
template <class F>
__device__ __forceinline__ bool spline_walk(double ax, double ay, const double *p, double tol, F &&emit) {
    const double bx = p[0], by = p[1], cx = p[2], cy = p[3], dx = p[4], dy = p[5];
    if (pt_eq(ax, ay, bx, by) && pt_eq(cx, cy, dx, dy)) {  // Spline.zig:39-42
        emit(dx, dy);
        return true;
    }
    const Tol t = make_tol(tol);
    Knots stack[kSplineStack];
    int sp = 0;
    stack[sp++] = Knots{ax, ay, bx, by, cx, cy, dx, dy};
    bool ok = true;
    int32_t budget = kSplineMaxSplits;  // bounds the walk even for pathological input
    while (sp > 0 && ok) {
        Knots k = stack[--sp];
        while (true) {
            if (--budget < 0) {
                ok = false;
                break;
            }
            if (below_tol(k, t)) {
                if (!pt_eq(k.ax, k.ay, ax, ay)) emit(k.ax, k.ay);
                break;
            }
            const Knots second = de_casteljau(k);
            if (sp >= kSplineStack) {  // cannot recurse deeper: give up on this branch
                ok = false;
                break;
            }
            stack[sp++] = second;  // processed after the first half
        }
    }
    emit(dx, dy);
    return ok;
}

}  // namespace z2dg
