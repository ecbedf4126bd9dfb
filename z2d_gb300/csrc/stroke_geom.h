// stroke_geom.h -- the geometry of z2d's stroke tessellation, shared by the
// host builder (stroke.cpp) and the device stroker (stroke_gpu.cu).
//
// Every function is plain IEEE f64 arithmetic (+, -, *, /, sqrt; the build
// turns off FMA contraction on both sides), so host and device produce the
// same bits for the same inputs.  On the device, divisions use the exact
// integer long division of f64_int.cuh (the same quotient as the f64
// instructions, which GB300 runs at 1/64 of its f32 rate).  Trigonometry
// (the pen) stays on the host.
#pragma once
#include <math.h>
#include <stdint.h>

#include "f64_int.cuh"
#ifdef __CUDACC__
#define Z2D_HD __host__ __device__ __forceinline__
// out of line on the device: one copy of the larger pieces serves every
// call site of the element kernels, which keeps them small in the
// instruction cache
#define Z2D_HD_CALL static __host__ __device__ __noinline__
#else
#define Z2D_HD inline
#define Z2D_HD_CALL inline
#endif

namespace z2dg {
namespace sg {

struct Pt {
    double x, y;
};
Z2D_HD bool eq(Pt a, Pt b) { return a.x == b.x && a.y == b.y; }

// a / b: on the device through the integer long division of f64_int.cuh
// (the same IEEE quotient; an f64 division costs several f64 instructions).
Z2D_HD double div(double a, double b) {
#ifdef __CUDA_ARCH__
    return f64_div_dev(a, b);
#else
    return a / b;
#endif
}

// Transformation.zig
struct Tf {
    double ax, by, cx, dy, tx, ty;
};
Z2D_HD bool is_identity(const Tf &a) {
    return a.ax == 1 && a.by == 0 && a.cx == 0 && a.dy == 1 && a.tx == 0 && a.ty == 0;
}
Z2D_HD double determinant(const Tf &a) { return a.ax * a.dy - a.by * a.cx; }
// Transformation.inverse (Transformation.zig:103-162)
Z2D_HD bool inverse(const Tf &a, Tf &out) {
    if (a.by == 0 && a.cx == 0) {
        if (a.ax == 0 || a.dy == 0) return false;
        if (a.ax != 1 || a.dy != 1) {
            out = Tf{1 / a.ax, 0, 0, 1 / a.dy, -a.tx / a.ax, -a.ty / a.dy};
        } else {
            out = Tf{1, 0, 0, 1, -a.tx, -a.ty};
        }
        return true;
    }
    const double det = determinant(a);
    if (det == 0) return false;
    const Tf adj{a.dy, -a.by, -a.cx, a.ax, a.by * a.ty - a.dy * a.tx, a.cx * a.tx - a.ax * a.ty};
    const double s = 1 / det;  // mulScalar(1 / det)
    out = Tf{adj.ax * s, adj.by * s, adj.cx * s, adj.dy * s, adj.tx * s, adj.ty * s};
    return true;
}
Z2D_HD void user_to_device_distance(const Tf &a, double &x, double &y) {
    const double ix = x, iy = y;
    x = a.ax * ix + a.by * iy;
    y = a.cx * ix + a.dy * iy;
}
Z2D_HD void device_to_user_distance(const Tf &a, double &x, double &y) {
    Tf inv;
    inverse(a, inv);  // validated by the caller
    user_to_device_distance(inv, x, y);
}

// The Euclidean norm of (x, y) for finite x, y: sqrt(x*x + y*y), with both
// operands scaled by a power of two first when a square could overflow or
// lose bits to underflow (the scaling is exact).
Z2D_HD double hypot2(double x, double y) {
    double a = fabs(x), b = fabs(y);
    if (a < b) {
        const double t = a;
        a = b;
        b = t;
    }
    if (a == 0) return 0;
    if (a < 0x1p500 && b > 0x1p-500) return sqrt(a * a + b * b);
    if (a < 0x1p500 && b == 0) return a;
    const double s = a >= 0x1p500 ? 0x1p-600 : 0x1p600;
    const double as = a * s, bs = b * s;
    return sqrt(as * as + bs * bs) / s;
}

// Slope.zig
struct Slope {
    double dx, dy;
};
Z2D_HD Slope slope(Pt a, Pt b) { return Slope{b.x - a.x, b.y - a.y}; }
Z2D_HD int fsign(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }
// Slope.compare (Slope.zig:46-85)
Z2D_HD int compare(Slope a, Slope b) {
    const double fe = 2.220446049250313e-16;  // floatEps(f64)
    const double bdy = (fabs(b.dy - a.dy) > fe) ? b.dy : a.dy;
    const double bdx = (fabs(b.dx - a.dx) > fe) ? b.dx : a.dx;
    const int cmp = fsign(a.dy * bdx - bdy * a.dx);
    if (cmp != 0) return cmp;
    if (a.dx == 0 && a.dy == 0 && bdx == 0 && bdy == 0) return 0;
    if (a.dx == 0 && a.dy == 0) return 1;
    if (bdx == 0 && bdy == 0) return -1;
    if (fsign(a.dx) != fsign(bdx) || fsign(a.dy) != fsign(bdy)) return (a.dx > 0 || (a.dx == 0 && a.dy > 0)) ? -1 : 1;
    return 0;
}
// Slope.normalize (Slope.zig:117-146)
Z2D_HD double normalize(Slope &s) {
    double rx, ry, mag;
    if (s.dx == 0.0) {
        rx = 0.0;
        if (s.dy > 0.0) {
            mag = s.dy;
            ry = 1.0;
        } else {
            mag = -s.dy;
            ry = -1.0;
        }
    } else if (s.dy == 0.0) {
        ry = 0.0;
        if (s.dx > 0.0) {
            mag = s.dx;
            rx = 1.0;
        } else {
            mag = -s.dx;
            rx = -1.0;
        }
    } else {
        mag = hypot2(s.dx, s.dy);
        rx = div(s.dx, mag);
        ry = div(s.dy, mag);
    }
    s.dx = rx;
    s.dy = ry;
    return mag;
}
Z2D_HD Slope normalized(Slope s) {
    normalize(s);
    return s;
}
// Slope.compare_for_miter_limit (Slope.zig:88-105)
Z2D_HD bool compare_for_miter_limit(Slope in, Slope out, double miter_limit) {
    const Slope a = normalized(in), b = normalized(out);
    const double in_dot_out = a.dx * b.dx + a.dy * b.dy;
    return 2 <= miter_limit * miter_limit * (1 + in_dot_out);
}

// Face.zig: a segment's start and end offset by half the line width on
// either side, the offsets taken in user space and mapped through the CTM.
struct Face {
    Pt p0, p1;
    double width;
    Slope dev_slope, user_slope;
    double half_width;
    Pt p0_cw, p0_ccw, p1_cw, p1_ccw;
};
// Face.initSlope (Face.zig:50-94)
Z2D_HD_CALL Face face_init2(Pt p0, Pt p1, Slope dev_slope, double thickness, const Tf &ctm) {
    const double half = thickness / 2;
    double ox, oy;
    Slope user_slope = dev_slope;
    if (!is_identity(ctm)) {
        double dx = dev_slope.dx, dy = dev_slope.dy;
        device_to_user_distance(ctm, dx, dy);
        user_slope = normalized(Slope{dx, dy});
        if (determinant(ctm) >= 0) {
            ox = -user_slope.dy * half;
            oy = user_slope.dx * half;
        } else {
            ox = user_slope.dy * half;
            oy = -user_slope.dx * half;
        }
        user_to_device_distance(ctm, ox, oy);
    } else {
        ox = -dev_slope.dy * half;
        oy = dev_slope.dx * half;
    }
    const double cwx = ox, cwy = oy, ccwx = -cwx, ccwy = -cwy;
    Face f;
    f.p0 = p0;
    f.p1 = p1;
    f.width = thickness;
    f.dev_slope = dev_slope;
    f.user_slope = user_slope;
    f.half_width = half;
    f.p0_cw = Pt{p0.x + cwx, p0.y + cwy};
    f.p0_ccw = Pt{p0.x + ccwx, p0.y + ccwy};
    f.p1_cw = Pt{p1.x + cwx, p1.y + cwy};
    f.p1_ccw = Pt{p1.x + ccwx, p1.y + ccwy};
    return f;
}
// Face.init (Face.zig:41-48)
Z2D_HD Face face_init(Pt p0, Pt p1, double thickness, const Tf &ctm) {
    return face_init2(p0, p1, normalized(slope(p0, p1)), thickness, ctm);
}
// Face.intersect (Face.zig:96-125)
Z2D_HD Pt intersect(const Face &in, const Face &out, bool clockwise) {
    const Pt ip = clockwise ? in.p1_ccw : in.p1_cw;
    const Pt op = clockwise ? out.p0_ccw : out.p0_cw;
    const Slope is = normalized(in.dev_slope), os = normalized(out.dev_slope);
    const double ry = div((op.x - ip.x) * is.dy * os.dy - op.y * os.dx * is.dy + ip.y * is.dx * os.dy,
                          is.dx * os.dy - os.dx * is.dy);
    const double rx = (fabs(is.dy) >= fabs(os.dy)) ? div((ry - ip.y) * is.dx, is.dy) + ip.x
                                                    : div((ry - op.y) * os.dx, os.dy) + op.x;
    return Pt{rx, ry};
}

// Pen.zig: vertices of the polygonal pen (computed on the host) with the
// slopes of the edges on either side of each.
struct PenVertex {
    Pt point;
    Slope slope_cw, slope_ccw;
};
// Pen.vertexIteratorFor (Pen.zig:100-195): the vertices from `from` to `to`
// are start, start+-1, ... up to but excluding end (+1 when clockwise,
// -1 otherwise, wrapping); returns how many.
Z2D_HD int32_t pen_range(const PenVertex *v, int32_t len, Slope from, Slope to, bool clockwise, int32_t &start) {
    start = 0;
    if (len <= 0) return 0;
    int32_t end;
    if (clockwise) {
        int32_t low = 0, high = len, i = (low + high) >> 1;
        while (high - low > 1) {
            if (compare(v[i].slope_cw, from) < 0) low = i;
            else high = i;
            i = (low + high) >> 1;
        }
        if (compare(v[i].slope_cw, from) < 0) {
            i += 1;
            if (i == len) i = 0;
        }
        start = i;
        if (compare(to, v[i].slope_ccw) >= 0) {
            low = i;
            high = i + len;
            i = (low + high) >> 1;
            while (high - low > 1) {
                const int32_t j = i >= len ? i - len : i;
                if (compare(v[j].slope_cw, to) > 0) high = i;
                else low = i;
                i = (low + high) >> 1;
            }
            if (i >= len) i -= len;
        }
        end = i;
    } else {
        int32_t low = 0, high = len, i = (low + high) >> 1;
        while (high - low > 1) {
            if (compare(from, v[i].slope_ccw) < 0) low = i;
            else high = i;
            i = (low + high) >> 1;
        }
        if (compare(from, v[i].slope_ccw) < 0) {
            i += 1;
            if (i == len) i = 0;
        }
        start = i;
        if (compare(v[i].slope_cw, to) <= 0) {
            low = i;
            high = i + len;
            i = (low + high) >> 1;
            while (high - low > 1) {
                const int32_t j = i >= len ? i - len : i;
                if (compare(to, v[j].slope_ccw) > 0) high = i;
                else low = i;
                i = (low + high) >> 1;
            }
            if (i >= len) i -= len;
        }
        end = i;
    }
    // VertexIterator.next (Pen.zig:204-222)
    if (start < 0) start = 0;
    if (end < 0) end = 0;
    return clockwise ? (end - start + len) % len : (start - end + len) % len;
}
// The k-th vertex index of a pen_range walk.
Z2D_HD int32_t pen_step(int32_t start, int32_t k, int32_t len, bool clockwise) {
    const int32_t i = clockwise ? start + k : start - k;
    return ((i % len) + len) % len;
}

}  // namespace sg
}  // namespace z2dg
