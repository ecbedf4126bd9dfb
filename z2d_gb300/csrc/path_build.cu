// path_build.cu -- z2d's Path builder on the device.
//
// A path program is the sequence of Path calls a caller makes (moveTo,
// lineTo, curveTo, their rel* forms, arc / arcNegative, close, setting the
// transformation or the tolerance, replaying a glyph outline); the kernel
// runs one program per thread and writes the device-space nodes z2d's Path
// would hold (src/Path.zig:116-479): every user point clamped to z2d's i24
// range, then mapped by the current transformation; a move_to to the point
// of a trailing move_to dropped; close_path followed by a move_to back to
// the subpath's start; rel* points taken from the current point mapped back
// through the inverse transformation; arcs split into cubic splines by
// arc.zig's error bound (src/internal/arc.zig:82-392) with Zig's f64
// sin / cos / tan (zig_trig.cuh).  Glyph outlines (src/internal/Glyph.zig:
// 483-869) are built into their own path with the outline transformation
// scale(1, -1).translate(0, -units_per_em) and replayed node by node into
// the program's path (Outline.appendToPath).
//
// Two passes: the first counts each program's nodes, the host scans the
// counts, the second writes them.  A program stops at its first error
// (NoCurrentPoint -> Z2D_ERR_INVALID_STATE, InvalidMatrix ->
// Z2D_ERR_INVALID_ARGUMENT); its nodes up to there are kept, as in z2d.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "z2d_internal.h"
#include "zig_trig.cuh"

namespace z2dg {

namespace {

struct Tf {
    double ax, by, cx, dy, tx, ty;
};

__device__ __forceinline__ Tf tf_mul(const Tf &a, const Tf &b) {  // Transformation.mul
    Tf r;
    r.ax = a.ax * b.ax + a.by * b.cx;
    r.by = a.ax * b.by + a.by * b.dy;
    r.cx = a.cx * b.ax + a.dy * b.cx;
    r.dy = a.cx * b.by + a.dy * b.dy;
    r.ty = a.cx * b.tx + a.dy * b.ty + a.ty;
    r.tx = a.ax * b.tx + a.by * b.ty + a.tx;
    return r;
}

// Transformation.inverse (src/Transformation.zig:103-162); false when the
// matrix cannot be inverted
__device__ bool tf_inverse(const Tf &a, Tf &o) {
    if (a.by == 0 && a.cx == 0) {
        if (a.ax == 0 || a.dy == 0) return false;
        if (a.ax != 1 || a.dy != 1) {
            o = Tf{1 / a.ax, 0, 0, 1 / a.dy, -a.tx / a.ax, -a.ty / a.dy};
        } else {
            o = Tf{1, 0, 0, 1, -a.tx, -a.ty};
        }
        return true;
    }
    const double det = a.ax * a.dy - a.by * a.cx;
    if (det == 0) return false;
    const Tf adj{a.dy, -a.by, -a.cx, a.ax, a.by * a.ty - a.dy * a.tx, a.cx * a.tx - a.ax * a.ty};
    const double s = 1 / det;
    o = Tf{adj.ax * s, adj.by * s, adj.cx * s, adj.dy * s, adj.tx * s, adj.ty * s};
    return true;
}

__device__ __forceinline__ void tf_apply(const Tf &t, double &x, double &y) {  // userToDevice
    const double ix = x, iy = y;
    x = t.ax * ix + t.by * iy;
    y = t.cx * ix + t.dy * iy;
    x += t.tx;
    y += t.ty;
}

// clampI24 (src/Path.zig:570-572): math.clamp to z2d's i24 range, as
// @max(lo, @min(v, hi)) (a NaN takes the upper bound, as with Zig's @min)
__device__ __forceinline__ double clamp_i24(double v) { return fmax(-8388608.0, fmin(v, 8388607.0)); }

constexpr int kErrNoCurrentPoint = Z2D_ERR_INVALID_STATE;
constexpr int kErrInvalidMatrix = Z2D_ERR_INVALID_ARGUMENT;

// The node sink: counts, and writes when `out` is set.  A reset or a
// rolled-back glyph moves n back; hw is the highest n reached, the room the
// program needs while it runs.
struct Sink {
    z2d_node *out;
    long long n;
    long long hw;
    __device__ void put(int32_t tag, double a = 0, double b = 0, double c = 0, double d = 0, double e = 0,
                        double f = 0) {
        if (out) {
            z2d_node &nd = out[n];
            nd.tag = tag;
            nd._pad = 0;
            nd.p[0] = a;
            nd.p[1] = b;
            nd.p[2] = c;
            nd.p[3] = d;
            nd.p[4] = e;
            nd.p[5] = f;
        }
        n++;
        if (n > hw) hw = n;
    }
};

// One Path's state.  Nodes go to the sink directly, or (for a glyph
// outline) are replayed into another Path.
struct PathState {
    Tf tf;
    double tolerance;
    bool has_cur = false, has_init = false;
    double cx = 0, cy = 0, ix = 0, iy = 0;
    int32_t last_tag = -1;  // the last node appended (for the move_to check)
    double lx = 0, ly = 0;
    Sink *sink = nullptr;
    PathState *replay = nullptr;
    int err = 0;
};

__device__ void path_move_to(PathState &P, double x, double y);
__device__ void path_line_to(PathState &P, double x, double y);
__device__ void path_curve_to(PathState &P, double x1, double y1, double x2, double y2, double x3, double y3);
__device__ void path_close(PathState &P);

__device__ void append(PathState &P, int32_t tag, double a = 0, double b = 0, double c = 0, double d = 0,
                       double e = 0, double f = 0) {
    P.last_tag = tag;
    if (tag == Z2D_MOVE_TO || tag == Z2D_LINE_TO) {
        P.lx = a;
        P.ly = b;
    }
    if (P.replay) {  // Outline.appendToPath (Glyph.zig:830-843)
        PathState &Q = *P.replay;
        if (Q.err) return;
        switch (tag) {
            case Z2D_MOVE_TO: path_move_to(Q, a, b); break;
            case Z2D_LINE_TO: path_line_to(Q, a, b); break;
            case Z2D_CURVE_TO: path_curve_to(Q, a, b, c, d, e, f); break;
            default: path_close(Q); break;
        }
        if (Q.err) P.err = Q.err;
        return;
    }
    P.sink->put(tag, a, b, c, d, e, f);
}

// Path.moveTo (Path.zig:116-145)
__device__ void path_move_to(PathState &P, double x, double y) {
    double px = clamp_i24(x), py = clamp_i24(y);
    tf_apply(P.tf, px, py);
    if (P.last_tag == Z2D_MOVE_TO && P.lx == px && P.ly == py) return;
    append(P, Z2D_MOVE_TO, px, py);
    P.ix = P.cx = px;
    P.iy = P.cy = py;
    P.has_init = P.has_cur = true;
}
// Path.lineTo (:163-183): a move_to without a current point
__device__ void path_line_to(PathState &P, double x, double y) {
    if (!P.has_cur) {
        path_move_to(P, x, y);
        return;
    }
    double px = clamp_i24(x), py = clamp_i24(y);
    tf_apply(P.tf, px, py);
    append(P, Z2D_LINE_TO, px, py);
    P.cx = px;
    P.cy = py;
}
// Path.curveTo (:205-262)
__device__ void path_curve_to(PathState &P, double x1, double y1, double x2, double y2, double x3, double y3) {
    if (!P.has_cur) {
        P.err = kErrNoCurrentPoint;
        return;
    }
    double p1x = clamp_i24(x1), p1y = clamp_i24(y1), p2x = clamp_i24(x2), p2y = clamp_i24(y2);
    double p3x = clamp_i24(x3), p3y = clamp_i24(y3);
    tf_apply(P.tf, p1x, p1y);
    tf_apply(P.tf, p2x, p2y);
    tf_apply(P.tf, p3x, p3y);
    append(P, Z2D_CURVE_TO, p1x, p1y, p2x, p2y, p3x, p3y);
    P.cx = p3x;
    P.cy = p3y;
}
// Path.close (:427-457): close_path, then a move_to back to the start; the
// current point is left where it was
__device__ void path_close(PathState &P) {
    if (!P.has_cur) return;
    append(P, Z2D_CLOSE_PATH);
    append(P, Z2D_MOVE_TO, P.ix, P.iy);
}
// The current point in user space (Point.applyInverseTransform)
__device__ bool current_user(PathState &P, double &x, double &y) {
    if (!P.has_cur) {
        P.err = kErrNoCurrentPoint;
        return false;
    }
    Tf inv;
    if (!tf_inverse(P.tf, inv)) {
        P.err = kErrInvalidMatrix;
        return false;
    }
    x = P.cx;
    y = P.cy;
    tf_apply(inv, x, y);
    return true;
}

// ---------------------------------------------------------------- arcs
// Zig evaluates `math.pi / k` at compile time in f128; pi/3 and pi/6 round
// differently from the f64 division, so the table holds the f64 values of
// those f128 quotients.
__device__ __forceinline__ double arc_table_angle(int i) {
    switch (i) {
        case 0: return 3.141592653589793116;                   // pi / 1
        case 1: return 1.570796326794896558;                   // pi / 2
        case 2: return zm::dfrom(0x3FF0C152382D7366ull);      // pi / 3 (f128 quotient)
        case 3: return 0.7853981633974482790;                  // pi / 4
        case 4: return zm::dfrom(0x3FE41B2F769CF0E0ull);      // pi / 5
        case 5: return zm::dfrom(0x3FE0C152382D7366ull);      // pi / 6 (f128 quotient)
        case 6: return zm::dfrom(0x3FDCB91F3BBBA140ull);      // pi / 7
        case 7: return 0.3926990816987241395;                  // pi / 8
        case 8: return zm::dfrom(0x3FD657184AE74487ull);      // pi / 9
        case 9: return zm::dfrom(0x3FD41B2F769CF0E0ull);      // pi / 10
        default: return zm::dfrom(0x3FD247426BD47DE3ull);     // pi / 11
    }
}
__device__ __forceinline__ double arc_table_err(int i) {
    const double e[11] = {0.0185185185185185036127,    0.000272567143730179811158, 2.38647043651461047433e-05,
                          4.2455377443222443279e-06,   1.11281001494389081528e-06, 3.72662000942734705475e-07,
                          1.47783685574284411325e-07,  6.63240432022601149057e-08, 3.2715520137536980553e-08,
                          1.73863223499021216974e-08,  9.81410988043554039085e-09};
    return e[i];
}

// arc_error_normalized (arc.zig:39-41)
__device__ double arc_error_normalized(double angle, bool &ok) {
    const double s = zm::sin_(angle / 4, ok), c = zm::cos_(angle / 4, ok);
    return 2.0 / 27.0 * zm::powi_(s, 6) / zm::powi_(c, 2);
}
// arc_max_angle_for_tolerance_normalized (arc.zig:43-80)
__device__ double arc_max_angle(double tolerance, bool &ok) {
    for (int i = 0; i < 11; i++)
        if (arc_table_err(i) < tolerance) return arc_table_angle(i);
    double angle = 0;
    for (int i = 11; i < 1000; i++) {
        angle = 3.141592653589793116 / (double)i;
        if (arc_error_normalized(angle, ok) <= tolerance) break;
    }
    return angle;
}
// transformed_circle_major_axis (arc.zig:92-262); hypot(g, h) as
// sqrt(g*g + h*h) (Zig's std.math.hypot is not in the reference tree)
__device__ double major_axis(const Tf &m, double radius) {
    const double a = m.ax, b = m.by, c = m.cx, d = m.dy;
    const double eps = 0.00390625;
    const double det = m.ax * m.dy - m.by * m.cx;
    if (fabs(det * det - 1.0) < eps) {
        if (fabs(m.by) < eps && fabs(m.cx) < eps) return radius;
        if (fabs(m.ax) < eps && fabs(m.dy) < eps) return radius;
    }
    const double i = a * a + b * b, j = c * c + d * d;
    const double f = 0.5 * (i + j), g = 0.5 * (i - j), h = a * c + b * d;
    return radius * sqrt(f + sqrt(g * g + h * h));
}

// arc_line_to (Path.zig:407-425): no-op when the current point equals the
// point (compared as stored: device current point against user point)
__device__ void arc_line_to(PathState &P, double x, double y) {
    if (P.has_cur && P.cx == x && P.cy == y) return;
    path_line_to(P, x, y);
}
// arc_segment (arc.zig:288-310)
__device__ void arc_segment(PathState &P, double xc, double yc, double r, double a, double b, bool &ok) {
    const double r_sin_A = r * zm::sin_(a, ok), r_cos_A = r * zm::cos_(a, ok);
    const double r_sin_B = r * zm::sin_(b, ok), r_cos_B = r * zm::cos_(b, ok);
    const double h = 4.0 / 3.0 * zm::tan_((b - a) / 4.0, ok);
    if (!ok) return;
    path_curve_to(P, xc + r_cos_A - h * r_sin_A, yc + r_sin_A + h * r_cos_A, xc + r_cos_B + h * r_sin_B,
                  yc + r_sin_B - h * r_cos_B, xc + r_cos_B, yc + r_sin_B);
}

// arc_in_direction (arc.zig:322-392).  The recursion on halves of arcs
// wider than pi is a stack of pending halves (depth <= 20 after the
// full-circle normalisation).
__device__ void arc_in_direction(PathState &P, double xc, double yc, double r, double amin0, double amax0,
                                 bool forward, double tolerance) {
    bool ok = true;
    auto finite = [](double x) { return x * x >= 0.0; };
    if (!finite(amax0) || !finite(amin0)) return;
    const double twopi = 6.283185307179586232;
    if (amax0 - amin0 > twopi * 65536.0) {
        double amax = zmod(amax0 - amin0, twopi);
        const double amin = zmod(amin0, twopi);
        amax += amin + twopi * 65536.0;
        amin0 = amin;
        amax0 = amax;
    }
    double lo[24], hi[24];
    int top = 0;
    lo[0] = amin0;
    hi[0] = amax0;
    top = 1;
    while (top > 0 && !P.err) {
        top--;
        double amin = lo[top], amax = hi[top];
        if (amax - amin > 3.141592653589793116) {
            const double amid = amin + (amax - amin) / 2.0;
            if (top + 2 > 24) {
                P.err = Z2D_ERR_INVALID_ARGUMENT;
                return;
            }
            // pushed in reverse of the order they are drawn
            if (forward) {
                lo[top] = amid, hi[top] = amax, top++;
                lo[top] = amin, hi[top] = amid, top++;
            } else {
                lo[top] = amin, hi[top] = amid, top++;
                lo[top] = amid, hi[top] = amax, top++;
            }
            continue;
        }
        if (amax != amin) {
            const double max_angle = arc_max_angle(tolerance / major_axis(P.tf, r), ok);
            int segments = (int)ceil(fabs(amax - amin) / max_angle);
            double step = (amax - amin) / (double)segments;
            segments -= 1;
            if (!forward) {
                const double t = amin;
                amin = amax;
                amax = t;
                step = -step;
            }
            const double c0 = zm::cos_(amin, ok), s0 = zm::sin_(amin, ok);
            if (ok) arc_line_to(P, xc + r * c0, yc + r * s0);
            for (int s = 0; s < segments && ok && !P.err; s++) {
                arc_segment(P, xc, yc, r, amin, amin + step, ok);
                amin += step;
            }
            if (ok && !P.err) arc_segment(P, xc, yc, r, amin, amax, ok);
        } else {
            const double c0 = zm::cos_(amin, ok), s0 = zm::sin_(amin, ok);
            if (ok) arc_line_to(P, xc + r * c0, yc + r * s0);
        }
        if (!ok) {
            P.err = Z2D_ERR_INVALID_ARGUMENT;  // an angle beyond 2^20 * pi/2
            return;
        }
    }
}

// Path.arc / arcNegative (Path.zig:345-405): angle2 brought past angle1 by
// whole turns first (bounded here: z2d would loop for ever on angles so far
// apart that adding 2 pi no longer changes them)
__device__ void path_arc(PathState &P, const double *v, bool negative) {
    const double xc = v[0], yc = v[1], r = v[2], a1 = v[3];
    double a2 = v[4];
    const double twopi = 6.283185307179586232;
    const double tol = P.tolerance > 0.001 ? P.tolerance : 0.001;
    int guard = 0;
    if (!negative) {
        while (a2 < a1) {
            a2 += twopi;
            if (++guard > (1 << 22)) {
                P.err = Z2D_ERR_INVALID_ARGUMENT;
                return;
            }
        }
        arc_in_direction(P, xc, yc, r, a1, a2, true, tol);
    } else {
        while (a2 > a1) {
            a2 -= twopi;
            if (++guard > (1 << 22)) {
                P.err = Z2D_ERR_INVALID_ARGUMENT;
                return;
            }
        }
        arc_in_direction(P, xc, yc, r, a2, a1, false, tol);
    }
}

// --------------------------------------------------------- glyph outlines
// Outline.quadCurveTo (Glyph.zig:845-869): the quadratic from the current
// point (mapped back to outline space) as a cubic
__device__ void outline_quad(PathState &O, int32_t qx, int32_t qy, int32_t tx, int32_t ty) {
    double x0, y0;
    if (!O.has_cur) {
        O.err = Z2D_ERR_INVALID_ARGUMENT;  // MalformedGlyph
        return;
    }
    if (!current_user(O, x0, y0)) return;
    const double x3 = (double)tx, y3 = (double)ty;
    const double x1 = x0 + 2.0 / 3.0 * ((double)qx - x0);
    const double y1 = y0 + 2.0 / 3.0 * ((double)qy - y0);
    const double x2 = x3 + 2.0 / 3.0 * ((double)qx - x3);
    const double y2 = y3 + 2.0 / 3.0 * ((double)qy - y3);
    path_curve_to(O, x1, y1, x2, y2, x3, y3);
}

// Outline.runOutline for a simple glyph (Glyph.zig:700-815): points with
// their on-curve flags and the contours' last point indices
__device__ void glyph_outline(PathState &P, const z2d_glyph_point *pts, int32_t n_pts, const uint16_t *ends,
                              int32_t n_ends, double units_per_em) {
    PathState O;
    const Tf id{1, 0, 0, 1, 0, 0};
    O.tf = tf_mul(tf_mul(id, Tf{1.0, 0, 0, -1.0, 0, 0}), Tf{1, 0, 0, 1, 0.0, units_per_em * -1.0});
    O.tolerance = P.tolerance;
    O.replay = &P;
    auto is_end = [&](int32_t i) {
        for (int32_t k = 0; k < n_ends; k++)
            if (ends[k] == i) return true;
        return false;
    };
    enum { MOVE, ON, OFF } state = MOVE;
    int32_t j = 0;
    for (int32_t i = 0; i < n_pts && !O.err && !P.err; i++) {
        const z2d_glyph_point &p = pts[i];
        const bool on = (p.flags & 1) != 0;
        switch (state) {
            case MOVE:
                if (!on || is_end(i)) continue;  // no usable start: dropped
                path_move_to(O, (double)p.x, (double)p.y);
                j = i;
                state = ON;
                break;
            case ON:
                if (!on) {
                    state = OFF;
                    break;
                }
                path_line_to(O, (double)p.x, (double)p.y);
                break;
            case OFF:
                if (on) {
                    outline_quad(O, pts[i - 1].x, pts[i - 1].y, p.x, p.y);
                    state = ON;
                    break;
                }
                // two off-curve points: the implied on-curve midpoint
                outline_quad(O, pts[i - 1].x, pts[i - 1].y, (int16_t)((p.x + pts[i - 1].x) >> 1),
                             (int16_t)((p.y + pts[i - 1].y) >> 1));
                break;
        }
        if (is_end(i)) {
            if (state == OFF) outline_quad(O, p.x, p.y, pts[j].x, pts[j].y);
            path_close(O);
            state = MOVE;
        }
    }
    if (O.err && !P.err) P.err = O.err;
}

struct BuildArgs {
    const z2d_path_program *progs;
    int64_t n_progs;
    const z2d_path_cmd *cmds;
    const z2d_glyph_point *gpts;
    int64_t n_gpts;
    const uint16_t *gends;
    int64_t n_gends;
    const unsigned long long *offsets;  // emit pass: each program's room in `nodes`
    z2d_node *nodes;
    unsigned long long *counts;  // count pass: nodes kept, then room needed (2 per program)
    int32_t *status;
};

__global__ void k_build_paths(const BuildArgs A) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.n_progs) return;
    const z2d_path_program &pg = A.progs[p];
    Sink sink{A.nodes ? A.nodes + A.offsets[p] : nullptr, 0, 0};
    PathState P;
    P.tf = Tf{pg.transformation[0], pg.transformation[1], pg.transformation[2], pg.transformation[3],
              pg.transformation[4], pg.transformation[5]};
    P.tolerance = pg.tolerance;
    P.sink = &sink;
    for (uint64_t k = 0; k < pg.n_cmds && !P.err; k++) {
        const z2d_path_cmd &c = A.cmds[pg.cmd_offset + k];
        const double *v = c.v;
        double ux, uy;
        switch (c.op) {
            case Z2D_PATH_MOVE_TO: path_move_to(P, v[0], v[1]); break;
            case Z2D_PATH_LINE_TO: path_line_to(P, v[0], v[1]); break;
            case Z2D_PATH_CURVE_TO: path_curve_to(P, v[0], v[1], v[2], v[3], v[4], v[5]); break;
            case Z2D_PATH_REL_MOVE_TO:
                if (current_user(P, ux, uy)) path_move_to(P, ux + v[0], uy + v[1]);
                break;
            case Z2D_PATH_REL_LINE_TO:
                if (current_user(P, ux, uy)) path_line_to(P, ux + v[0], uy + v[1]);
                break;
            case Z2D_PATH_REL_CURVE_TO:
                if (current_user(P, ux, uy))
                    path_curve_to(P, ux + v[0], uy + v[1], ux + v[2], uy + v[3], ux + v[4], uy + v[5]);
                break;
            case Z2D_PATH_ARC: path_arc(P, v, false); break;
            case Z2D_PATH_ARC_NEGATIVE: path_arc(P, v, true); break;
            case Z2D_PATH_CLOSE: path_close(P); break;
            case Z2D_PATH_SET_TRANSFORMATION: P.tf = Tf{v[0], v[1], v[2], v[3], v[4], v[5]}; break;
            case Z2D_PATH_SET_TOLERANCE: P.tolerance = v[0]; break;
            case Z2D_PATH_RESET:  // Path.reset: the nodes and the state are cleared
                sink.n = 0;
                P.has_cur = P.has_init = false;
                P.last_tag = -1;
                break;
            case Z2D_PATH_GLYPH: {
                const int64_t po = (int64_t)v[0], np = (int64_t)v[1], eo = (int64_t)v[2], ne = (int64_t)v[3];
                if (po < 0 || np < 0 || eo < 0 || ne < 0 || po + np > A.n_gpts || eo + ne > A.n_gends ||
                    np > 0xFFFF || ne > 0xFFFF) {
                    P.err = Z2D_ERR_INVALID_ARGUMENT;
                    break;
                }
                // the outline is built whole before it is appended: on an
                // error nothing of it reaches the path
                const PathState saved = P;
                const long long saved_n = sink.n;
                glyph_outline(P, A.gpts + po, (int32_t)np, A.gends + eo, (int32_t)ne, v[4]);
                if (P.err) {
                    const int e = P.err;
                    P = saved;
                    sink.n = saved_n;
                    P.err = e;
                }
                break;
            }
            default: P.err = Z2D_ERR_INVALID_ARGUMENT; break;
        }
    }
    if (A.counts) {
        A.counts[2 * p] = (unsigned long long)sink.n;
        A.counts[2 * p + 1] = (unsigned long long)sink.hw;
    }
    if (A.status) A.status[p] = P.err;
}

// Programs whose room exceeded their kept nodes: their nodes move from the
// room layout to the packed one (one CTA per program).
__global__ void k_pack_nodes(const unsigned long long *__restrict__ room, const unsigned long long *__restrict__ out_off,
                             int64_t n_progs, const z2d_node *__restrict__ src, z2d_node *__restrict__ dst) {
    for (int64_t p = blockIdx.x; p < n_progs; p += gridDim.x) {
        const unsigned long long s = room[p], d = out_off[p], n = out_off[p + 1] - out_off[p];
        for (unsigned long long k = threadIdx.x; k < n; k += blockDim.x) dst[d + k] = src[s + k];
    }
}

}  // namespace

int build_paths(Ctx &c, const z2d_path_program *progs, size_t n_progs, const z2d_path_cmd *cmds, size_t n_cmds,
                const z2d_glyph_point *gpts, size_t n_gpts, const uint16_t *gends, size_t n_gends, z2d_node *nodes,
                size_t cap_nodes, uint64_t *offsets, int32_t *status) {
    if ((n_progs > 0 && (!progs || !offsets)) || (n_cmds > 0 && !cmds) || (n_gpts > 0 && !gpts) ||
        (n_gends > 0 && !gends) || (cap_nodes > 0 && !nodes))
        return Z2D_ERR_INVALID_ARGUMENT;
    if (n_progs == 0) {
        if (offsets) offsets[0] = 0;
        return Z2D_OK;
    }
    for (size_t p = 0; p < n_progs; p++)
        if (progs[p].cmd_offset > n_cmds || progs[p].n_cmds > n_cmds - progs[p].cmd_offset) {
            set_error("build_paths: program commands outside the command array");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t o_progs = 0, o_cmds = al(sizeof(z2d_path_program) * n_progs);
    const size_t o_gpts = o_cmds + al(sizeof(z2d_path_cmd) * n_cmds);
    const size_t o_gends = o_gpts + al(sizeof(z2d_glyph_point) * n_gpts);
    const size_t o_cnt = o_gends + al(sizeof(uint16_t) * n_gends);
    const size_t o_room = o_cnt + al(sizeof(unsigned long long) * 2 * n_progs);
    const size_t o_out = o_room + al(sizeof(unsigned long long) * (n_progs + 1));
    const size_t o_st = o_out + al(sizeof(unsigned long long) * (n_progs + 1));
    const size_t in_bytes = o_cnt;
    const size_t total = o_st + al(sizeof(int32_t) * n_progs);
    if (c.params.ensure(total) || c.staging.ensure(std::max(in_bytes, sizeof(unsigned long long) * 2 * (n_progs + 1)) + 16))
        return Z2D_ERR_OUT_OF_MEMORY;
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    uint8_t *h = c.staging.as<uint8_t>(), *dv = c.params.as<uint8_t>();
    memcpy(h + o_progs, progs, sizeof(z2d_path_program) * n_progs);
    if (n_cmds) memcpy(h + o_cmds, cmds, sizeof(z2d_path_cmd) * n_cmds);
    if (n_gpts) memcpy(h + o_gpts, gpts, sizeof(z2d_glyph_point) * n_gpts);
    if (n_gends) memcpy(h + o_gends, gends, sizeof(uint16_t) * n_gends);
    Z2D_CUDA(cudaMemcpyAsync(dv, h, in_bytes, cudaMemcpyHostToDevice, c.stream));
    BuildArgs A;
    A.progs = reinterpret_cast<const z2d_path_program *>(dv + o_progs);
    A.n_progs = (int64_t)n_progs;
    A.cmds = reinterpret_cast<const z2d_path_cmd *>(dv + o_cmds);
    A.gpts = reinterpret_cast<const z2d_glyph_point *>(dv + o_gpts);
    A.n_gpts = (int64_t)n_gpts;
    A.gends = reinterpret_cast<const uint16_t *>(dv + o_gends);
    A.n_gends = (int64_t)n_gends;
    unsigned long long *d_cnt = reinterpret_cast<unsigned long long *>(dv + o_cnt);
    unsigned long long *d_room = reinterpret_cast<unsigned long long *>(dv + o_room);
    unsigned long long *d_out = reinterpret_cast<unsigned long long *>(dv + o_out);
    int32_t *d_st = reinterpret_cast<int32_t *>(dv + o_st);
    const unsigned blocks = (unsigned)((n_progs + 127) / 128);
    // count pass: nodes kept and room needed per program
    A.offsets = nullptr;
    A.nodes = nullptr;
    A.counts = d_cnt;
    A.status = d_st;
    k_build_paths<<<blocks, 128, 0, c.stream>>>(A);
    c.launches++;
    std::vector<unsigned long long> cnt(2 * n_progs), room(n_progs + 1);
    Z2D_CUDA(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(unsigned long long) * 2 * n_progs, cudaMemcpyDeviceToHost,
                             c.stream));
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    unsigned long long tot = 0, rtot = 0;
    bool packed = true;
    for (size_t p = 0; p < n_progs; p++) {
        offsets[p] = tot;
        room[p] = rtot;
        tot += cnt[2 * p];
        rtot += cnt[2 * p + 1];
        packed = packed && cnt[2 * p] == cnt[2 * p + 1];
    }
    offsets[n_progs] = tot;
    room[n_progs] = rtot;
    if (tot > cap_nodes) {
        set_error("build_paths: the node array holds fewer nodes than the programs build (offsets are filled)");
        return Z2D_ERR_OUT_OF_MEMORY;
    }
    // emit pass into device scratch laid out by room, packed when a reset or
    // a rolled-back glyph left a program with fewer nodes than its room,
    // then to the caller
    const size_t scratch = (size_t)std::max<unsigned long long>(rtot, 1) + (packed ? 0 : (size_t)std::max<unsigned long long>(tot, 1));
    if (c.edges.ensure(sizeof(z2d_node) * scratch)) return Z2D_ERR_OUT_OF_MEMORY;
    memcpy(h, room.data(), sizeof(unsigned long long) * (n_progs + 1));
    memcpy(h + sizeof(unsigned long long) * (n_progs + 1), offsets, sizeof(unsigned long long) * (n_progs + 1));
    Z2D_CUDA(cudaMemcpyAsync(d_room, h, sizeof(unsigned long long) * (n_progs + 1), cudaMemcpyHostToDevice, c.stream));
    Z2D_CUDA(cudaMemcpyAsync(d_out, h + sizeof(unsigned long long) * (n_progs + 1),
                             sizeof(unsigned long long) * (n_progs + 1), cudaMemcpyHostToDevice, c.stream));
    A.offsets = d_room;
    A.nodes = c.edges.as<z2d_node>();
    A.counts = nullptr;
    k_build_paths<<<blocks, 128, 0, c.stream>>>(A);
    c.launches++;
    z2d_node *result = A.nodes;
    if (!packed) {
        result = A.nodes + std::max<unsigned long long>(rtot, 1);
        const unsigned pb = (unsigned)std::min<size_t>(n_progs, (size_t)c.sm_count * 16);
        k_pack_nodes<<<pb, 128, 0, c.stream>>>(d_room, d_out, (int64_t)n_progs, A.nodes, result);
        c.launches++;
    }
    Z2D_CUDA(cudaGetLastError());
    if (tot) Z2D_CUDA(cudaMemcpyAsync(nodes, result, sizeof(z2d_node) * (size_t)tot, cudaMemcpyDefault, c.stream));
    if (status) Z2D_CUDA(cudaMemcpyAsync(status, d_st, sizeof(int32_t) * n_progs, cudaMemcpyDeviceToHost, c.stream));
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    return Z2D_OK;
}

}  // namespace z2dg
