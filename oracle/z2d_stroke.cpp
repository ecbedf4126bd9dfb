// z2d_stroke.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// The oracle's own restatement of z2d's stroke tessellation, written from
// the reference's Zig sources (paths inside the z2d project) independently
// of the library's stroke builders, so that stroke parity tests compare the
// library with something other than itself:
//   painter.stroke option handling      src/painter.zig:214-344
//   stroke_plotter (solid strokes)      src/internal/tess/stroke_plotter.zig:40-575
//   dashed_plotter                      src/internal/tess/dashed_plotter.zig:30-470
//   polyline_plotter (hairlines)        src/internal/tess/polyline_plotter.zig:22-221
//   Face, Pen, Slope, Dasher            src/internal/tess/{Face,Pen,Slope,Dasher}.zig
//   PointBuffer                         src/internal/tess/point_buffer.zig:14-60
//   Polygon.Contour / addEdgesFromContour src/internal/tess/Polygon.zig:115-137, 359-430
//   Spline.decompose                    src/internal/tess/Spline.zig:37-165
//   arc.transformed_circle_major_axis   src/internal/arc.zig:92-262
//   Transformation (inverse, distances)  src/Transformation.zig:50-212
// Operation order follows the Zig code so that every coordinate rounds the
// same.  Shared with the library by necessity, not by code: the pen's cos,
// sin and acos come from the host libm (z2d calls Zig's std.math versions),
// and hypot is sqrt(x*x + y*y) in f64 (Zig's std.math.hypot is not in the
// reference tree); the stroke goldens pin both choices.
//
// Export: z2doracle_stroke_contours, the closed contours (or, for hairlines,
// the open polylines) painter.stroke would rasterise, in the library's
// z2dgpu_stroke_contours layout.
#include "../include/z2dgpu.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <iterator>
#include <list>
#include <vector>

namespace {

struct P {
    double x, y;
};
bool same(P a, P b) { return a.x == b.x && a.y == b.y; }

// ---------------------------------------------------------- Transformation
struct Tf {
    double ax = 1, by = 0, cx = 0, dy = 1, tx = 0, ty = 0;
    bool identity() const { return ax == 1 && by == 0 && cx == 0 && dy == 1 && tx == 0 && ty == 0; }
    double det() const { return ax * dy - by * cx; }
    // Transformation.inverse (Transformation.zig:103-161)
    bool inverse(Tf &o) const {
        if (by == 0 && cx == 0) {
            if (ax == 0 || dy == 0) return false;
            if (ax != 1 || dy != 1) {
                o = Tf{1 / ax, 0, 0, 1 / dy, -tx / ax, -ty / dy};
            } else {
                o = Tf{1, 0, 0, 1, -tx, -ty};
            }
            return true;
        }
        const double d = det();
        if (d == 0) return false;
        const double s = 1 / d;
        o = Tf{dy * s, -by * s, -cx * s, ax * s, (by * ty - dy * tx) * s, (cx * tx - ax * ty) * s};
        return true;
    }
    void to_device_dist(double &x, double &y) const {  // userToDeviceDistance
        const double ix = x, iy = y;
        x = ax * ix + by * iy;
        y = cx * ix + dy * iy;
    }
    void to_user_dist(double &x, double &y) const {  // deviceToUserDistance (ctm pre-validated)
        Tf inv;
        inverse(inv);
        inv.to_device_dist(x, y);
    }
};

double hyp(double x, double y) { return std::sqrt(x * x + y * y); }

// ------------------------------------------------------------------ Slope
struct Slope {
    double dx = 0, dy = 0;
    static Slope of(P a, P b) { return Slope{b.x - a.x, b.y - a.y}; }
    double normalize() {  // Slope.normalize
        double rx, ry, mag;
        if (dx == 0.0) {
            rx = 0.0;
            if (dy > 0.0) {
                mag = dy;
                ry = 1.0;
            } else {
                mag = -dy;
                ry = -1.0;
            }
        } else if (dy == 0.0) {
            ry = 0.0;
            if (dx > 0.0) {
                mag = dx;
                rx = 1.0;
            } else {
                mag = -dx;
                rx = -1.0;
            }
        } else {
            mag = hyp(dx, dy);
            rx = dx / mag;
            ry = dy / mag;
        }
        dx = rx;
        dy = ry;
        return mag;
    }
    Slope normalized() const {
        Slope s = *this;
        s.normalize();
        return s;
    }
};
int sgn(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }
// Slope.compare: b's components are replaced by a's where they differ by
// no more than f64 epsilon
int cmp(Slope a, Slope b) {
    const double eps = 2.220446049250313e-16;
    const double bdy = std::fabs(b.dy - a.dy) > eps ? b.dy : a.dy;
    const double bdx = std::fabs(b.dx - a.dx) > eps ? b.dx : a.dx;
    const int c = sgn(a.dy * bdx - bdy * a.dx);
    if (c != 0) return c;
    if (a.dx == 0 && a.dy == 0 && bdx == 0 && bdy == 0) return 0;
    if (a.dx == 0 && a.dy == 0) return 1;
    if (bdx == 0 && bdy == 0) return -1;
    if (sgn(a.dx) != sgn(bdx) || sgn(a.dy) != sgn(bdy)) return (a.dx > 0 || (a.dx == 0 && a.dy > 0)) ? -1 : 1;
    return 0;
}
bool miter_ok(Slope in, Slope out, double limit) {  // Slope.compare_for_miter_limit
    const Slope a = in.normalized(), b = out.normalized();
    const double dot = a.dx * b.dx + a.dy * b.dy;
    return 2 <= limit * limit * (1 + dot);
}

// ---------------------------------------------------------------- Contour
// A polygon contour: points scaled as they are plotted; std::list keeps the
// positions `before` refers to valid while points are inserted.
struct Contour {
    std::list<P> pts;
    double scale = 1;
    using It = std::list<P>::iterator;
    void plot(P p, It before) { pts.insert(before, P{p.x * scale, p.y * scale}); }
    void append(P p) { pts.push_back(P{p.x * scale, p.y * scale}); }
    void prepend(P p) { pts.push_front(P{p.x * scale, p.y * scale}); }
};
using Contours = std::vector<std::vector<P>>;
void emit(Contours &out, const Contour &c) {  // Polygon.addEdgesFromContour: the closed ring of the corners
    if (c.pts.empty()) return;
    out.emplace_back(c.pts.begin(), c.pts.end());
}

// --------------------------------------------------------------------- Pen
struct PenVertex {
    P pt;
    Slope cw, ccw;
};
struct Pen {
    std::vector<PenVertex> v;
};
// arc.transformed_circle_major_axis (arc.zig:92-262)
double major_axis(const Tf &m, double radius) {
    const double eps = 0.00390625;
    const double det = m.ax * m.dy - m.by * m.cx;
    if (std::fabs(det * det - 1.0) < eps) {
        if (std::fabs(m.by) < eps && std::fabs(m.cx) < eps) return radius;
        if (std::fabs(m.ax) < eps && std::fabs(m.dy) < eps) return radius;
    }
    const double i = m.ax * m.ax + m.by * m.by, j = m.cx * m.cx + m.dy * m.dy;
    const double f = 0.5 * (i + j), g = 0.5 * (i - j), h = m.ax * m.cx + m.by * m.dy;
    return radius * std::sqrt(f + hyp(g, h));
}
Pen make_pen(double thickness, double tol, const Tf &ctm) {  // Pen.init
    const double radius = thickness / 2;
    int n;
    const double axis = major_axis(ctm, radius);
    if (tol >= axis * 4) n = 1;
    else if (tol >= axis) n = 4;
    else {
        const double delta = std::acos(1 - tol / axis);
        if (delta == 0) n = 4;
        else {
            const int k = (int)std::ceil(2 * M_PI / delta);
            n = k < 4 ? 4 : (k % 2 != 0 ? k + 1 : k);
        }
    }
    Pen pen;
    const bool reflect = ctm.det() < 0;
    for (int i = 0; i < n; i++) {
        double t = 2 * M_PI * (double)i / (double)n;
        if (reflect) t = -t;
        double dx = radius * std::cos(t), dy = radius * std::sin(t);
        ctm.to_device_dist(dx, dy);
        pen.v.push_back(PenVertex{P{dx, dy}, Slope{}, Slope{}});
    }
    for (int i = 0; i < n; i++) {
        const int next = i >= n - 1 ? 0 : i + 1, prev = i == 0 ? n - 1 : i - 1;
        pen.v[i].cw = Slope::of(pen.v[prev].pt, pen.v[i].pt);
        pen.v[i].ccw = Slope::of(pen.v[i].pt, pen.v[next].pt);
    }
    return pen;
}
// Pen.vertexIteratorFor: the vertex indices from `from` to `to`, in order
std::vector<int> pen_arc(const Pen &pen, Slope from, Slope to, bool clockwise) {
    const int n = (int)pen.v.size();
    int start, end, i, lo, hi;
    if (clockwise) {
        lo = 0;
        hi = n;
        for (i = (lo + hi) >> 1; hi - lo > 1; i = (lo + hi) >> 1) {
            if (cmp(pen.v[i].cw, from) < 0) lo = i;
            else hi = i;
        }
        if (cmp(pen.v[i].cw, from) < 0 && ++i == n) i = 0;
        start = i;
        if (cmp(to, pen.v[i].ccw) >= 0) {
            lo = i;
            hi = i + n;
            for (i = (lo + hi) >> 1; hi - lo > 1; i = (lo + hi) >> 1) {
                const int j = i >= n ? i - n : i;
                if (cmp(pen.v[j].cw, to) > 0) hi = i;
                else lo = i;
            }
            if (i >= n) i -= n;
        }
        end = i;
    } else {
        lo = 0;
        hi = n;
        for (i = (lo + hi) >> 1; hi - lo > 1; i = (lo + hi) >> 1) {
            if (cmp(from, pen.v[i].ccw) < 0) lo = i;
            else hi = i;
        }
        if (cmp(from, pen.v[i].ccw) < 0 && ++i == n) i = 0;
        start = i;
        if (cmp(pen.v[i].cw, to) <= 0) {
            lo = i;
            hi = i + n;
            for (i = (lo + hi) >> 1; hi - lo > 1; i = (lo + hi) >> 1) {
                const int j = i >= n ? i - n : i;
                if (cmp(to, pen.v[j].ccw) > 0) hi = i;
                else lo = i;
            }
            if (i >= n) i -= n;
        }
        end = i;
    }
    std::vector<int> out;
    for (int k = start < 0 ? 0 : start, e = end < 0 ? 0 : end; k != e;) {
        out.push_back(k);
        if (clockwise) {
            if (++k == n) k = 0;
        } else {
            if (k == 0) k = n;
            k--;
        }
    }
    return out;
}

// -------------------------------------------------------------------- Face
struct Face {
    P p0, p1;
    double width, half;
    Slope dev, user;
    P p0_cw, p0_ccw, p1_cw, p1_ccw;
    Tf ctm;
};
Face face_with(P p0, P p1, Slope dev, double thickness, const Tf &ctm) {  // Face._init
    Face f;
    f.p0 = p0;
    f.p1 = p1;
    f.width = thickness;
    f.half = thickness / 2;
    f.dev = dev;
    f.user = dev;
    f.ctm = ctm;
    double ox, oy;
    if (!ctm.identity()) {
        double dx = dev.dx, dy = dev.dy;
        ctm.to_user_dist(dx, dy);
        f.user = Slope{dx, dy}.normalized();
        if (ctm.det() >= 0) {
            ox = -f.user.dy * f.half;
            oy = f.user.dx * f.half;
        } else {
            ox = f.user.dy * f.half;
            oy = -f.user.dx * f.half;
        }
        ctm.to_device_dist(ox, oy);
    } else {
        ox = -dev.dy * f.half;
        oy = dev.dx * f.half;
    }
    f.p0_cw = P{p0.x + ox, p0.y + oy};
    f.p0_ccw = P{p0.x + -ox, p0.y + -oy};
    f.p1_cw = P{p1.x + ox, p1.y + oy};
    f.p1_ccw = P{p1.x + -ox, p1.y + -oy};
    return f;
}
Face face(P p0, P p1, double thickness, const Tf &ctm) {
    return face_with(p0, p1, Slope::of(p0, p1).normalized(), thickness, ctm);
}
P intersect(const Face &in, const Face &out, bool clockwise) {  // Face.intersect
    const P ip = clockwise ? in.p1_ccw : in.p1_cw, op = clockwise ? out.p0_ccw : out.p0_cw;
    const Slope a = in.dev.normalized(), b = out.dev.normalized();
    const double y = ((op.x - ip.x) * a.dy * b.dy - op.y * b.dx * a.dy + ip.y * a.dx * b.dy) / (a.dx * b.dy - b.dx * a.dy);
    const double x = std::fabs(a.dy) >= std::fabs(b.dy) ? (y - ip.y) * a.dx / a.dy + ip.x : (y - op.y) * b.dx / b.dy + op.x;
    return P{x, y};
}
// Face.cap on the face's p1 end, each point through `sink`
template <class Sink>
void cap(const Face &f, int mode, bool clockwise, const Pen *pen, Sink &&sink) {
    if (mode == Z2D_CAP_BUTT) {
        sink(clockwise ? f.p1_ccw : f.p1_cw);
        sink(clockwise ? f.p1_cw : f.p1_ccw);
    } else if (mode == Z2D_CAP_SQUARE) {
        double ox = f.user.dx * f.half, oy = f.user.dy * f.half;
        f.ctm.to_device_dist(ox, oy);
        const P a = clockwise ? f.p1_ccw : f.p1_cw, b = clockwise ? f.p1_cw : f.p1_ccw;
        sink(a);
        sink(P{a.x + ox, a.y + oy});
        sink(P{b.x + ox, b.y + oy});
        sink(b);
    } else {
        sink(clockwise ? f.p1_ccw : f.p1_cw);
        for (int k : pen_arc(*pen, f.dev, Slope{-f.dev.dx, -f.dev.dy}, clockwise))
            sink(P{f.p1.x + pen->v[k].pt.x, f.p1.y + pen->v[k].pt.y});
        sink(clockwise ? f.p1_cw : f.p1_ccw);
    }
}
template <class Sink>
void cap_p0(const Face &f, int mode, bool clockwise, const Pen *pen, Sink &&sink) {
    cap(face(f.p1, f.p0, f.width, f.ctm), mode, clockwise, pen, sink);
}

// ------------------------------------------------------------ PointBuffer
template <size_t SPLIT, size_t LEN>
struct PointBuffer {
    P items[LEN];
    size_t len = 0;
    void add(P p) {
        if (len < LEN) {
            items[len++] = p;
        } else {
            for (size_t i = SPLIT; i < LEN - 1; i++) items[i] = items[i + 1];
            items[LEN - 1] = p;
        }
    }
    P head(size_t n) const { return items[n]; }
    P tail(size_t n) const { return items[len - n]; }
    P last() const { return items[len - 1]; }
    P first() const { return items[0]; }
};

// ----------------------------------------------------------------- Spline
struct Knots {
    P a, b, c, d;
};
double error_sq(const Knots &k) {  // Spline.Knots.errorSq
    double bx = k.b.x - k.a.x, by = k.b.y - k.a.y;
    double cx = k.c.x - k.a.x, cy = k.c.y - k.a.y;
    if (k.a.x != k.d.x || k.a.y != k.d.y) {
        const double dx = k.d.x - k.a.x, dy = k.d.y - k.a.y;
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
P half(P a, P b) { return P{a.x + ((b.x - a.x) / 2), a.y + ((b.y - a.y) / 2)}; }
template <class F>
void decompose_into(Knots s1, P start, double tol2, F &line_to, int depth) {
    if (error_sq(s1) < tol2 || depth > 64) {
        if (!same(s1.a, start)) line_to(s1.a);
        return;
    }
    const P ab = half(s1.a, s1.b), bc = half(s1.b, s1.c), cd = half(s1.c, s1.d);
    const P abbc = half(ab, bc), bccd = half(bc, cd), fin = half(abbc, bccd);
    const Knots s2{fin, bccd, cd, s1.d};
    decompose_into(Knots{s1.a, ab, abbc, fin}, start, tol2, line_to, depth + 1);
    decompose_into(s2, start, tol2, line_to, depth + 1);
}
template <class F>
void spline(P a, P b, P c, P d, double tol, F &&line_to) {  // Spline.decompose
    if (same(a, b) && same(c, d)) {
        line_to(d);
        return;
    }
    decompose_into(Knots{a, b, c, d}, a, tol * tol, line_to, 0);
    line_to(d);
}

// --------------------------------------------------------------- plotting
struct Opts {
    int cap, join;
    Tf ctm;
    std::vector<double> dashes;
    double dash_offset, miter_limit, scale, thickness, tolerance;
};

// The state the shared plotting routines of stroke_plotter.zig act on
// (join, plotSingle, plotOpenJoined, plotClosedJoined are generic over it):
// the contours in progress, the direction of the first join, the result.
struct State {
    const Opts *o = nullptr;
    const Pen *pen = nullptr;
    PointBuffer<2, 5> points;
    int cw = -1;  // clockwise_: -1 unset, 0 false, 1 true
    Contours *result = nullptr;
    Contour outer, inner;
    Slope current_slope;
    void reset_contours() {
        outer = Contour{{}, o->scale};
        inner = Contour{{}, o->scale};
    }
};

void join(State &s, int mode, P p0, P p1, P p2, bool before_first) {  // stroke_plotter.join
    if (same(p0, p1) || same(p1, p2)) {
        if (s.cw < 0) s.cw = 0;
        return;
    }
    const Opts &o = *s.o;
    const Face in = face(p0, p1, o.thickness, o.ctm), out = face(p1, p2, o.thickness, o.ctm);
    const bool jcw = cmp(in.dev, out.dev) < 0;
    const bool pcw = s.cw >= 0 ? s.cw != 0 : jcw;
    const bool switched = jcw != pcw;
    // where a point of the join's outer / inner side goes
    const Contour::It before = before_first ? s.outer.pts.begin() : s.outer.pts.end();
    auto to_outer = [&](P p) { s.outer.plot(p, before); };
    auto to_inner = [&](P p) { s.inner.prepend(p); };
    auto outer_side = [&](P p) {
        if (switched) to_inner(p);
        else to_outer(p);
    };
    auto inner_side = [&](P p) {
        if (switched) to_outer(p);
        else to_inner(p);
    };
    if (cmp(in.dev, out.dev) == 0) {
        outer_side(jcw ? in.p1_ccw : in.p1_cw);
        inner_side(jcw ? in.p1_cw : in.p1_ccw);
        if (s.cw < 0) s.cw = pcw;
        return;
    }
    if (mode == Z2D_JOIN_MITER || mode == Z2D_JOIN_BEVEL) {
        if (mode == Z2D_JOIN_MITER && miter_ok(in.dev, out.dev, o.miter_limit)) {
            outer_side(intersect(in, out, jcw));
        } else {
            outer_side(jcw ? in.p1_ccw : in.p1_cw);
            outer_side(jcw ? out.p0_ccw : out.p0_cw);
        }
    } else {
        outer_side(jcw ? in.p1_ccw : in.p1_cw);
        for (int k : pen_arc(*s.pen, in.dev, out.dev, jcw))
            outer_side(P{p1.x + s.pen->v[k].pt.x, p1.y + s.pen->v[k].pt.y});
        outer_side(jcw ? out.p0_ccw : out.p0_cw);
    }
    inner_side(jcw ? in.p1_cw : in.p1_ccw);
    inner_side(p1);
    inner_side(jcw ? out.p0_cw : out.p0_ccw);
    if (s.cw < 0) s.cw = pcw;
}

void plot_single(State &s, P start, P end) {  // stroke_plotter.plotSingle
    const Face f = face(start, end, s.o->thickness, s.o->ctm);
    auto sink = [&](P p) { s.outer.append(p); };
    cap_p0(f, s.o->cap, true, s.pen, sink);
    cap(f, s.o->cap, true, s.pen, sink);
    emit(*s.result, s.outer);
    s.outer = Contour{{}, s.o->scale};
    s.cw = -1;
}

void plot_open_joined(State &s, P start0, P end0, P start1, P end1) {  // stroke_plotter.plotOpenJoined
    const Face fs = face(start0, end0, s.o->thickness, s.o->ctm), fe = face(start1, end1, s.o->thickness, s.o->ctm);
    const bool clockwise = s.cw >= 0 ? s.cw != 0 : true;
    const Contour::It first = s.outer.pts.begin();
    cap_p0(fs, s.o->cap, clockwise, s.pen, [&](P p) { s.outer.plot(p, first); });
    cap(fe, s.o->cap, clockwise, s.pen, [&](P p) { s.outer.append(p); });
    s.outer.pts.splice(s.outer.pts.end(), s.inner.pts);
    emit(*s.result, s.outer);
    s.reset_contours();
    s.cw = -1;
}

void plot_closed_joined(State &s, P i0, P i1, P p1, P p2) {  // stroke_plotter.plotClosedJoined
    if (!same(p2, i0)) {
        join(s, s.o->join, p1, p2, i0, false);
        join(s, s.o->join, p2, i0, i1, false);
    } else {
        join(s, s.o->join, p1, i0, i1, false);
    }
    emit(*s.result, s.outer);
    emit(*s.result, s.inner);
    s.reset_contours();
    s.cw = -1;
}

// stroke_plotter.Plotter (solid strokes)
struct Solid : State {
    int run(const z2d_node *nodes, size_t n) {
        for (size_t i = 0; i < n; i++) {
            const z2d_node &nd = nodes[i];
            switch (nd.tag) {
                case Z2D_MOVE_TO:
                    if (points.len > 0) finish();
                    points.len = 0;
                    points.add(P{nd.p[0], nd.p[1]});
                    break;
                case Z2D_LINE_TO:
                    if (points.len == 0) return Z2D_ERR_INVALID_STATE;
                    line_to(o->join, P{nd.p[0], nd.p[1]});
                    break;
                case Z2D_CURVE_TO:
                    if (points.len == 0) return Z2D_ERR_INVALID_STATE;
                    spline(points.last(), P{nd.p[0], nd.p[1]}, P{nd.p[2], nd.p[3]}, P{nd.p[4], nd.p[5]}, o->tolerance,
                           [&](P p) { line_to(Z2D_JOIN_ROUND, p); });
                    break;
                case Z2D_CLOSE_PATH:
                    close();
                    break;
                default: return Z2D_ERR_INVALID_ARGUMENT;
            }
        }
        finish();
        return Z2D_OK;
    }
    void line_to(int mode, P p) {
        if (same(p, points.last())) return;
        points.add(p);
        if (points.len > 2) join(*this, mode, points.tail(3), points.tail(2), points.tail(1), false);
    }
    void close() {
        if (points.len == 1) dotted(points.first());
        else if (points.len == 2) plot_single(*this, points.head(0), points.head(1));
        else if (points.len > 2) plot_closed_joined(*this, points.head(0), points.head(1), points.tail(2), points.tail(1));
        points.len = 0;
    }
    void finish() {
        if (points.len == 2) plot_single(*this, points.head(0), points.head(1));
        else if (points.len > 2) plot_open_joined(*this, points.head(0), points.head(1), points.tail(2), points.tail(1));
    }
    void dotted(P p) {  // Plotter.plotDotted: round caps draw the pen around the point
        if (o->cap != Z2D_CAP_ROUND) return;
        for (const PenVertex &v : pen->v) outer.append(P{p.x + v.pt.x, p.y + v.pt.y});
        emit(*result, outer);
        outer = Contour{{}, o->scale};
        cw = -1;
    }
};

// Dasher.zig
struct Dasher {
    const std::vector<double> *d = nullptr;
    double offset = 0, remain = 0;
    size_t idx = 0;
    bool on = true;
    static bool valid(const std::vector<double> &v) {
        bool ok = false;
        for (double x : v) {
            if (x < 0) return false;
            if (x > 0) ok = true;
        }
        return ok;
    }
    void reset() {
        idx = 0;
        on = true;
        remain = (*d)[0];
        remain -= offset;
        while (remain < 0 || remain > (*d)[idx]) {
            if (remain < 0) {
                remain += (*d)[idx];
                idx = idx >= d->size() - 1 ? 0 : idx + 1;
            } else {
                remain -= (*d)[idx];
                idx = idx == 0 ? d->size() - 1 : idx - 1;
            }
            on = !on;
        }
    }
    bool step(double len) {
        remain -= len;
        if (remain <= 0) {
            on = !on;
            if (++idx >= d->size()) idx = 0;
            remain = (*d)[idx];
            return true;
        }
        return false;
    }
};

// dashed_plotter.Plotter
struct Dashed : State {
    Dasher dasher;
    enum { NONE, OFF, ON } initial = NONE;
    P initial_off{0, 0};
    State init_poly;  // the first dash of the subpath, kept open until the path closes or ends

    int run(const z2d_node *nodes, size_t n) {
        for (size_t i = 0; i < n; i++) {
            const z2d_node &nd = nodes[i];
            int rc = Z2D_OK;
            switch (nd.tag) {
                case Z2D_MOVE_TO:
                    rc = finish();
                    dasher.reset();
                    points.len = 0;
                    points.add(P{nd.p[0], nd.p[1]});
                    break;
                case Z2D_LINE_TO:
                    if (points.len == 0) return Z2D_ERR_INVALID_STATE;
                    line_to(o->join, P{nd.p[0], nd.p[1]});
                    break;
                case Z2D_CURVE_TO:
                    if (points.len == 0) return Z2D_ERR_INVALID_STATE;
                    spline(points.last(), P{nd.p[0], nd.p[1]}, P{nd.p[2], nd.p[3]}, P{nd.p[4], nd.p[5]}, o->tolerance,
                           [&](P p) { line_to(Z2D_JOIN_ROUND, p); });
                    break;
                case Z2D_CLOSE_PATH: rc = close(); break;
                default: return Z2D_ERR_INVALID_ARGUMENT;
            }
            if (rc) return rc;
        }
        return finish();
    }

    void line_to(int mode, P p) {
        const P first = points.last();
        if (same(p, first)) return;
        Slope slope = Slope::of(first, p);
        current_slope = slope.normalized();
        o->ctm.to_user_dist(slope.dx, slope.dy);
        const double total = slope.normalize();
        double remaining = total;
        double step = dasher.remain < remaining ? dasher.remain : remaining;
        while (remaining > 0) {
            remaining -= step;
            double xo = slope.dx * (total - remaining), yo = slope.dy * (total - remaining);
            o->ctm.to_device_dist(xo, yo);
            const P cur{first.x + xo, first.y + yo};
            if (!same(cur, points.last())) points.add(cur);
            if (dasher.on && points.len > 2) join(*this, mode, points.tail(3), points.tail(2), points.tail(1), false);
            if (dasher.step(step)) next_segment(cur);
            step = dasher.remain < remaining ? dasher.remain : remaining;
        }
    }

    void next_segment(P p) {
        if (initial == NONE) {
            save_initial();
        } else if (!dasher.on) {
            open_end(*this);
        }
        points.len = 0;
        points.add(p);
    }

    // the end of an open piece: a dot, a single segment or a joined polyline
    void open_end(State &st) {
        if (st.points.len == 1) dotted(st, st.points.first(), st.current_slope);
        else if (st.points.len == 2) plot_single(st, st.points.head(0), st.points.head(1));
        else if (st.points.len > 2)
            plot_open_joined(st, st.points.head(0), st.points.head(1), st.points.tail(2), st.points.tail(1));
    }

    void save_initial() {
        if (!dasher.on) {
            init_poly.o = o;
            init_poly.pen = pen;
            init_poly.points = points;
            init_poly.cw = cw;
            init_poly.result = result;
            init_poly.outer = std::move(outer);
            init_poly.inner = std::move(inner);
            init_poly.current_slope = current_slope;
            initial = ON;
        } else {
            initial_off = points.first();
            initial = OFF;
        }
        reset_contours();
        cw = -1;
    }

    int close() {
        if (points.len == 0) return Z2D_ERR_INVALID_STATE;
        const P target = initial == ON ? init_poly.points.first() : initial == OFF ? initial_off : points.first();
        line_to(o->join, target);
        if (initial == ON) {
            if (dasher.on && points.len > 1) {
                if (init_poly.points.len == 1) {
                    plot_open_joined(*this, points.head(0), points.head(1), points.tail(2), points.tail(1));
                    initial = NONE;
                } else {
                    join_and_cap_initial();
                }
            } else {
                if (init_poly.points.len == 1) finish_initial_dotted();
                else finish_initial(init_poly.points.head(0), init_poly.points.head(1));
            }
        } else if (initial == OFF) {
            initial = NONE;
        } else {
            if (points.len == 1) {
                dotted(*this, points.first(), current_slope);
            } else if (points.len == 2) {
                plot_single(*this, points.head(0), points.head(1));
            } else {
                join(*this, o->join, points.tail(2), points.head(0), points.head(1), false);
                emit(*result, outer);
                emit(*result, inner);
                reset_contours();
                cw = -1;
            }
        }
        points.len = 0;
        return Z2D_OK;
    }

    int finish() {
        if (initial == ON) {
            if (init_poly.points.len == 0) return Z2D_ERR_INVALID_STATE;
            if (init_poly.points.len == 1) finish_initial_dotted();
            else finish_initial(init_poly.points.head(0), init_poly.points.head(1));
        } else if (initial == OFF) {
            initial = NONE;
        }
        if (dasher.on) open_end(*this);
        return Z2D_OK;
    }

    // dashed_plotter.plotDotted: a zero-length dash is a dot (round cap) or
    // a square across the current direction (square cap)
    void dotted(State &st, P p, Slope slope) {
        if (st.o->cap == Z2D_CAP_ROUND) {
            for (const PenVertex &v : pen->v) st.outer.append(P{p.x + v.pt.x, p.y + v.pt.y});
            emit(*st.result, st.outer);
        } else if (st.o->cap == Z2D_CAP_SQUARE) {
            const Face f = face_with(p, p, slope, o->thickness, o->ctm);
            double ox = f.user.dx * f.half, oy = f.user.dy * f.half;
            o->ctm.to_device_dist(ox, oy);
            st.outer.append(P{f.p1_cw.x - ox, f.p1_cw.y - oy});
            st.outer.append(P{f.p1_cw.x + ox, f.p1_cw.y + oy});
            st.outer.append(P{f.p1_ccw.x + ox, f.p1_ccw.y + oy});
            st.outer.append(P{f.p1_ccw.x - ox, f.p1_ccw.y - oy});
            emit(*st.result, st.outer);
        }
        st.outer = Contour{{}, o->scale};
        st.cw = -1;
    }

    void finish_initial_dotted() {
        dotted(*this, init_poly.points.first(), init_poly.current_slope);
        initial = NONE;
    }

    void finish_initial(P last, P second_to_last) {
        plot_open_joined(init_poly, last, second_to_last, init_poly.points.tail(2), init_poly.points.tail(1));
        initial = NONE;
    }

    // the path closes while a dash is on: the last dash joins the first one
    void join_and_cap_initial() {
        if (points.len > 2) {
            join(*this, o->join, points.tail(2), init_poly.points.head(0), init_poly.points.head(1), false);
            outer.pts.splice(outer.pts.end(), init_poly.outer.pts);
            init_poly.inner.pts.splice(init_poly.inner.pts.end(), inner.pts);
            init_poly.outer = std::move(outer);
            plot_open_joined(init_poly, points.head(0), points.head(1), init_poly.points.tail(2), init_poly.points.tail(1));
        } else {
            join(init_poly, o->join, points.tail(2), init_poly.points.head(0), init_poly.points.head(1), true);
            plot_open_joined(init_poly, points.first(), init_poly.points.first(), init_poly.points.tail(2),
                             init_poly.points.tail(1));
        }
        initial = NONE;
        reset_contours();
        cw = -1;
    }
};

// polyline_plotter.plot (hairlines): open polylines, dashes split them
int polylines(const z2d_node *nodes, size_t n, double tol, const std::vector<double> &dashes, double dash_offset,
              Contours &out) {
    std::vector<P> cur;
    PointBuffer<1, 2> points;
    Dasher dasher;
    const bool dashed = Dasher::valid(dashes);
    if (dashed) {
        dasher.d = &dashes;
        dasher.offset = dash_offset;
        dasher.reset();
    }
    auto push = [&]() {
        if (!cur.empty()) out.push_back(cur);
        cur.clear();
    };
    auto dashed_line = [&](P p0, P p1) {
        Slope slope = Slope::of(p0, p1);
        const double total = slope.normalize();
        double remaining = total;
        double step = dasher.remain < remaining ? dasher.remain : remaining;
        while (remaining > 0) {
            remaining -= step;
            const P c{p0.x + slope.dx * (total - remaining), p0.y + slope.dy * (total - remaining)};
            if (!same(c, points.last())) points.add(c);
            if (dasher.on) cur.push_back(c);
            if (dasher.step(step)) {
                out.push_back(cur);
                cur.clear();
                if (dasher.on) cur.push_back(c);
            }
            step = dasher.remain < remaining ? dasher.remain : remaining;
        }
    };
    auto line = [&](P p) {
        if (same(points.last(), p)) return;
        if (dashed) {
            dashed_line(points.last(), p);
        } else {
            cur.push_back(p);
            points.add(p);
        }
    };
    for (size_t i = 0; i < n; i++) {
        const z2d_node &nd = nodes[i];
        switch (nd.tag) {
            case Z2D_MOVE_TO:
                push();
                points.len = 0;
                if (dashed) dasher.reset();
                if (i == n - 1) break;
                cur.push_back(P{nd.p[0], nd.p[1]});
                points.add(P{nd.p[0], nd.p[1]});
                break;
            case Z2D_LINE_TO:
                if (points.len == 0) return Z2D_ERR_INVALID_STATE;
                line(P{nd.p[0], nd.p[1]});
                break;
            case Z2D_CURVE_TO:
                if (points.len == 0) return Z2D_ERR_INVALID_STATE;
                spline(points.last(), P{nd.p[0], nd.p[1]}, P{nd.p[2], nd.p[3]}, P{nd.p[4], nd.p[5]}, tol, line);
                break;
            case Z2D_CLOSE_PATH:
                if (points.len >= 2 && !same(points.last(), points.first())) {
                    if (dashed) {
                        dashed_line(points.last(), points.first());
                    } else {
                        cur.push_back(points.first());
                        points.add(points.first());
                    }
                }
                break;
            default: return Z2D_ERR_INVALID_ARGUMENT;
        }
    }
    push();
    return Z2D_OK;
}

bool finite_nodes(const z2d_node *nodes, size_t n) {
    for (size_t i = 0; i < n; i++) {
        const int k = nodes[i].tag == Z2D_CURVE_TO ? 6 : (nodes[i].tag == Z2D_CLOSE_PATH ? 0 : 2);
        for (int j = 0; j < k; j++)
            if (!std::isfinite(nodes[i].p[j])) return false;
    }
    return true;
}

}  // namespace

extern "C" {

// painter.stroke up to the polygon (painter.zig:214-344): the contours the
// rasteriser would fill, points already multiplied by the rasteriser scale
// (returned in *scale); for hairlines the polylines, scale 1.
__attribute__((visibility("default"))) int z2doracle_stroke_contours(
    const z2d_node *nodes, size_t n_nodes, const z2d_stroke_opts *opts, int32_t surface_format, double *points,
    size_t cap_points, uint64_t *n_points, uint64_t *contour_ends, size_t cap_contours, uint64_t *n_contours,
    double *scale) {
    if (!opts || !n_points || !n_contours || !scale || (n_nodes && !nodes)) return Z2D_ERR_INVALID_ARGUMENT;
    *n_points = *n_contours = 0;
    Tf ctm{opts->transformation[0], opts->transformation[1], opts->transformation[2],
           opts->transformation[3], opts->transformation[4], opts->transformation[5]};
    Tf inv;
    if (!ctm.inverse(inv)) return Z2D_ERR_INVALID_ARGUMENT;  // Transformation.Error.InvalidMatrix
    if (!finite_nodes(nodes, n_nodes)) return Z2D_ERR_INVALID_STATE;
    std::vector<double> dashes(opts->dashes, opts->dashes + (opts->dashes ? opts->n_dashes : 0));
    Contours out;
    int rc = Z2D_OK;
    *scale = 1.0;
    if (n_nodes == 0) {
    } else if (opts->hairline) {
        rc = polylines(nodes, n_nodes, opts->tolerance, dashes, opts->dash_offset, out);
    } else {
        const int aa = surface_format == Z2D_FORMAT_ALPHA1 ? Z2D_AA_NONE : opts->anti_aliasing;
        *scale = aa == Z2D_AA_NONE ? 1.0 : 4.0;
        const bool wide = opts->line_width >= 2;
        Opts o;
        o.cap = wide ? opts->line_cap : Z2D_CAP_BUTT;
        o.join = wide ? opts->line_join : Z2D_JOIN_MITER;
        o.miter_limit = wide ? opts->miter_limit : 10.0;
        o.ctm = ctm;
        o.dashes = dashes;
        o.dash_offset = opts->dash_offset;
        o.scale = *scale;
        o.thickness = opts->line_width >= 0.00390625 ? opts->line_width : 0.00390625;
        o.tolerance = opts->tolerance > 0.001 ? opts->tolerance : 0.001;
        // the pen exists from the start for round joins or caps, else it is
        // made at the first curve (same vertices either way)
        const Pen pen = make_pen(o.thickness, o.tolerance, o.ctm);
        if (Dasher::valid(o.dashes)) {
            Dashed p;
            p.o = &o;
            p.pen = &pen;
            p.result = &out;
            p.reset_contours();
            p.dasher.d = &o.dashes;
            p.dasher.offset = o.dash_offset;
            p.dasher.reset();
            rc = p.run(nodes, n_nodes);
        } else {
            Solid p;
            p.o = &o;
            p.pen = &pen;
            p.result = &out;
            p.reset_contours();
            rc = p.run(nodes, n_nodes);
        }
    }
    if (rc) return rc;
    uint64_t np = 0;
    for (const auto &c : out) {
        for (const P &p : c) {
            if (np < cap_points && points) {
                points[2 * np] = p.x;
                points[2 * np + 1] = p.y;
            }
            np++;
        }
        if (*n_contours < cap_contours && contour_ends) contour_ends[*n_contours] = np;
        (*n_contours)++;
    }
    *n_points = np;
    return Z2D_OK;
}

}  // extern "C"
