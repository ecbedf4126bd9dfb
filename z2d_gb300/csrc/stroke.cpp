// stroke.cpp -- painter.stroke's polygon builder, on the host.
//
// Restates z2d's stroke tessellation (src/internal/tess/stroke_plotter.zig,
// Face.zig, Pen.zig, Slope.zig, the Contour of Polygon.zig, and the parts of
// Spline.zig, Transformation.zig and arc.zig it uses) operation by operation
// in f64.  The result is the list of closed contours (points already
// multiplied by the rasteriser scale) whose edges painter.stroke hands to
// the rasteriser with the non-zero rule; the GPU fill pipeline draws them.
// Dashes and hairlines are not restated yet (the callers reject them).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <type_traits>
#include <utility>
#include <vector>

#include "stroke.h"
#include "stroke_geom.h"

namespace z2dg {
namespace stroke {

int32_t pen_vertex_count(double thickness, double tolerance, const double m[6]) {  // Pen.init (Pen.zig:25-60)
    const sg::Tf ctm{m[0], m[1], m[2], m[3], m[4], m[5]};
    const double radius = thickness / 2;
    const double a = ctm.ax, b = ctm.by, c = ctm.cx, d = ctm.dy;
    // arc.transformed_circle_major_axis (arc.zig:92-262)
    double major;
    const double eps = 0.00390625;
    const double det = a * d - b * c;
    if (std::fabs(det * det - 1.0) < eps &&
        ((std::fabs(b) < eps && std::fabs(c) < eps) || (std::fabs(a) < eps && std::fabs(d) < eps))) {
        major = radius;
    } else {
        const double i = a * a + b * b;
        const double j = c * c + d * d;
        const double f = 0.5 * (i + j);
        const double g = 0.5 * (i - j);
        const double h = a * c + b * d;
        major = radius * std::sqrt(f + std::hypot(g, h));
    }
    if (tolerance >= major * 4) return 1;
    if (tolerance >= major) return 4;
    const double delta = std::acos(1 - tolerance / major);
    if (delta == 0) return 4;
    const double nf = std::ceil(2 * M_PI / delta);
    const int32_t k = (int32_t)nf;
    return k < 4 ? 4 : ((k % 2 != 0) ? k + 1 : k);
}

void pen_trig(int32_t n, bool reflect, double *out) {  // Pen.init (Pen.zig:62-75)
    for (int32_t i = 0; i < n; i++) {
        double t = 2 * M_PI * (double)i / (double)n;
        if (reflect) t = -t;
        out[2 * (size_t)i] = std::cos(t);
        out[2 * (size_t)i + 1] = std::sin(t);
    }
}

namespace {

using sg::compare;
using sg::compare_for_miter_limit;
using sg::determinant;
using sg::eq;
using sg::Face;
using sg::intersect;
using sg::normalized;
using sg::PenVertex;
using sg::Pt;
using sg::slope;
using sg::Slope;
using sg::Tf;
using sg::user_to_device_distance;



// Pen.zig
struct Pen {
    std::vector<PenVertex> v;
    bool ok = false;
};
// Pen.init (Pen.zig:25-88)
Pen make_pen(double thickness, double tolerance, const Tf &ctm) {
    Pen pen;
    pen.ok = true;
    const double radius = thickness / 2;
    const double m[6] = {ctm.ax, ctm.by, ctm.cx, ctm.dy, ctm.tx, ctm.ty};
    const int32_t n = pen_vertex_count(thickness, tolerance, m);
    std::vector<double> trig((size_t)std::max(0, n) * 2);
    pen_trig(n, determinant(ctm) < 0, trig.data());
    pen.v.resize((size_t)std::max(0, n));
    for (int32_t i = 0; i < n; i++) {
        double dx = radius * trig[2 * (size_t)i], dy = radius * trig[2 * (size_t)i + 1];
        user_to_device_distance(ctm, dx, dy);
        pen.v[(size_t)i].point = Pt{dx, dy};
    }
    for (int32_t i = 0; i < n; i++) {
        const int32_t next = (i >= n - 1) ? 0 : i + 1;
        const int32_t prev = std::max(0, i == 0 ? n - 1 : i - 1);
        pen.v[(size_t)i].slope_cw = slope(pen.v[(size_t)prev].point, pen.v[(size_t)i].point);
        pen.v[(size_t)i].slope_ccw = slope(pen.v[(size_t)i].point, pen.v[(size_t)next].point);
    }
    return pen;
}
// A doubly linked list of points whose nodes live in one per-thread arena
// (reset by each plot call), so that inserting a point allocates nothing
// and splicing two lists is O(1).  Position -1 is end().
struct ListNode {
    Pt p;
    int32_t prev, next;
};
thread_local std::vector<ListNode> t_arena;

struct PtList {
    int32_t head = -1, tail = -1;
    size_t n = 0;
    using It = int32_t;
    It begin() const { return head; }
    It end() const { return -1; }
    size_t size() const { return n; }
    void clear() {
        head = tail = -1;
        n = 0;
    }
    void insert(It before, Pt p) {
        const int32_t k = (int32_t)t_arena.size();
        if (before < 0) {
            t_arena.push_back(ListNode{p, tail, -1});
            if (tail >= 0) t_arena[(size_t)tail].next = k;
            else head = k;
            tail = k;
        } else {
            const int32_t pv = t_arena[(size_t)before].prev;
            t_arena.push_back(ListNode{p, pv, before});
            t_arena[(size_t)before].prev = k;
            if (pv >= 0) t_arena[(size_t)pv].next = k;
            else head = k;
        }
        n++;
    }
    void push_back(Pt p) { insert(-1, p); }
    void push_front(Pt p) { insert(head, p); }
    // std::list::splice(end(), other): other's points move to the back
    void splice_back(PtList &o) {
        if (o.head < 0) return;
        if (tail >= 0) {
            t_arena[(size_t)tail].next = o.head;
            t_arena[(size_t)o.head].prev = tail;
        } else {
            head = o.head;
        }
        tail = o.tail;
        n += o.n;
        o.clear();
    }
    void swap(PtList &o) {
        std::swap(head, o.head);
        std::swap(tail, o.tail);
        std::swap(n, o.n);
    }
    template <class F>
    void for_each(F &&f) const {
        for (int32_t i = head; i >= 0; i = t_arena[(size_t)i].next) f(t_arena[(size_t)i].p);
    }
};

// Polygon.Contour: a doubly linked list of scaled points.
struct Contour {
    PtList pts;
    double scale = 1;
    using It = PtList::It;
    void plot(Pt p, It before) { pts.insert(before, Pt{p.x * scale, p.y * scale}); }
    void plot(Pt p) { pts.push_back(Pt{p.x * scale, p.y * scale}); }
    void plot_reverse(Pt p) { pts.push_front(Pt{p.x * scale, p.y * scale}); }
};

// PointBuffer(2, 5) (point_buffer.zig:14-60)
struct PointBuffer {
    Pt items[5];
    size_t len = 0;
    void add(Pt p) {
        if (len < 5) {
            items[len++] = p;
        } else {
            for (size_t i = 2; i < 4; i++) items[i] = items[i + 1];
            items[4] = p;
        }
    }
    Pt head(size_t n) const { return items[n]; }
    Pt tail(size_t n) const { return items[len - n]; }
};

// The contours and clockwise state of one polygon under construction: the
// plotter's own, or the saved first dash of a closed dashed path (the
// InitialPolygon of dashed_plotter.zig:54-64).
struct Side {
    Contour outer, inner;
    int clockwise = -1;  // -1: unset (null)
    void set_scale(double sc) { outer.scale = inner.scale = sc; }
};

// Dasher.zig
struct Dasher {
    const double *dashes = nullptr;
    size_t n = 0;
    double offset = 0;
    size_t idx = 0;
    bool on = true;
    double remain = 0;
    void init(const double *d, size_t count, double off) {
        dashes = d;
        n = count;
        offset = off;
        reset();
    }
    bool stuck = false;  // the offset did not settle (guard; z2d would loop)
    void apply_offset() {  // Dasher.applyOffset (Dasher.zig:40-54)
        remain -= offset;
        int64_t guard = 0;
        while (remain < 0 || remain > dashes[idx]) {
            if (++guard > (int64_t)1 << 26) {
                stuck = true;
                return;
            }
            if (remain < 0) {
                remain += dashes[idx];
                idx = (idx >= n - 1) ? 0 : idx + 1;
            } else {
                remain -= dashes[idx];
                idx = (idx == 0) ? n - 1 : idx - 1;
            }
            on = !on;
        }
    }
    void reset() {
        idx = 0;
        on = true;
        remain = dashes[0];
        apply_offset();
    }
    bool step(double len) {  // Dasher.step (Dasher.zig:63-76)
        bool stepped = false;
        remain -= len;
        if (remain <= 0) {
            stepped = true;
            on = !on;
            idx += 1;
            if (idx >= n) idx = 0;
            remain = dashes[idx];
        }
        return stepped;
    }
};
// Dasher.validate (Dasher.zig:15-26)
bool dashes_valid(const double *d, size_t n) {
    bool valid = false;
    for (size_t i = 0; i < n; i++) {
        if (d[i] < 0) return false;
        if (d[i] > 0) valid = true;
    }
    return valid;
}

// What both plotters share: options, pen, the result and the polygon
// pieces of stroke_plotter.zig that operate on a Side.
struct Common {
    const Options &o;
    Tf ctm;
    Pen pen;
    Polygon &result;
    int error = 0;

    Common(const Options &opts, Polygon &res) : o(opts), result(res) {
        ctm = Tf{o.ctm[0], o.ctm[1], o.ctm[2], o.ctm[3], o.ctm[4], o.ctm[5]};
        if (o.join == kJoinRound || o.cap == kCapRound) pen = make_pen(o.thickness, o.tolerance, ctm);
    }

    // Polygon.addEdgesFromContour: the contour's points, closed later
    void emit(const Contour &c) {
        if (c.pts.size() == 0) return;
        c.pts.for_each([&](Pt p) {
            result.xy.push_back(p.x);
            result.xy.push_back(p.y);
        });
        result.ends.push_back(result.points());
    }

    // join (stroke_plotter.zig:405-545)
    void join(Side &sd, int mode, Pt p0, Pt p1, Pt p2, bool use_before, Contour::It before_outer) {
        if (eq(p0, p1) || eq(p1, p2)) {
            if (sd.clockwise < 0) sd.clockwise = 0;
            return;
        }
        const Face in = sg::face_init(p0, p1, o.thickness, ctm);
        const Face out = sg::face_init(p1, p2, o.thickness, ctm);
        const bool jcw = compare(in.dev_slope, out.dev_slope) < 0;
        const bool pcw = sd.clockwise >= 0 ? sd.clockwise != 0 : jcw;
        const bool switched = jcw != pcw;
        auto to_outer = [&](Pt p) {
            if (use_before) sd.outer.plot(p, before_outer);
            else sd.outer.plot(p);
        };
        auto plot_outer = [&](Pt p) {
            if (switched) sd.inner.plot_reverse(p);
            else to_outer(p);
        };
        auto plot_inner = [&](Pt p) {
            if (switched) to_outer(p);
            else sd.inner.plot_reverse(p);
        };
        if (compare(in.dev_slope, out.dev_slope) == 0) {
            plot_outer(jcw ? in.p1_ccw : in.p1_cw);
            plot_inner(jcw ? in.p1_cw : in.p1_ccw);
            if (sd.clockwise < 0) sd.clockwise = pcw ? 1 : 0;
            return;
        }
        if (mode == kJoinMiter || mode == kJoinBevel) {
            if (mode == kJoinMiter && compare_for_miter_limit(in.dev_slope, out.dev_slope, o.miter_limit)) {
                plot_outer(intersect(in, out, jcw));
            } else {
                plot_outer(jcw ? in.p1_ccw : in.p1_cw);
                plot_outer(jcw ? out.p0_ccw : out.p0_cw);
            }
        } else {
            plot_outer(jcw ? in.p1_ccw : in.p1_cw);
            const int32_t len = (int32_t)pen.v.size();
            int32_t start;
            const int32_t n = sg::pen_range(pen.v.data(), len, in.dev_slope, out.dev_slope, jcw, start);
            for (int32_t k = 0; k < n; k++) {
                const Pt v = pen.v[(size_t)sg::pen_step(start, k, len, jcw)].point;
                plot_outer(Pt{p1.x + v.x, p1.y + v.y});
            }
            plot_outer(jcw ? out.p0_ccw : out.p0_cw);
        }
        plot_inner(jcw ? in.p1_cw : in.p1_ccw);
        plot_inner(p1);
        plot_inner(jcw ? out.p0_cw : out.p0_ccw);
        if (sd.clockwise < 0) sd.clockwise = pcw ? 1 : 0;
    }

    // Face.cap (Face.zig:156-246); points go to `sink`
    template <class Sink>
    void cap(const Face &f, bool cw, Sink &&sink) {
        if (o.cap == kCapButt) {
            if (cw) {
                sink(f.p1_ccw);
                sink(f.p1_cw);
            } else {
                sink(f.p1_cw);
                sink(f.p1_ccw);
            }
        } else if (o.cap == kCapSquare) {
            double ox = f.user_slope.dx * f.half_width, oy = f.user_slope.dy * f.half_width;
            user_to_device_distance(ctm, ox, oy);
            if (cw) {
                sink(f.p1_ccw);
                sink(Pt{f.p1_ccw.x + ox, f.p1_ccw.y + oy});
                sink(Pt{f.p1_cw.x + ox, f.p1_cw.y + oy});
                sink(f.p1_cw);
            } else {
                sink(f.p1_cw);
                sink(Pt{f.p1_cw.x + ox, f.p1_cw.y + oy});
                sink(Pt{f.p1_ccw.x + ox, f.p1_ccw.y + oy});
                sink(f.p1_ccw);
            }
        } else {
            sink(cw ? f.p1_ccw : f.p1_cw);
            const int32_t len = (int32_t)pen.v.size();
            int32_t start;
            const int32_t n =
                sg::pen_range(pen.v.data(), len, f.dev_slope, Slope{-f.dev_slope.dx, -f.dev_slope.dy}, cw, start);
            for (int32_t k = 0; k < n; k++) {
                const Pt v = pen.v[(size_t)sg::pen_step(start, k, len, cw)].point;
                sink(Pt{f.p1.x + v.x, f.p1.y + v.y});
            }
            sink(cw ? f.p1_cw : f.p1_ccw);
        }
    }
    template <class Sink>
    void cap_p0(const Face &f, bool cw, Sink &&sink) {
        cap(sg::face_init(f.p1, f.p0, f.width, ctm), cw, sink);
    }

    void clear(Side &sd) {
        sd.outer.pts.clear();
        sd.inner.pts.clear();
        sd.clockwise = -1;
    }

    // plotSingle (stroke_plotter.zig:232-279)
    void plot_single(Side &sd, Pt start, Pt end) {
        const Face f = sg::face_init(start, end, o.thickness, ctm);
        auto sink = [&](Pt p) { sd.outer.plot(p); };
        cap_p0(f, true, sink);
        cap(f, true, sink);
        emit(sd.outer);
        sd.outer.pts.clear();
        sd.clockwise = -1;
    }

    // plotOpenJoined (stroke_plotter.zig:281-363)
    void plot_open_joined(Side &sd, Pt s0, Pt e0, Pt s1, Pt e1) {
        const Face fs = sg::face_init(s0, e0, o.thickness, ctm);
        const Face fe = sg::face_init(s1, e1, o.thickness, ctm);
        const bool cw = sd.clockwise >= 0 ? sd.clockwise != 0 : true;
        const Contour::It first = sd.outer.pts.begin();  // the insertion point is captured before plotting
        auto before_first = [&](Pt p) { sd.outer.plot(p, first); };
        cap_p0(fs, cw, before_first);
        auto append = [&](Pt p) { sd.outer.plot(p); };
        cap(fe, cw, append);
        sd.outer.pts.splice_back(sd.inner.pts);
        emit(sd.outer);
        clear(sd);
    }

    // The dots of zero-length strokes: round caps draw the pen; the dashed
    // plotter also draws square dots and always resets the state
    // (stroke_plotter.zig:183-219, dashed_plotter.zig:387-470).
    void plot_dot(Side &sd, Pt p, bool dashed_plotter, Slope slope) {
        if (o.cap == kCapRound) {
            for (const PenVertex &v : pen.v) sd.outer.plot(Pt{p.x + v.point.x, p.y + v.point.y});
            emit(sd.outer);
        } else if (dashed_plotter && o.cap == kCapSquare) {
            const Face f = sg::face_init2(p, p, slope, o.thickness, ctm);
            double ox = f.user_slope.dx * f.half_width, oy = f.user_slope.dy * f.half_width;
            user_to_device_distance(ctm, ox, oy);
            sd.outer.plot(Pt{f.p1_cw.x - ox, f.p1_cw.y - oy});
            sd.outer.plot(Pt{f.p1_cw.x + ox, f.p1_cw.y + oy});
            sd.outer.plot(Pt{f.p1_ccw.x + ox, f.p1_ccw.y + oy});
            sd.outer.plot(Pt{f.p1_ccw.x - ox, f.p1_ccw.y - oy});
            emit(sd.outer);
        } else if (!dashed_plotter) {
            return;  // stroke_plotter's dot draws nothing and leaves the state alone
        }
        sd.outer.pts.clear();
        sd.clockwise = -1;
    }

    // Spline.decompose (Spline.zig:37-71) with `line` as the lineTo
    template <class Line>
    void spline(Pt a, Pt b, Pt c, Pt d, Line &&line) {
        if (eq(a, b) && eq(c, d)) {
            line(d);
            return;
        }
        struct K {
            Pt a, b, c, d;
        };
        auto error_sq = [](const K &k) {
            double bx = k.b.x - k.a.x, by = k.b.y - k.a.y, cx = k.c.x - k.a.x, cy = k.c.y - k.a.y;
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
        };
        auto lerp = [](Pt p, Pt q) { return Pt{p.x + ((q.x - p.x) / 2), p.y + ((q.y - p.y) / 2)}; };
        const double tol = o.tolerance * o.tolerance;
        std::vector<K> stack{K{a, b, c, d}};
        int64_t budget = 1 << 22;
        while (!stack.empty() && error == 0) {
            K k = stack.back();
            stack.pop_back();
            while (error == 0) {
                if (--budget < 0 || stack.size() > 64) {
                    error = kErrInvalidState;
                    break;
                }
                if (error_sq(k) < tol) {
                    if (!eq(k.a, a)) line(k.a);
                    break;
                }
                const Pt ab = lerp(k.a, k.b), bc = lerp(k.b, k.c), cd = lerp(k.c, k.d);
                const Pt abbc = lerp(ab, bc), bccd = lerp(bc, cd), fin = lerp(abbc, bccd);
                stack.push_back(K{fin, bccd, cd, k.d});
                k = K{k.a, ab, abbc, fin};
            }
        }
        if (error == 0) line(d);
    }
};

// stroke_plotter.Plotter (stroke_plotter.zig:77-230)
struct SolidPlotter : Common {
    PointBuffer points;
    Side sd;

    SolidPlotter(const Options &opts, Polygon &res) : Common(opts, res) {
        sd.set_scale(opts.scale);
    }

    void line_to(int join_mode, Pt p) {
        if (points.len == 0) {
            error = kErrInvalidState;
            return;
        }
        if (eq(p, points.tail(1))) return;  // degenerate node
        points.add(p);
        if (points.len > 2) join(sd, join_mode, points.tail(3), points.tail(2), points.tail(1), false, sd.outer.pts.end());
    }

    void curve_to(Pt b, Pt c, Pt d) {  // curves join their pieces round (stroke_plotter.zig:126-150)
        if (points.len == 0) {
            error = kErrInvalidState;
            return;
        }
        if (!pen.ok) pen = make_pen(o.thickness, o.tolerance, ctm);
        spline(points.tail(1), b, c, d, [&](Pt q) { line_to(kJoinRound, q); });
    }

    // plotClosedJoined (stroke_plotter.zig:365-403)
    void plot_closed_joined(Pt i0, Pt i1, Pt p1, Pt p2) {
        if (!eq(p2, i0)) {
            join(sd, o.join, p1, p2, i0, false, sd.outer.pts.end());
            join(sd, o.join, p2, i0, i1, false, sd.outer.pts.end());
        } else {
            join(sd, o.join, p1, i0, i1, false, sd.outer.pts.end());
        }
        emit(sd.outer);
        emit(sd.inner);
        clear(sd);
    }

    void close_path() {
        switch (points.len) {
            case 0: break;
            case 1: plot_dot(sd, points.head(0), false, Slope{0, 0}); break;
            case 2: plot_single(sd, points.head(0), points.head(1)); break;
            default: plot_closed_joined(points.head(0), points.head(1), points.tail(2), points.tail(1)); break;
        }
        points.len = 0;
    }

    void finish() {
        if (points.len == 2) plot_single(sd, points.head(0), points.head(1));
        else if (points.len > 2) plot_open_joined(sd, points.head(0), points.head(1), points.tail(2), points.tail(1));
    }

    void move_to(Pt p) {
        if (points.len > 0) finish();
        points.len = 0;
        points.add(p);
    }
};

// dashed_plotter.Plotter (dashed_plotter.zig:52-600)
struct DashedPlotter : Common {
    PointBuffer points;
    Side sd;
    Dasher dasher;
    Slope current_slope{0, 0};
    enum { kNone, kOff, kOn } init_kind = kNone;
    Pt init_off{0, 0};
    PointBuffer init_points;
    Side init_side;
    Slope init_slope{0, 0};

    DashedPlotter(const Options &opts, Polygon &res) : Common(opts, res) {
        sd.set_scale(opts.scale);
        init_side.set_scale(opts.scale);
        dasher.init(opts.dashes, opts.n_dashes, opts.dash_offset);
        if (dasher.stuck) error = kErrInvalidState;
    }

    void line_to(int join_mode, Pt p) {  // _runLineTo (dashed_plotter.zig:113-187)
        if (points.len == 0) {
            error = kErrInvalidState;
            return;
        }
        const Pt first = points.tail(1);
        if (eq(p, first)) return;
        Slope sl = slope(first, p);
        current_slope = normalized(sl);
        device_to_user_distance(ctm, sl.dx, sl.dy);
        const double total = normalize(sl);
        double remaining = total;
        double step_len = std::min(dasher.remain, remaining);
        int64_t guard = 0;
        while (remaining > 0 && error == 0) {
            if (++guard > (int64_t)1 << 26) {  // dash steps of one segment (guard)
                error = kErrInvalidState;
                break;
            }
            remaining -= step_len;
            double xo = sl.dx * (total - remaining), yo = sl.dy * (total - remaining);
            user_to_device_distance(ctm, xo, yo);
            const Pt cdp{first.x + xo, first.y + yo};
            if (!eq(cdp, points.tail(1))) points.add(cdp);
            if (dasher.on && points.len > 2)
                join(sd, join_mode, points.tail(3), points.tail(2), points.tail(1), false, sd.outer.pts.end());
            if (dasher.step(step_len)) next_segment(cdp);
            step_len = std::min(dasher.remain, remaining);
        }
    }

    void curve_to(Pt b, Pt c, Pt d) {
        if (points.len == 0) {
            error = kErrInvalidState;
            return;
        }
        if (!pen.ok) pen = make_pen(o.thickness, o.tolerance, ctm);
        spline(points.tail(1), b, c, d, [&](Pt q) { line_to(kJoinRound, q); });
    }

    // the segment that just ended, if it was on (dashed_plotter.zig:283-310)
    void plot_segment() {
        switch (points.len) {
            case 0: break;
            case 1: plot_dot(sd, points.head(0), true, current_slope); break;
            case 2: plot_single(sd, points.head(0), points.head(1)); break;
            default: plot_open_joined(sd, points.head(0), points.head(1), points.tail(2), points.tail(1)); break;
        }
    }

    void next_segment(Pt p) {
        if (init_kind == kNone) save_initial();
        else if (!dasher.on) plot_segment();
        points.len = 0;
        points.add(p);
    }

    void save_initial() {  // saveInitial (dashed_plotter.zig:472-501)
        if (!dasher.on) {
            init_kind = kOn;
            init_points = points;
            init_side.outer.pts.clear();
            init_side.inner.pts.clear();
            init_side.outer.pts.splice_back(sd.outer.pts);
            init_side.inner.pts.splice_back(sd.inner.pts);
            init_side.clockwise = sd.clockwise;
            init_slope = current_slope;
        } else {
            init_kind = kOff;
            init_off = points.head(0);
        }
        clear(sd);
    }

    void finish_initial_dotted() {
        plot_dot(sd, init_points.head(0), true, init_slope);
        init_kind = kNone;
    }

    void finish_initial(Pt a, Pt b) {
        plot_open_joined(init_side, a, b, init_points.tail(2), init_points.tail(1));
        init_kind = kNone;
    }

    void join_and_cap_initial() {  // joinAndCapInitial (dashed_plotter.zig:531-588)
        if (points.len > 2) {
            join(sd, o.join, points.tail(2), init_points.head(0), init_points.head(1), false, sd.outer.pts.end());
            sd.outer.pts.splice_back(init_side.outer.pts);
            init_side.inner.pts.splice_back(sd.inner.pts);
            init_side.outer.pts.swap(sd.outer.pts);
            sd.outer.pts.clear();
            plot_open_joined(init_side, points.head(0), points.head(1), init_points.tail(2), init_points.tail(1));
        } else {
            join(init_side, o.join, points.tail(2), init_points.head(0), init_points.head(1), true,
                 init_side.outer.pts.begin());
            plot_open_joined(init_side, points.head(0), init_points.head(0), init_points.tail(2), init_points.tail(1));
        }
        init_kind = kNone;
        clear(sd);
    }

    void close_path() {  // runClosePath (dashed_plotter.zig:201-281)
        if (points.len == 0) {
            error = kErrInvalidState;
            return;
        }
        const Pt target = init_kind == kOn ? init_points.head(0) : (init_kind == kOff ? init_off : points.head(0));
        line_to(o.join, target);
        if (error) return;
        if (init_kind == kOn) {
            if (dasher.on && points.len > 1) {
                if (init_points.len == 1) {
                    plot_open_joined(sd, points.head(0), points.head(1), points.tail(2), points.tail(1));
                    init_kind = kNone;
                } else {
                    join_and_cap_initial();
                }
            } else if (init_points.len == 1) {
                finish_initial_dotted();
            } else {
                finish_initial(init_points.head(0), init_points.head(1));
            }
        } else if (init_kind == kOff) {
            init_kind = kNone;
        } else {
            switch (points.len) {
                case 1: plot_dot(sd, points.head(0), true, current_slope); break;
                case 2: plot_single(sd, points.head(0), points.head(1)); break;
                default:
                    join(sd, o.join, points.tail(2), points.head(0), points.head(1), false, sd.outer.pts.end());
                    emit(sd.outer);
                    emit(sd.inner);
                    clear(sd);
                    break;
            }
        }
        points.len = 0;
    }

    void finish() {  // finish (dashed_plotter.zig:346-385)
        if (init_kind == kOn) {
            if (init_points.len == 1) finish_initial_dotted();
            else finish_initial(init_points.head(0), init_points.head(1));
        } else if (init_kind == kOff) {
            init_kind = kNone;
        }
        if (dasher.on) plot_segment();
    }

    void move_to(Pt p) {
        finish();
        dasher.reset();
        if (dasher.stuck) error = kErrInvalidState;
        points.len = 0;
        points.add(p);
    }
};

// polyline_plotter.plot (polyline_plotter.zig:27-221): the path as open
// polylines for hairline strokes, without transformation or scale.
struct PolylinePlotter : Common {
    Pt first{0, 0}, last{0, 0};
    int len = 0;  // PointBuffer(1, 2) length, saturating at 3
    bool use_dasher = false;
    Dasher dasher;
    size_t contour_start = 0;  // first point of the current polyline

    PolylinePlotter(const Options &opts, Polygon &res) : Common(opts, res) {
        use_dasher = dashed(opts);
        if (use_dasher) {
            dasher.init(opts.dashes, opts.n_dashes, opts.dash_offset);
            if (dasher.stuck) error = kErrInvalidState;
        }
    }
    void add(Pt p) {
        if (len == 0) first = p;
        last = p;
        if (len < 3) len++;
    }
    void plot_pt(Pt p) {  // Contour.plot with scale 1
        result.xy.push_back(p.x);
        result.xy.push_back(p.y);
    }
    void end_polyline() {  // the current polyline goes to the result if it has points
        if (result.points() > contour_start) result.ends.push_back(result.points());
        contour_start = result.points();
    }
    // dashedLineTo (polyline_plotter.zig:186-221)
    void dashed_line(Pt p0, Pt p1) {
        Slope sl = slope(p0, p1);
        const double total = normalize(sl);
        double remaining = total;
        double step_len = std::min(dasher.remain, remaining);
        int64_t guard = 0;
        while (remaining > 0) {
            if (++guard > (int64_t)1 << 26) {
                error = kErrInvalidState;
                return;
            }
            remaining -= step_len;
            const Pt cdp{p0.x + sl.dx * (total - remaining), p0.y + sl.dy * (total - remaining)};
            if (!eq(cdp, last)) add(cdp);
            if (dasher.on) plot_pt(cdp);
            if (dasher.step(step_len)) {
                end_polyline();
                if (dasher.on) plot_pt(cdp);
            }
            step_len = std::min(dasher.remain, remaining);
        }
    }
    void move_to(Pt p, bool last_node) {
        end_polyline();
        len = 0;
        if (use_dasher) dasher.reset();
        if (last_node) return;  // the move_to a Path adds after close_path
        plot_pt(p);
        add(p);
    }
    void line_to(int, Pt p) {
        if (len == 0) {
            error = kErrInvalidState;
            return;
        }
        if (eq(last, p)) return;
        if (use_dasher) {
            dashed_line(last, p);
        } else {
            plot_pt(p);
            add(p);
        }
    }
    void curve_to(Pt b, Pt c, Pt d) {
        if (len == 0) {
            error = kErrInvalidState;
            return;
        }
        spline(last, b, c, d, [&](Pt q) { line_to(0, q); });
    }
    void close_path() {
        if (len < 2 || eq(last, first)) return;
        if (use_dasher) {
            dashed_line(last, first);
        } else {
            plot_pt(first);
            add(first);
        }
    }
    void finish() { end_polyline(); }
};

template <class P>
int run(P &p, const z2d_node *nodes, size_t n_nodes) {
    for (size_t i = 0; i < n_nodes && p.error == 0; i++) {
        const z2d_node &nd = nodes[i];
        switch (nd.tag) {
            case Z2D_MOVE_TO:
                if constexpr (std::is_same<P, PolylinePlotter>::value) {
                    p.move_to(Pt{nd.p[0], nd.p[1]}, i == n_nodes - 1);
                } else {
                    p.move_to(Pt{nd.p[0], nd.p[1]});
                }
                break;
            case Z2D_LINE_TO: p.line_to(p.o.join, Pt{nd.p[0], nd.p[1]}); break;
            case Z2D_CURVE_TO: p.curve_to(Pt{nd.p[0], nd.p[1]}, Pt{nd.p[2], nd.p[3]}, Pt{nd.p[4], nd.p[5]}); break;
            case Z2D_CLOSE_PATH: p.close_path(); break;
            default: return kErrInvalidState;
        }
    }
    if (p.error) return p.error;
    p.finish();
    return p.error;
}

}  // namespace

bool transformation_invertible(const double m[6]) {
    Tf inv;
    return inverse(Tf{m[0], m[1], m[2], m[3], m[4], m[5]}, inv);
}

bool dashed(const Options &opts) { return opts.n_dashes > 0 && dashes_valid(opts.dashes, opts.n_dashes); }

int polyline(const z2d_node *nodes, size_t n_nodes, const Options &opts, Polygon &out) {
    out.clear();
    t_arena.clear();
    Options o = opts;
    o.join = kJoinMiter;  // no pen
    o.cap = kCapButt;
    PolylinePlotter p(o, out);
    if (p.error) return p.error;
    return run(p, nodes, n_nodes);
}

int plot(const z2d_node *nodes, size_t n_nodes, const Options &opts, Polygon &contours) {
    contours.clear();
    t_arena.clear();
    if (dashed(opts)) {  // stroke_plotter.plot (stroke_plotter.zig:40-44)
        DashedPlotter p(opts, contours);
        return run(p, nodes, n_nodes);
    }
    SolidPlotter p(opts, contours);
    return run(p, nodes, n_nodes);
}

}  // namespace stroke
}  // namespace z2dg
