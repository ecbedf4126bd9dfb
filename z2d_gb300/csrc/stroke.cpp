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
#include <list>
#include <vector>

#include "stroke.h"

namespace z2dg {
namespace stroke {
namespace {

struct Pt {
    double x, y;
};
inline bool eq(Pt a, Pt b) { return a.x == b.x && a.y == b.y; }

// Transformation.zig
struct Tf {
    double ax, by, cx, dy, tx, ty;
};
const Tf kIdentity{1, 0, 0, 1, 0, 0};
inline bool tf_equal(const Tf &a, const Tf &b) {
    return a.ax == b.ax && a.by == b.by && a.cx == b.cx && a.dy == b.dy && a.tx == b.tx && a.ty == b.ty;
}
inline double determinant(const Tf &a) { return a.ax * a.dy - a.by * a.cx; }
// Transformation.inverse (Transformation.zig:103-162)
bool inverse(const Tf &a, Tf &out) {
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
inline void user_to_device_distance(const Tf &a, double &x, double &y) {
    const double ix = x, iy = y;
    x = a.ax * ix + a.by * iy;
    y = a.cx * ix + a.dy * iy;
}
inline void device_to_user_distance(const Tf &a, double &x, double &y) {
    Tf inv;
    inverse(a, inv);  // validated by the caller
    user_to_device_distance(inv, x, y);
}

// arc.transformed_circle_major_axis (arc.zig:92-262)
double transformed_circle_major_axis(const Tf &m, double radius) {
    const double a = m.ax, b = m.by, c = m.cx, d = m.dy;
    const double eps = 0.00390625;
    const double det = m.ax * m.dy - m.by * m.cx;
    if (std::fabs(det * det - 1.0) < eps) {
        if (std::fabs(m.by) < eps && std::fabs(m.cx) < eps) return radius;
        if (std::fabs(m.ax) < eps && std::fabs(m.dy) < eps) return radius;
    }
    const double i = a * a + b * b;
    const double j = c * c + d * d;
    const double f = 0.5 * (i + j);
    const double g = 0.5 * (i - j);
    const double h = a * c + b * d;
    return radius * std::sqrt(f + std::hypot(g, h));
}

// Slope.zig
struct Slope {
    double dx, dy;
};
inline Slope slope(Pt a, Pt b) { return Slope{b.x - a.x, b.y - a.y}; }
inline int fsign(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }
// Slope.compare (Slope.zig:46-85)
int compare(Slope a, Slope b) {
    const double fe = 2.220446049250313e-16;  // floatEps(f64)
    const double bdy = (std::fabs(b.dy - a.dy) > fe) ? b.dy : a.dy;
    const double bdx = (std::fabs(b.dx - a.dx) > fe) ? b.dx : a.dx;
    const int cmp = fsign(a.dy * bdx - bdy * a.dx);
    if (cmp != 0) return cmp;
    if (a.dx == 0 && a.dy == 0 && bdx == 0 && bdy == 0) return 0;
    if (a.dx == 0 && a.dy == 0) return 1;
    if (bdx == 0 && bdy == 0) return -1;
    if (fsign(a.dx) != fsign(bdx) || fsign(a.dy) != fsign(bdy)) return (a.dx > 0 || (a.dx == 0 && a.dy > 0)) ? -1 : 1;
    return 0;
}
// Slope.normalize (Slope.zig:117-146)
double normalize(Slope &s) {
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
        mag = std::hypot(s.dx, s.dy);
        rx = s.dx / mag;
        ry = s.dy / mag;
    }
    s.dx = rx;
    s.dy = ry;
    return mag;
}
inline Slope normalized(Slope s) {
    normalize(s);
    return s;
}
// Slope.compare_for_miter_limit (Slope.zig:88-105)
bool compare_for_miter_limit(Slope in, Slope out, double miter_limit) {
    const Slope a = normalized(in), b = normalized(out);
    const double in_dot_out = a.dx * b.dx + a.dy * b.dy;
    return 2 <= miter_limit * miter_limit * (1 + in_dot_out);
}

// Pen.zig
struct PenVertex {
    Pt point;
    Slope slope_cw, slope_ccw;
};
struct Pen {
    std::vector<PenVertex> v;
    bool ok = false;
};
// Pen.init (Pen.zig:25-88)
Pen make_pen(double thickness, double tolerance, const Tf &ctm) {
    Pen pen;
    pen.ok = true;
    const double radius = thickness / 2;
    int32_t n;
    const double major = transformed_circle_major_axis(ctm, radius);
    if (tolerance >= major * 4) {
        n = 1;
    } else if (tolerance >= major) {
        n = 4;
    } else {
        const double delta = std::acos(1 - tolerance / major);
        if (delta == 0) {
            n = 4;
        } else {
            const double nf = std::ceil(2 * M_PI / delta);
            const int32_t k = (int32_t)nf;
            n = k < 4 ? 4 : ((k % 2 != 0) ? k + 1 : k);
        }
    }
    const bool reflect = determinant(ctm) < 0;
    pen.v.resize((size_t)std::max(0, n));
    for (int32_t i = 0; i < n; i++) {
        double t = 2 * M_PI * (double)i / (double)n;
        if (reflect) t = -t;
        double dx = radius * std::cos(t), dy = radius * std::sin(t);
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
// Pen.vertexIteratorFor (Pen.zig:100-195): the vertex indices to visit.
std::vector<int32_t> pen_vertices_for(const Pen &pen, Slope from, Slope to, bool clockwise) {
    const int32_t len = (int32_t)pen.v.size();
    int32_t start = 0, end = 0;
    auto V = [&](int32_t k) -> const PenVertex & { return pen.v[(size_t)k]; };
    if (len == 0) return {};
    if (clockwise) {
        int32_t low = 0, high = len, i = (low + high) >> 1;
        while (high - low > 1) {
            if (compare(V(i).slope_cw, from) < 0) low = i;
            else high = i;
            i = (low + high) >> 1;
        }
        if (compare(V(i).slope_cw, from) < 0) {
            i += 1;
            if (i == len) i = 0;
        }
        start = i;
        if (compare(to, V(i).slope_ccw) >= 0) {
            low = i;
            high = i + len;
            i = (low + high) >> 1;
            while (high - low > 1) {
                const int32_t j = i >= len ? i - len : i;
                if (compare(V(j).slope_cw, to) > 0) high = i;
                else low = i;
                i = (low + high) >> 1;
            }
            if (i >= len) i -= len;
        }
        end = i;
    } else {
        int32_t low = 0, high = len, i = (low + high) >> 1;
        while (high - low > 1) {
            if (compare(from, V(i).slope_ccw) < 0) low = i;
            else high = i;
            i = (low + high) >> 1;
        }
        if (compare(from, V(i).slope_ccw) < 0) {
            i += 1;
            if (i == len) i = 0;
        }
        start = i;
        if (compare(V(i).slope_cw, to) <= 0) {
            low = i;
            high = i + len;
            i = (low + high) >> 1;
            while (high - low > 1) {
                const int32_t j = i >= len ? i - len : i;
                if (compare(to, V(j).slope_ccw) > 0) high = i;
                else low = i;
                i = (low + high) >> 1;
            }
            if (i >= len) i -= len;
        }
        end = i;
    }
    // VertexIterator.next (Pen.zig:204-222)
    std::vector<int32_t> out;
    int32_t idx = std::max(0, start);
    const int32_t e = std::max(0, end);
    while (idx != e) {
        out.push_back(idx);
        if (clockwise) {
            idx += 1;
            if (idx == len) idx = 0;
        } else {
            if (idx == 0) idx = len;
            idx -= 1;
        }
        if (out.size() > (size_t)len + 1) break;  // cannot happen; guards a corrupt pen
    }
    return out;
}

// Face.zig
struct Face {
    Pt p0, p1;
    double width;
    Slope dev_slope, user_slope;
    double half_width;
    Pt p0_cw, p0_ccw, p1_cw, p1_ccw;
    Tf ctm;
};
Face face_init2(Pt p0, Pt p1, Slope dev_slope, double thickness, const Tf &ctm) {
    const double half = thickness / 2;
    double ox, oy;
    Slope user_slope = dev_slope;
    if (!tf_equal(ctm, kIdentity)) {
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
    f.ctm = ctm;
    return f;
}
// Face.init (Face.zig:41-48)
Face face_init(Pt p0, Pt p1, double thickness, const Tf &ctm) {
    return face_init2(p0, p1, normalized(slope(p0, p1)), thickness, ctm);
}
// Face.intersect (Face.zig:96-125)
Pt intersect(const Face &in, const Face &out, bool clockwise) {
    const Pt ip = clockwise ? in.p1_ccw : in.p1_cw;
    const Pt op = clockwise ? out.p0_ccw : out.p0_cw;
    const Slope is = normalized(in.dev_slope), os = normalized(out.dev_slope);
    const double ry = ((op.x - ip.x) * is.dy * os.dy - op.y * os.dx * is.dy + ip.y * is.dx * os.dy) /
                      (is.dx * os.dy - os.dx * is.dy);
    const double rx = (std::fabs(is.dy) >= std::fabs(os.dy)) ? (ry - ip.y) * is.dx / is.dy + ip.x
                                                              : (ry - op.y) * os.dx / os.dy + op.x;
    return Pt{rx, ry};
}

// Polygon.Contour: a doubly linked list of scaled points.
struct Contour {
    std::list<Pt> pts;
    double scale = 1;
    using It = std::list<Pt>::iterator;
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
    std::vector<std::vector<double>> &result;
    int error = 0;

    Common(const Options &opts, std::vector<std::vector<double>> &res) : o(opts), result(res) {
        ctm = Tf{o.ctm[0], o.ctm[1], o.ctm[2], o.ctm[3], o.ctm[4], o.ctm[5]};
        if (o.join == kJoinRound || o.cap == kCapRound) pen = make_pen(o.thickness, o.tolerance, ctm);
    }

    // Polygon.addEdgesFromContour: the contour's points, closed later
    void emit(const Contour &c) {
        std::vector<double> pts;
        pts.reserve(c.pts.size() * 2);
        for (const Pt &p : c.pts) {
            pts.push_back(p.x);
            pts.push_back(p.y);
        }
        result.push_back(std::move(pts));
    }

    // join (stroke_plotter.zig:405-545)
    void join(Side &sd, int mode, Pt p0, Pt p1, Pt p2, bool use_before, Contour::It before_outer) {
        if (eq(p0, p1) || eq(p1, p2)) {
            if (sd.clockwise < 0) sd.clockwise = 0;
            return;
        }
        const Face in = face_init(p0, p1, o.thickness, ctm);
        const Face out = face_init(p1, p2, o.thickness, ctm);
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
            for (int32_t k : pen_vertices_for(pen, in.dev_slope, out.dev_slope, jcw)) {
                const Pt v = pen.v[(size_t)k].point;
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
            user_to_device_distance(f.ctm, ox, oy);
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
            for (int32_t k : pen_vertices_for(pen, f.dev_slope, Slope{-f.dev_slope.dx, -f.dev_slope.dy}, cw)) {
                const Pt v = pen.v[(size_t)k].point;
                sink(Pt{f.p1.x + v.x, f.p1.y + v.y});
            }
            sink(cw ? f.p1_cw : f.p1_ccw);
        }
    }
    template <class Sink>
    void cap_p0(const Face &f, bool cw, Sink &&sink) {
        cap(face_init(f.p1, f.p0, f.width, f.ctm), cw, sink);
    }

    void clear(Side &sd) {
        sd.outer.pts.clear();
        sd.inner.pts.clear();
        sd.clockwise = -1;
    }

    // plotSingle (stroke_plotter.zig:232-279)
    void plot_single(Side &sd, Pt start, Pt end) {
        const Face f = face_init(start, end, o.thickness, ctm);
        auto sink = [&](Pt p) { sd.outer.plot(p); };
        cap_p0(f, true, sink);
        cap(f, true, sink);
        emit(sd.outer);
        sd.outer.pts.clear();
        sd.clockwise = -1;
    }

    // plotOpenJoined (stroke_plotter.zig:281-363)
    void plot_open_joined(Side &sd, Pt s0, Pt e0, Pt s1, Pt e1) {
        const Face fs = face_init(s0, e0, o.thickness, ctm);
        const Face fe = face_init(s1, e1, o.thickness, ctm);
        const bool cw = sd.clockwise >= 0 ? sd.clockwise != 0 : true;
        const Contour::It first = sd.outer.pts.begin();  // the insertion point is captured before plotting
        auto before_first = [&](Pt p) { sd.outer.plot(p, first); };
        cap_p0(fs, cw, before_first);
        auto append = [&](Pt p) { sd.outer.plot(p); };
        cap(fe, cw, append);
        sd.outer.pts.splice(sd.outer.pts.end(), sd.inner.pts);
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
            const Face f = face_init2(p, p, slope, o.thickness, ctm);
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

    SolidPlotter(const Options &opts, std::vector<std::vector<double>> &res) : Common(opts, res) {
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

    DashedPlotter(const Options &opts, std::vector<std::vector<double>> &res) : Common(opts, res) {
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
            init_side.outer.pts.splice(init_side.outer.pts.end(), sd.outer.pts);
            init_side.inner.pts.splice(init_side.inner.pts.end(), sd.inner.pts);
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
            sd.outer.pts.splice(sd.outer.pts.end(), init_side.outer.pts);
            init_side.inner.pts.splice(init_side.inner.pts.end(), sd.inner.pts);
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

template <class P>
int run(P &p, const z2d_node *nodes, size_t n_nodes) {
    for (size_t i = 0; i < n_nodes && p.error == 0; i++) {
        const z2d_node &nd = nodes[i];
        switch (nd.tag) {
            case Z2D_MOVE_TO: p.move_to(Pt{nd.p[0], nd.p[1]}); break;
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

int plot(const z2d_node *nodes, size_t n_nodes, const Options &opts, std::vector<std::vector<double>> &contours) {
    contours.clear();
    if (dashed(opts)) {  // stroke_plotter.plot (stroke_plotter.zig:40-44)
        DashedPlotter p(opts, contours);
        return run(p, nodes, n_nodes);
    }
    SolidPlotter p(opts, contours);
    return run(p, nodes, n_nodes);
}

}  // namespace stroke
}  // namespace z2dg
