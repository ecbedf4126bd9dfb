// z2d_path.cpp -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.
//
// The oracle's restatement of z2d's Path builder, written from the
// reference's Zig sources (paths inside the z2d project) independently of
// the library's device builder:
//   Path.moveTo / lineTo / curveTo / rel* / close / reset  src/Path.zig:108-479
//   clampI24                                               src/Path.zig:570-572
//   Path.arc / arcNegative, arc_line_to / arc_curve_to     src/Path.zig:345-425
//   arc_in_direction and its helpers                       src/internal/arc.zig:39-392
//   Transformation mul / inverse / userToDevice            src/Transformation.zig:63-220
//   Outline.init / runOutline (simple glyphs) / appendToPath / quadCurveTo
//                                                          src/internal/Glyph.zig:483-869
// The builder keeps z2d's structure: nodes in a vector, the arc recursion as
// recursion, the outline built whole into its own path and then replayed.
// Zig's f64 sin / cos / tan are its compiler_rt ports of musl (kernels
// k_sin / k_cos / k_tan and __rem_pio2 from FreeBSD msun) and std.math.pow
// is Go's algorithm; they are restated here from those published sources.
// Zig folds `math.pi / k` in f128 at compile time, which gives other f64
// values than the f64 division for k = 3 and 6; the table uses the f128
// results.  std.math.hypot is not in the reference tree: hypot(g, h) is
// sqrt(g*g + h*h) here and in the library.
//
// Export: z2doracle_build_paths, with z2dgpu_build_paths' layout.
#include "../include/z2dgpu.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

uint64_t bits_of(double d) {
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return u;
}
double from_bits(uint64_t u) {
    double d;
    std::memcpy(&d, &u, 8);
    return d;
}
uint32_t high_word(double d) { return (uint32_t)(bits_of(d) >> 32); }

// ------------------------------------------------ musl's f64 trigonometry
// e_rem_pio2.c, medium arguments only (|x| < 2^20 pi/2); false otherwise
bool rem_pio2(double x, int &n, double y[2]) {
    static const double toint = 1.5 / 2.220446049250313080847e-16, pio4 = 7.85398163397448278999e-01,
                        invpio2 = 6.36619772367581382433e-01, pio2_1 = 1.57079632673412561417e+00,
                        pio2_1t = 6.07710050650619224932e-11, pio2_2 = 6.07710050630396597660e-11,
                        pio2_2t = 2.02226624879595063154e-21, pio2_3 = 2.02226624871116645580e-21,
                        pio2_3t = 8.47842766036889956997e-32;
    const int sign = (int)(bits_of(x) >> 63);
    const uint32_t ix = high_word(x) & 0x7fffffff;
    // |x| ~<= 9pi/4 away from the multiples of pi/2 that cancel: k * pi/2
    // subtracted in one step
    auto small_step = [&](int k) {
        const double z = sign ? x + k * pio2_1 : x - k * pio2_1;
        y[0] = sign ? z + k * pio2_1t : z - k * pio2_1t;
        y[1] = sign ? (z - y[0]) + k * pio2_1t : (z - y[0]) - k * pio2_1t;
        n = sign ? -k : k;
        return true;
    };
    bool medium = false;
    if (ix <= 0x400f6a7a) {
        if ((ix & 0xfffff) == 0x921fb) medium = true;
        else if (ix <= 0x4002d97c) return small_step(1);
        else return small_step(2);
    } else if (ix <= 0x401c463b) {
        if (ix <= 0x4015fdbc) {
            if (ix == 0x4012d97c) medium = true;
            else return small_step(3);
        } else {
            if (ix == 0x401921fb) medium = true;
            else return small_step(4);
        }
    }
    if (!medium && ix >= 0x413921fb) return false;
    double fn = x * invpio2 + toint - toint;
    n = (int32_t)fn;
    double r = x - fn * pio2_1, w = fn * pio2_1t;
    if (r - w < -pio4) {
        n--;
        fn--;
        r = x - fn * pio2_1;
        w = fn * pio2_1t;
    } else if (r - w > pio4) {
        n++;
        fn++;
        r = x - fn * pio2_1;
        w = fn * pio2_1t;
    }
    y[0] = r - w;
    const int ex = (int)(ix >> 20);
    int ey = (int)(bits_of(y[0]) >> 52 & 0x7ff);
    if (ex - ey > 16) {
        double t = r;
        w = fn * pio2_2;
        r = t - w;
        w = fn * pio2_2t - ((t - r) - w);
        y[0] = r - w;
        ey = (int)(bits_of(y[0]) >> 52 & 0x7ff);
        if (ex - ey > 49) {
            t = r;
            w = fn * pio2_3;
            r = t - w;
            w = fn * pio2_3t - ((t - r) - w);
            y[0] = r - w;
        }
    }
    y[1] = (r - y[0]) - w;
    return true;
}

double kernel_sin(double x, double y, int iy) {  // k_sin.c
    static const double S1 = -1.66666666666666324348e-01, S2 = 8.33333333332248946124e-03,
                        S3 = -1.98412698298579493134e-04, S4 = 2.75573137070700676789e-06,
                        S5 = -2.50507602534068634195e-08, S6 = 1.58969099521155010221e-10;
    const double z = x * x, w = z * z;
    const double r = S2 + z * (S3 + z * S4) + z * w * (S5 + z * S6);
    const double v = z * x;
    return iy == 0 ? x + v * (S1 + z * r) : x - ((z * (0.5 * y - v * r) - y) - v * S1);
}
double kernel_cos(double x, double y) {  // k_cos.c
    static const double C1 = 4.16666666666666019037e-02, C2 = -1.38888888888741095749e-03,
                        C3 = 2.48015872894767294178e-05, C4 = -2.75573143513906633035e-07,
                        C5 = 2.08757232129817482790e-09, C6 = -1.13596475577881948265e-11;
    const double z = x * x, w = z * z;
    const double r = z * (C1 + z * (C2 + z * C3)) + w * w * (C4 + z * (C5 + z * C6));
    const double hz = 0.5 * z, ww = 1.0 - hz;
    return ww + (((1.0 - ww) - hz) + (z * r - x * y));
}
double kernel_tan(double x, double y, int odd) {  // k_tan.c
    static const double T[13] = {3.33333333333334091986e-01,  1.33333333333201242699e-01, 5.39682539762260521377e-02,
                                 2.18694882948595424599e-02,  8.86323982359930005737e-03, 3.59207910759131235356e-03,
                                 1.45620945432529025516e-03,  5.88041240820264096874e-04, 2.46463134818469906812e-04,
                                 7.81794442939557092300e-05,  7.14072491382608190305e-05, -1.85586374855275456654e-05,
                                 2.59073051863633712884e-05};
    static const double pio4 = 7.85398163397448278999e-01, pio4lo = 3.06161699786838301793e-17;
    const uint32_t hx = high_word(x);
    const bool big = (hx & 0x7fffffff) >= 0x3FE59428;
    const bool sign = (hx >> 31) != 0;
    if (big) {
        if (sign) {
            x = -x;
            y = -y;
        }
        x = (pio4 - x) + (pio4lo - y);
        y = 0.0;
    }
    const double z = x * x, w = z * z;
    double r = T[1] + w * (T[3] + w * (T[5] + w * (T[7] + w * (T[9] + w * T[11]))));
    const double v = z * (T[2] + w * (T[4] + w * (T[6] + w * (T[8] + w * (T[10] + w * T[12])))));
    const double s = z * x;
    r = y + z * (s * (r + v) + y) + s * T[0];
    const double sum = x + r;
    if (big) {
        const double sg = 1 - 2 * odd;
        const double vv = sg - 2.0 * (x + (r - sum * sum / (sum + sg)));
        return sign ? -vv : vv;
    }
    if (!odd) return sum;
    const double w0 = from_bits(bits_of(sum) & 0xffffffff00000000ull);
    const double vv = r - (w0 - x);
    const double a = -1.0 / sum;
    const double a0 = from_bits(bits_of(a) & 0xffffffff00000000ull);
    return a0 + a * (1.0 + a0 * w0 + a0 * vv);
}

struct BadAngle {};  // an argument beyond the medium reduction range

double zsin(double x) {
    const uint32_t ix = high_word(x) & 0x7fffffff;
    if (ix <= 0x3fe921fb) return ix < 0x3e500000 ? x : kernel_sin(x, 0.0, 0);
    if (ix >= 0x7ff00000) return x - x;
    int n;
    double y[2];
    if (!rem_pio2(x, n, y)) throw BadAngle{};
    switch (n & 3) {
        case 0: return kernel_sin(y[0], y[1], 1);
        case 1: return kernel_cos(y[0], y[1]);
        case 2: return -kernel_sin(y[0], y[1], 1);
        default: return -kernel_cos(y[0], y[1]);
    }
}
double zcos(double x) {
    const uint32_t ix = high_word(x) & 0x7fffffff;
    if (ix <= 0x3fe921fb) return ix < 0x3e46a09e ? 1.0 : kernel_cos(x, 0.0);
    if (ix >= 0x7ff00000) return x - x;
    int n;
    double y[2];
    if (!rem_pio2(x, n, y)) throw BadAngle{};
    switch (n & 3) {
        case 0: return kernel_cos(y[0], y[1]);
        case 1: return -kernel_sin(y[0], y[1], 1);
        case 2: return -kernel_cos(y[0], y[1]);
        default: return kernel_sin(y[0], y[1], 1);
    }
}
double ztan(double x) {
    const uint32_t ix = high_word(x) & 0x7fffffff;
    if (ix <= 0x3fe921fb) return ix < 0x3e400000 ? x : kernel_tan(x, 0.0, 0);
    if (ix >= 0x7ff00000) return x - x;
    int n;
    double y[2];
    if (!rem_pio2(x, n, y)) throw BadAngle{};
    return kernel_tan(y[0], y[1], n & 1);
}

// std.math.pow(f64, x, y) for a positive integer y and finite nonzero x:
// frexp, square-and-multiply with the exponent apart, ldexp
double zpow_int(double x, int y) {
    if (y == 0 || x == 1.0) return 1.0;
    if (y == 1) return x;
    int xe;
    double x1 = std::frexp(x, &xe);
    double a1 = 1.0;
    int ae = 0;
    for (long long i = y; i != 0; i >>= 1) {
        if (xe < -(1 << 12) || (1 << 12) < xe) {
            ae += xe;
            break;
        }
        if (i & 1) {
            a1 *= x1;
            ae += xe;
        }
        x1 *= x1;
        xe <<= 1;
        if (x1 < 0.5) {
            x1 += x1;
            xe -= 1;
        }
    }
    return std::ldexp(a1, ae);
}

double zmod_f64(double a, double b) {  // @mod: fmod, into [0, b) for a negative a
    const double r = std::fmod(a, b);
    return a < 0.0 ? std::fmod(r + b, b) : r;
}

// ------------------------------------------------------ Transformation
struct Mat {
    double ax, by, cx, dy, tx, ty;
};
Mat mat_mul(const Mat &a, const Mat &b) {
    return Mat{a.ax * b.ax + a.by * b.cx,        a.ax * b.by + a.by * b.dy, a.cx * b.ax + a.dy * b.cx,
               a.cx * b.by + a.dy * b.dy,        a.ax * b.tx + a.by * b.ty + a.tx,
               a.cx * b.tx + a.dy * b.ty + a.ty};
}
bool mat_inverse(const Mat &a, Mat &o) {
    if (a.by == 0 && a.cx == 0) {
        if (a.ax == 0 || a.dy == 0) return false;
        if (a.ax != 1 || a.dy != 1) o = Mat{1 / a.ax, 0, 0, 1 / a.dy, -a.tx / a.ax, -a.ty / a.dy};
        else o = Mat{1, 0, 0, 1, -a.tx, -a.ty};
        return true;
    }
    const double det = a.ax * a.dy - a.by * a.cx;
    if (det == 0) return false;
    const double k = 1 / det;
    const Mat adj{a.dy, -a.by, -a.cx, a.ax, a.by * a.ty - a.dy * a.tx, a.cx * a.tx - a.ax * a.ty};
    o = Mat{adj.ax * k, adj.by * k, adj.cx * k, adj.dy * k, adj.tx * k, adj.ty * k};
    return true;
}
void user_to_device(const Mat &m, double &x, double &y) {
    const double ix = x, iy = y;
    x = m.ax * ix + m.by * iy;
    y = m.cx * ix + m.dy * iy;
    x += m.tx;
    y += m.ty;
}

struct PathError {
    int code;
};

// ----------------------------------------------------------------- Path
struct Path {
    std::vector<z2d_node> nodes;
    bool has_init = false, has_cur = false;
    double ix = 0, iy = 0, cx = 0, cy = 0;
    double tolerance = 0.1;
    Mat tf{1, 0, 0, 1, 0, 0};

    static double clamp24(double v) { return std::fmax(-8388608.0, std::fmin(v, 8388607.0)); }
    void add(int tag, std::initializer_list<double> pts) {
        z2d_node n;
        std::memset(&n, 0, sizeof n);
        n.tag = tag;
        int k = 0;
        for (double v : pts) n.p[k++] = v;
        nodes.push_back(n);
    }
    void mapped(double x, double y, double &ox, double &oy) const {
        ox = clamp24(x);
        oy = clamp24(y);
        user_to_device(tf, ox, oy);
    }
    void move_to(double x, double y) {
        double px, py;
        mapped(x, y, px, py);
        if (!nodes.empty() && nodes.back().tag == Z2D_MOVE_TO && nodes.back().p[0] == px && nodes.back().p[1] == py)
            return;
        add(Z2D_MOVE_TO, {px, py});
        has_init = has_cur = true;
        ix = cx = px;
        iy = cy = py;
    }
    void line_to(double x, double y) {
        if (!has_cur) return move_to(x, y);
        double px, py;
        mapped(x, y, px, py);
        add(Z2D_LINE_TO, {px, py});
        cx = px;
        cy = py;
    }
    void curve_to(double x1, double y1, double x2, double y2, double x3, double y3) {
        if (!has_cur) throw PathError{Z2D_ERR_INVALID_STATE};
        double a, b, c, d, e, f;
        mapped(x1, y1, a, b);
        mapped(x2, y2, c, d);
        mapped(x3, y3, e, f);
        add(Z2D_CURVE_TO, {a, b, c, d, e, f});
        cx = e;
        cy = f;
    }
    void user_current(double &x, double &y) const {
        if (!has_cur) throw PathError{Z2D_ERR_INVALID_STATE};
        Mat inv;
        if (!mat_inverse(tf, inv)) throw PathError{Z2D_ERR_INVALID_ARGUMENT};
        x = cx;
        y = cy;
        user_to_device(inv, x, y);
    }
    void close() {
        if (!has_cur) return;
        add(Z2D_CLOSE_PATH, {});
        add(Z2D_MOVE_TO, {ix, iy});
    }
    void reset() {
        nodes.clear();
        has_init = has_cur = false;
    }

    // ---- arcs (arc.zig)
    static double arc_error(double angle) {
        return 2.0 / 27.0 * zpow_int(zsin(angle / 4), 6) / zpow_int(zcos(angle / 4), 2);
    }
    static double max_angle_for(double tolerance) {
        static const double angle[11] = {
            3.141592653589793116, 1.570796326794896558, from_bits(0x3FF0C152382D7366ull), 0.7853981633974482790,
            from_bits(0x3FE41B2F769CF0E0ull), from_bits(0x3FE0C152382D7366ull), from_bits(0x3FDCB91F3BBBA140ull),
            0.3926990816987241395, from_bits(0x3FD657184AE74487ull), from_bits(0x3FD41B2F769CF0E0ull),
            from_bits(0x3FD247426BD47DE3ull)};
        static const double err[11] = {0.0185185185185185036127, 0.000272567143730179811158, 2.38647043651461047433e-05,
                                       4.2455377443222443279e-06, 1.11281001494389081528e-06, 3.72662000942734705475e-07,
                                       1.47783685574284411325e-07, 6.63240432022601149057e-08,
                                       3.2715520137536980553e-08, 1.73863223499021216974e-08, 9.81410988043554039085e-09};
        for (int i = 0; i < 11; i++)
            if (err[i] < tolerance) return angle[i];
        double a = 0;
        for (int i = 11; i < 1000; i++) {
            a = 3.141592653589793116 / (double)i;
            if (arc_error(a) <= tolerance) break;
        }
        return a;
    }
    static double major_axis(const Mat &m, double radius) {
        const double eps = 0.00390625;
        const double det = m.ax * m.dy - m.by * m.cx;
        if (std::fabs(det * det - 1.0) < eps) {
            if (std::fabs(m.by) < eps && std::fabs(m.cx) < eps) return radius;
            if (std::fabs(m.ax) < eps && std::fabs(m.dy) < eps) return radius;
        }
        const double i = m.ax * m.ax + m.by * m.by, j = m.cx * m.cx + m.dy * m.dy;
        const double f = 0.5 * (i + j), g = 0.5 * (i - j), h = m.ax * m.cx + m.by * m.dy;
        return radius * std::sqrt(f + std::sqrt(g * g + h * h));
    }
    void arc_line(double x, double y) {
        if (has_cur && cx == x && cy == y) return;
        line_to(x, y);
    }
    void arc_segment(double xc, double yc, double r, double a, double b) {
        const double rsa = r * zsin(a), rca = r * zcos(a), rsb = r * zsin(b), rcb = r * zcos(b);
        const double h = 4.0 / 3.0 * ztan((b - a) / 4.0);
        curve_to(xc + rca - h * rsa, yc + rsa + h * rca, xc + rcb + h * rsb, yc + rsb - h * rcb, xc + rcb, yc + rsb);
    }
    void arc_in_direction(double xc, double yc, double r, double amin, double amax, bool forward, double tol) {
        if (!(amax * amax >= 0.0) || !(amin * amin >= 0.0)) return;
        const double twopi = 2 * 3.141592653589793116;
        if (amax - amin > twopi * 65536.0) {
            amax = zmod_f64(amax - amin, twopi);
            amin = zmod_f64(amin, twopi);
            amax += amin + twopi * 65536.0;
        }
        if (amax - amin > 3.141592653589793116) {
            const double amid = amin + (amax - amin) / 2.0;
            if (forward) {
                arc_in_direction(xc, yc, r, amin, amid, forward, tol);
                arc_in_direction(xc, yc, r, amid, amax, forward, tol);
            } else {
                arc_in_direction(xc, yc, r, amid, amax, forward, tol);
                arc_in_direction(xc, yc, r, amin, amid, forward, tol);
            }
        } else if (amax != amin) {
            int segments = (int)std::ceil(std::fabs(amax - amin) / max_angle_for(tol / major_axis(tf, r)));
            double step = (amax - amin) / (double)segments;
            segments -= 1;
            if (!forward) {
                std::swap(amin, amax);
                step = -step;
            }
            arc_line(xc + r * zcos(amin), yc + r * zsin(amin));
            for (int s = 0; s < segments; s++) {
                arc_segment(xc, yc, r, amin, amin + step);
                amin += step;
            }
            arc_segment(xc, yc, r, amin, amax);
        } else {
            arc_line(xc + r * zcos(amin), yc + r * zsin(amin));
        }
    }
    void arc(double xc, double yc, double r, double a1, double a2, bool negative) {
        const double twopi = 3.141592653589793116 * 2;
        const double tol = std::fmax(tolerance, 0.001);
        long guard = 0;
        if (!negative) {
            while (a2 < a1) {
                a2 += twopi;
                if (++guard > (1 << 22)) throw PathError{Z2D_ERR_INVALID_ARGUMENT};
            }
            arc_in_direction(xc, yc, r, a1, a2, true, tol);
        } else {
            while (a2 > a1) {
                a2 -= twopi;
                if (++guard > (1 << 22)) throw PathError{Z2D_ERR_INVALID_ARGUMENT};
            }
            arc_in_direction(xc, yc, r, a2, a1, false, tol);
        }
    }
};

// ----------------------------------------------------------- glyphs
// Outline.init + runOutline (simple glyph) + appendToPath
void append_glyph(Path &path, const z2d_glyph_point *pts, int n, const uint16_t *ends, int n_ends, double upem) {
    Path o;
    o.tolerance = path.tolerance;
    const Mat id{1, 0, 0, 1, 0, 0};
    o.tf = mat_mul(mat_mul(id, Mat{1.0, 0, 0, -1.0, 0, 0}), Mat{1, 0, 0, 1, 0.0, upem * -1.0});
    auto is_end = [&](int i) {
        for (int k = 0; k < n_ends; k++)
            if (ends[k] == i) return true;
        return false;
    };
    auto quad = [&](int cx_, int cy_, int tx, int ty) {
        if (!o.has_cur) throw PathError{Z2D_ERR_INVALID_ARGUMENT};  // MalformedGlyph
        double x0, y0;
        o.user_current(x0, y0);
        const double x3 = tx, y3 = ty;
        o.curve_to(x0 + 2.0 / 3.0 * ((double)cx_ - x0), y0 + 2.0 / 3.0 * ((double)cy_ - y0),
                   x3 + 2.0 / 3.0 * ((double)cx_ - x3), y3 + 2.0 / 3.0 * ((double)cy_ - y3), x3, y3);
    };
    int state = 0;  // 0 move_to, 1 on curve, 2 off curve
    int j = 0;
    for (int i = 0; i < n; i++) {
        const bool on = (pts[i].flags & 1) != 0;
        if (state == 0) {
            if (!on || is_end(i)) continue;
            o.move_to(pts[i].x, pts[i].y);
            j = i;
            state = 1;
        } else if (state == 1) {
            if (!on) state = 2;
            else o.line_to(pts[i].x, pts[i].y);
        } else {
            if (on) {
                quad(pts[i - 1].x, pts[i - 1].y, pts[i].x, pts[i].y);
                state = 1;
            } else {
                quad(pts[i - 1].x, pts[i - 1].y, (int16_t)((pts[i].x + pts[i - 1].x) >> 1),
                     (int16_t)((pts[i].y + pts[i - 1].y) >> 1));
            }
        }
        if (is_end(i)) {
            if (state == 2) quad(pts[i].x, pts[i].y, pts[j].x, pts[j].y);
            o.close();
            state = 0;
        }
    }
    for (const z2d_node &nd : o.nodes) {
        switch (nd.tag) {
            case Z2D_MOVE_TO: path.move_to(nd.p[0], nd.p[1]); break;
            case Z2D_LINE_TO: path.line_to(nd.p[0], nd.p[1]); break;
            case Z2D_CURVE_TO: path.curve_to(nd.p[0], nd.p[1], nd.p[2], nd.p[3], nd.p[4], nd.p[5]); break;
            default: path.close(); break;
        }
    }
}

}  // namespace

extern "C" {

// Zig's f64 sin (0), cos (1) and tan (2) as restated here; *ok = 0 beyond
// the medium reduction range.
__attribute__((visibility("default"))) double z2doracle_zig_trig(int which, double x, int *ok) {
    *ok = 1;
    try {
        return which == 0 ? zsin(x) : which == 1 ? zcos(x) : ztan(x);
    } catch (const BadAngle &) {
        *ok = 0;
        return 0.0;
    }
}

__attribute__((visibility("default"))) int z2doracle_build_paths(
    const z2d_path_program *progs, size_t n_progs, const z2d_path_cmd *cmds, size_t n_cmds,
    const z2d_glyph_point *gpts, size_t n_gpts, const uint16_t *gends, size_t n_gends, z2d_node *nodes,
    size_t cap_nodes, uint64_t *offsets, int32_t *status) {
    std::vector<std::vector<z2d_node>> built(n_progs);
    for (size_t p = 0; p < n_progs; p++) {
        const z2d_path_program &pg = progs[p];
        if (pg.cmd_offset > n_cmds || pg.n_cmds > n_cmds - pg.cmd_offset) return Z2D_ERR_INVALID_ARGUMENT;
        Path path;
        const double *t = pg.transformation;
        path.tf = Mat{t[0], t[1], t[2], t[3], t[4], t[5]};
        path.tolerance = pg.tolerance;
        int err = 0;
        for (uint64_t k = 0; k < pg.n_cmds && !err; k++) {
            const z2d_path_cmd &c = cmds[pg.cmd_offset + k];
            const double *v = c.v;
            try {
                double ux, uy;
                switch (c.op) {
                    case Z2D_PATH_MOVE_TO: path.move_to(v[0], v[1]); break;
                    case Z2D_PATH_LINE_TO: path.line_to(v[0], v[1]); break;
                    case Z2D_PATH_CURVE_TO: path.curve_to(v[0], v[1], v[2], v[3], v[4], v[5]); break;
                    case Z2D_PATH_REL_MOVE_TO:
                        path.user_current(ux, uy);
                        path.move_to(ux + v[0], uy + v[1]);
                        break;
                    case Z2D_PATH_REL_LINE_TO:
                        path.user_current(ux, uy);
                        path.line_to(ux + v[0], uy + v[1]);
                        break;
                    case Z2D_PATH_REL_CURVE_TO:
                        path.user_current(ux, uy);
                        path.curve_to(ux + v[0], uy + v[1], ux + v[2], uy + v[3], ux + v[4], uy + v[5]);
                        break;
                    case Z2D_PATH_ARC: path.arc(v[0], v[1], v[2], v[3], v[4], false); break;
                    case Z2D_PATH_ARC_NEGATIVE: path.arc(v[0], v[1], v[2], v[3], v[4], true); break;
                    case Z2D_PATH_CLOSE: path.close(); break;
                    case Z2D_PATH_SET_TRANSFORMATION: path.tf = Mat{v[0], v[1], v[2], v[3], v[4], v[5]}; break;
                    case Z2D_PATH_SET_TOLERANCE: path.tolerance = v[0]; break;
                    case Z2D_PATH_RESET: path.reset(); break;
                    case Z2D_PATH_GLYPH: {
                        const long long po = (long long)v[0], np = (long long)v[1], eo = (long long)v[2],
                                        ne = (long long)v[3];
                        if (po < 0 || np < 0 || eo < 0 || ne < 0 || po + np > (long long)n_gpts ||
                            eo + ne > (long long)n_gends || np > 0xFFFF || ne > 0xFFFF)
                            throw PathError{Z2D_ERR_INVALID_ARGUMENT};
                        // built whole first: on an error nothing is appended
                        Path trial = path;
                        append_glyph(trial, gpts + po, (int)np, gends + eo, (int)ne, v[4]);
                        path = trial;
                        break;
                    }
                    default: throw PathError{Z2D_ERR_INVALID_ARGUMENT};
                }
            } catch (const PathError &e) {
                err = e.code;
            } catch (const BadAngle &) {
                err = Z2D_ERR_INVALID_ARGUMENT;
            }
        }
        built[p] = std::move(path.nodes);
        if (status) status[p] = err;
    }
    uint64_t tot = 0;
    for (size_t p = 0; p < n_progs; p++) {
        offsets[p] = tot;
        tot += built[p].size();
    }
    offsets[n_progs] = tot;
    if (tot > cap_nodes) return Z2D_ERR_OUT_OF_MEMORY;
    for (size_t p = 0; p < n_progs; p++)
        if (!built[p].empty()) std::memcpy(nodes + offsets[p], built[p].data(), sizeof(z2d_node) * built[p].size());
    return Z2D_OK;
}

}  // extern "C"
