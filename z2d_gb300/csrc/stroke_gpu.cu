// stroke_gpu.cu -- the stroke polygon of painter.stroke, tessellated on the
// device (solid strokes; the stages are listed in stroke_gpu.cuh).
//
// The polygon is the one stroke_plotter.Plotter builds
// (src/internal/tess/stroke_plotter.zig:77-403): per subpath, an outer
// contour that joins append to and an inner contour that joins prepend to;
// closed subpaths give both as separate contours, open ones one contour
// [start cap, outer, end cap, inner].  Every join and cap writes its points
// straight into their final contour positions, found by prefix sums over
// the elements' point counts, so the edges (consecutive contour points) are
// the reference's in its order.  Geometry is stroke_geom.h, shared with the
// host builder; the curve subdivision is spline.cuh, shared with fills.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include "edges.cuh"
#include "spline.cuh"
#include "stroke_geom.h"
#include "stroke_gpu.cuh"
#include "z2d_internal.h"

namespace z2dg {

using sg::Face;
using sg::PenVertex;
using sg::Pt;
using sg::Slope;
using sg::Tf;

namespace {

enum : int32_t { SK_NONE = 0, SK_OPEN = 1, SK_CLOSED = 2, SK_SINGLE = 3, SK_DOT = 4 };

// per subpath, after deduplication
struct SubState {
    int32_t q0, n;   // kept points [q0, q0 + n)
    int32_t kind;    // SK_*
    int32_t pcw;     // direction of the first join (the plotter's `clockwise`)
};
// per stroke: its outer points [a0, a0 + na) and inner points [b0, b0 + nb)
struct StrokeTot {
    long long a0, na, b0, nb;
};

// device pointers of one run
struct State {
    long long *raw_cnt, *raw_off;   // n_local + 1
    PenVertex *pen;                 // n_pen
    SubState *sub;                  // n_subs
    StrokeTot *tot;                 // n_strokes
    long long *totals;              // outer, inner totals (read back)
    // sized by the raw point count R
    double2 *raw_pt;
    int32_t *raw_sub;
    uint8_t *raw_mode;
    int32_t *keep, *kept_off;       // R + 1
    double2 *q_pt;
    int32_t *q_sub;
    uint8_t *q_mode;
    long long *cnt_a, *cnt_b, *off_a, *off_b;  // R + 1
    // contour points
    double2 *pa, *pb;
};

__device__ __forceinline__ Tf tf_of(const StrokeDev &s) {
    return Tf{s.ctm[0], s.ctm[1], s.ctm[2], s.ctm[3], s.ctm[4], s.ctm[5]};
}
__device__ __forceinline__ Pt node_end(const z2d_node &nd) {
    return nd.tag == Z2D_CURVE_TO ? Pt{nd.p[4], nd.p[5]} : Pt{nd.p[0], nd.p[1]};
}

// ----------------------------------------------------------------- pens
// Pen.init (Pen.zig:25-88) from the host's cos/sin table: vertex points
// through the CTM, then the slopes to either neighbour.
__global__ void ks_pen(const StrokeDev *__restrict__ strokes, int32_t n_strokes, const double *__restrict__ trig,
                       PenVertex *__restrict__ pen) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_strokes) return;
    const StrokeDev S = strokes[s];
    const int32_t n = S.pen_n;
    if (n <= 0) return;
    const Tf ctm = tf_of(S);
    const double radius = S.thickness / 2;
    PenVertex *v = pen + S.pen_off;
    const double *t = trig + 2 * (size_t)S.pen_tab;
    for (int32_t i = 0; i < n; i++) {
        double dx = radius * t[2 * i], dy = radius * t[2 * i + 1];
        sg::user_to_device_distance(ctm, dx, dy);
        v[i].point = Pt{dx, dy};
    }
    for (int32_t i = 0; i < n; i++) {
        const int32_t next = (i >= n - 1) ? 0 : i + 1;
        const int32_t prev = max(0, i == 0 ? n - 1 : i - 1);
        v[i].slope_cw = sg::slope(v[prev].point, v[i].point);
        v[i].slope_ccw = sg::slope(v[i].point, v[next].point);
    }
}

// ------------------------------------------------------------ raw points
__global__ void ks_local_sub(const SubpathDev *__restrict__ subs, int32_t n_subs, int32_t *__restrict__ local_sub) {
    const int32_t sp = blockIdx.x * blockDim.x + threadIdx.x;
    if (sp >= n_subs) return;
    const SubpathDev S = subs[sp];
    for (int32_t j = 0; j < S.n_nodes; j++) local_sub[S.local0 + j] = sp;
}

// The points one node hands to the plotter: move_to its point, line_to its
// end, curve_to Spline.decompose's lineTo calls (stroke_plotter.zig:126-150).
template <class Emit>
__device__ __forceinline__ bool node_points(const z2d_node *__restrict__ nodes, const SubpathDev &S, int32_t j,
                                           double tol, Emit &&emit) {
    const z2d_node nd = nodes[S.node0 + j];
    if (j == 0 || nd.tag == Z2D_LINE_TO) {
        emit(nd.p[0], nd.p[1]);
        return true;
    }
    const Pt a = node_end(nodes[S.node0 + j - 1]);
    return spline_walk(a.x, a.y, nd.p, tol, emit);
}

__global__ void ks_raw_count(const z2d_node *__restrict__ nodes, const SubpathDev *__restrict__ subs,
                             const int32_t *__restrict__ local_sub, const StrokeDev *__restrict__ strokes,
                             long long n_local, long long *__restrict__ raw_cnt, int32_t *__restrict__ status) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n_local) return;
    if (i == n_local) {
        raw_cnt[i] = 0;
        return;
    }
    const int32_t sp = local_sub[i];
    const SubpathDev S = subs[sp];
    int32_t cnt = 0;
    if (!node_points(nodes, S, (int32_t)(i - S.local0), strokes[S.stroke].tolerance, [&](double, double) { cnt++; }))
        atomicExch(status, Z2D_ERR_INVALID_STATE);
    raw_cnt[i] = cnt;
}

__global__ void ks_raw_emit(const z2d_node *__restrict__ nodes, const SubpathDev *__restrict__ subs,
                            const int32_t *__restrict__ local_sub, const StrokeDev *__restrict__ strokes,
                            long long n_local, const long long *__restrict__ raw_off, long long n_raw,
                            double2 *__restrict__ raw_pt, int32_t *__restrict__ raw_sub,
                            uint8_t *__restrict__ raw_mode, int32_t *__restrict__ keep) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_local) {
        if (i == n_local) keep[n_raw] = 0;
        return;
    }
    const int32_t sp = local_sub[i];
    const SubpathDev S = subs[sp];
    const int32_t j = (int32_t)(i - S.local0);
    const StrokeDev &T = strokes[S.stroke];
    const z2d_node nd = nodes[S.node0 + j];
    // the previous point the plotter saw, for the degenerate-node check
    Pt prev = j == 0 ? Pt{nd.p[0], nd.p[1]} : node_end(nodes[S.node0 + j - 1]);
    const uint8_t mode = (j > 0 && nd.tag == Z2D_CURVE_TO) ? (uint8_t)Z2D_JOIN_ROUND : (uint8_t)T.join;
    long long r = raw_off[i];
    const long long r_end = raw_off[i + 1];
    bool first = true;
    node_points(nodes, S, j, T.tolerance, [&](double x, double y) {
        if (r < r_end) {
            raw_pt[r] = make_double2(x, y);
            raw_sub[r] = sp;
            raw_mode[r] = mode;
            keep[r] = (j == 0 && first) ? 1 : !sg::eq(Pt{x, y}, prev);
        }
        first = false;
        prev = Pt{x, y};
        r++;
    });
}

__global__ void ks_compact(const double2 *__restrict__ raw_pt, const int32_t *__restrict__ raw_sub,
                           const uint8_t *__restrict__ raw_mode, const int32_t *__restrict__ keep,
                           const int32_t *__restrict__ kept_off, long long n_raw, double2 *__restrict__ q_pt,
                           int32_t *__restrict__ q_sub, uint8_t *__restrict__ q_mode) {
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_raw || !keep[r]) return;
    const int32_t q = kept_off[r];
    q_pt[q] = raw_pt[r];
    q_sub[q] = raw_sub[r];
    q_mode[q] = raw_mode[r];
}

// close_path / finish of the plotter (stroke_plotter.zig:152-230): what a
// subpath of n kept points draws.
__global__ void ks_sub_setup(const SubpathDev *__restrict__ subs, int32_t n_subs, const StrokeDev *__restrict__ strokes,
                             const long long *__restrict__ raw_off, const int32_t *__restrict__ kept_off,
                             const double2 *__restrict__ q_pt, SubState *__restrict__ sub) {
    const int32_t sp = blockIdx.x * blockDim.x + threadIdx.x;
    if (sp >= n_subs) return;
    const SubpathDev S = subs[sp];
    const long long r0 = raw_off[S.local0], r1 = raw_off[S.local0 + S.n_nodes];
    SubState st;
    st.q0 = kept_off[r0];
    st.n = kept_off[r1] - st.q0;
    if (st.n >= 3) st.kind = S.closed ? SK_CLOSED : SK_OPEN;
    else if (st.n == 2) st.kind = SK_SINGLE;
    else if (st.n == 1 && S.closed && strokes[S.stroke].cap == Z2D_CAP_ROUND) st.kind = SK_DOT;
    else st.kind = SK_NONE;
    st.pcw = 1;
    if (st.n >= 3) {
        const double2 a = q_pt[st.q0], b = q_pt[st.q0 + 1], c = q_pt[st.q0 + 2];
        const Slope in = sg::normalized(Slope{b.x - a.x, b.y - a.y});
        const Slope out = sg::normalized(Slope{c.x - b.x, c.y - b.y});
        st.pcw = sg::compare(in, out) < 0 ? 1 : 0;
    }
    sub[sp] = st;
}

// ------------------------------------------------------------- elements
// Receives an element's points: A = appended to the outer contour, B =
// prepended to the inner one (in plot order).  Counting only when !EMIT.
template <bool EMIT>
struct Out {
    long long na = 0, nb = 0;
    double2 *pa = nullptr;      // A point k goes to pa[k]
    double2 *pb_end = nullptr;  // B point k goes to pb_end[-1 - k]
    double scale = 1;
    __device__ __forceinline__ void A(Pt p) {
        if (EMIT) pa[na] = make_double2(p.x * scale, p.y * scale);
        na++;
    }
    __device__ __forceinline__ void B(Pt p) {
        if (EMIT) pb_end[-1 - nb] = make_double2(p.x * scale, p.y * scale);
        nb++;
    }
    // pen vertices around c, to A or B
    __device__ __forceinline__ void pen(bool to_a, Pt c, const PenVertex *v, int32_t len, int32_t start,
                                        int32_t cnt, bool cw) {
        if (!EMIT) {
            (to_a ? na : nb) += cnt;
            return;
        }
        for (int32_t k = 0; k < cnt; k++) {
            const Pt p = v[sg::pen_step(start, k, len, cw)].point;
            const Pt q{c.x + p.x, c.y + p.y};
            if (to_a) A(q);
            else B(q);
        }
    }
};

// join (stroke_plotter.zig:405-545) at p1 between p0->p1 and p1->p2, with
// the subpath's first-join direction pcw.
template <class O>
__device__ __forceinline__ void join(O &o, const StrokeDev &T, const Tf &ctm, const PenVertex *pen, int mode, Pt p0,
                                     Pt p1, Pt p2, bool pcw) {
    if (sg::eq(p0, p1) || sg::eq(p1, p2)) return;
    const Face in = sg::face_init(p0, p1, T.thickness, ctm);
    const Face out = sg::face_init(p1, p2, T.thickness, ctm);
    const int cmp = sg::compare(in.dev_slope, out.dev_slope);
    const bool jcw = cmp < 0;
    const bool sw = jcw != pcw;  // outer and inner trade places
    auto outer = [&](Pt p) {
        if (sw) o.B(p);
        else o.A(p);
    };
    auto inner = [&](Pt p) {
        if (sw) o.A(p);
        else o.B(p);
    };
    if (cmp == 0) {
        outer(jcw ? in.p1_ccw : in.p1_cw);
        inner(jcw ? in.p1_cw : in.p1_ccw);
        return;
    }
    if (mode == Z2D_JOIN_MITER || mode == Z2D_JOIN_BEVEL) {
        if (mode == Z2D_JOIN_MITER && sg::compare_for_miter_limit(in.dev_slope, out.dev_slope, T.miter_limit)) {
            outer(sg::intersect(in, out, jcw));
        } else {
            outer(jcw ? in.p1_ccw : in.p1_cw);
            outer(jcw ? out.p0_ccw : out.p0_cw);
        }
    } else {
        outer(jcw ? in.p1_ccw : in.p1_cw);
        int32_t start;
        const int32_t cnt = sg::pen_range(pen, T.pen_n, in.dev_slope, out.dev_slope, jcw, start);
        o.pen(!sw, p1, pen, T.pen_n, start, cnt, jcw);
        outer(jcw ? out.p0_ccw : out.p0_cw);
    }
    inner(jcw ? in.p1_cw : in.p1_ccw);
    inner(p1);
    inner(jcw ? out.p0_cw : out.p0_ccw);
}

// Face.cap (Face.zig:156-246), to A
template <class O>
__device__ __forceinline__ void cap(O &o, const StrokeDev &T, const Tf &ctm, const PenVertex *pen, const Face &f,
                                    bool cw) {
    if (T.cap == Z2D_CAP_BUTT) {
        o.A(cw ? f.p1_ccw : f.p1_cw);
        o.A(cw ? f.p1_cw : f.p1_ccw);
    } else if (T.cap == Z2D_CAP_SQUARE) {
        double ox = f.user_slope.dx * f.half_width, oy = f.user_slope.dy * f.half_width;
        sg::user_to_device_distance(ctm, ox, oy);
        const Pt a = cw ? f.p1_ccw : f.p1_cw, b = cw ? f.p1_cw : f.p1_ccw;
        o.A(a);
        o.A(Pt{a.x + ox, a.y + oy});
        o.A(Pt{b.x + ox, b.y + oy});
        o.A(b);
    } else {
        o.A(cw ? f.p1_ccw : f.p1_cw);
        int32_t start;
        const int32_t cnt =
            sg::pen_range(pen, T.pen_n, f.dev_slope, Slope{-f.dev_slope.dx, -f.dev_slope.dy}, cw, start);
        o.pen(true, f.p1, pen, T.pen_n, start, cnt, cw);
        o.A(cw ? f.p1_cw : f.p1_ccw);
    }
}

// Everything element k of a subpath contributes (see stroke_gpu.cuh).
template <class O>
__device__ __forceinline__ void element(O &o, const StrokeDev &T, const PenVertex *pen, const SubState &st,
                                        const double2 *__restrict__ q_pt, const uint8_t *__restrict__ q_mode,
                                        int32_t k) {
    const int32_t n = st.n;
    auto P = [&](int32_t i) {
        const double2 v = q_pt[st.q0 + i];
        return Pt{v.x, v.y};
    };
    const Tf ctm = tf_of(T);
    const bool pcw = st.pcw != 0;
    // Every case below draws at most two caps or one join; they are
    // gathered into one cap call and one join call, so that the kernel
    // holds a single copy of each.
    int n_caps = 0, jmode = -1;
    Pt c0{}, c1{}, j0{}, j1{}, j2{};
    bool ccw = pcw;
    switch (st.kind) {
        case SK_DOT:  // plot_dot of stroke_plotter (round caps only)
            if (k == 0) {
                const Pt c = P(0);
                for (int32_t i = 0; i < T.pen_n; i++) o.A(Pt{c.x + pen[i].point.x, c.y + pen[i].point.y});
            }
            return;
        case SK_SINGLE:  // plotSingle (stroke_plotter.zig:232-279): caps of b->a, then a->b
            if (k != 0) return;
            n_caps = 2;
            c0 = P(1);
            c1 = P(0);
            ccw = true;
            break;
        case SK_OPEN:  // plotOpenJoined (stroke_plotter.zig:281-363)
            if (k == 0) {
                n_caps = 1;
                c0 = P(1);
                c1 = P(0);
            } else if (k == n - 1) {
                n_caps = 1;
                c0 = P(n - 2);
                c1 = P(n - 1);
            } else {
                jmode = q_mode[st.q0 + k + 1];
                j0 = P(k - 1);
                j1 = P(k);
                j2 = P(k + 1);
            }
            break;
        case SK_CLOSED: {  // plotClosedJoined (stroke_plotter.zig:365-403)
            const bool back_to_start = sg::eq(P(n - 1), P(0));
            if (k >= 1 && k <= n - 2) {
                jmode = q_mode[st.q0 + k + 1];
                j0 = P(k - 1);
                j1 = P(k);
                j2 = P(k + 1);
            } else if (k == n - 1) {
                if (back_to_start) return;
                jmode = T.join;
                j0 = P(n - 2);
                j1 = P(n - 1);
                j2 = P(0);
            } else {
                jmode = T.join;
                j0 = back_to_start ? P(n - 2) : P(n - 1);
                j1 = P(0);
                j2 = P(1);
            }
            break;
        }
        default: return;
    }
#pragma unroll 1
    for (int i = 0; i < n_caps; i++) {
        cap(o, T, ctm, pen, sg::face_init(c0, c1, T.thickness, ctm), ccw);
        const Pt t = c0;  // the second cap of plotSingle runs the other way
        c0 = c1;
        c1 = t;
    }
    if (jmode >= 0) join(o, T, ctm, pen, jmode, j0, j1, j2, pcw);
}

__global__ void ks_elem_count(const SubpathDev *__restrict__ subs, const StrokeDev *__restrict__ strokes,
                              const PenVertex *__restrict__ pen, const SubState *__restrict__ sub,
                              const double2 *__restrict__ q_pt, const int32_t *__restrict__ q_sub,
                              const uint8_t *__restrict__ q_mode, const int32_t *__restrict__ kept_off,
                              long long n_raw, long long *__restrict__ cnt_a, long long *__restrict__ cnt_b) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q > n_raw) return;
    const long long n_kept = kept_off[n_raw];
    if (q >= n_kept) {
        cnt_a[q] = 0;
        cnt_b[q] = 0;
        return;
    }
    const int32_t sp = q_sub[q];
    const SubState st = sub[sp];
    const StrokeDev T = strokes[subs[sp].stroke];
    Out<false> o;
    element(o, T, pen + T.pen_off, st, q_pt, q_mode, (int32_t)(q - st.q0));
    cnt_a[q] = o.na;
    cnt_b[q] = o.nb;
}

__global__ void ks_stroke_tot(const StrokeDev *__restrict__ strokes, int32_t n_strokes,
                              const SubState *__restrict__ sub, const long long *__restrict__ off_a,
                              const long long *__restrict__ off_b, long long n_raw, StrokeTot *__restrict__ tot,
                              int32_t *__restrict__ stroke_edges, long long *__restrict__ totals) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) {
        totals[0] = off_a[n_raw];
        totals[1] = off_b[n_raw];
    }
    if (s >= n_strokes) return;
    const StrokeDev S = strokes[s];
    StrokeTot t{0, 0, 0, 0};
    if (S.n_sub > 0) {
        const int32_t e0 = sub[S.sub0].q0;
        const SubState last = sub[S.sub0 + S.n_sub - 1];
        const int32_t e1 = last.q0 + last.n;
        t.a0 = off_a[e0];
        t.na = off_a[e1] - t.a0;
        t.b0 = off_b[e0];
        t.nb = off_b[e1] - t.b0;
    }
    tot[s] = t;
    const long long e = t.na + t.nb;
    stroke_edges[s] = e > 0x7FFFFFFFll ? -1 : (int32_t)e;
}

// Region layout of one element: where its A points start and where its B
// points end (B points are stored in contour order, i.e. reversed).
struct Place {
    long long ra, sa, rb, sb;  // the subpath's outer and inner regions
    long long pos_a, end_b;
};
__device__ __forceinline__ Place place(const SubState &st, int32_t k, long long q, const long long *__restrict__ off_a,
                                       const long long *__restrict__ off_b) {
    Place p;
    p.ra = off_a[st.q0];
    p.sa = off_a[st.q0 + st.n] - p.ra;
    p.rb = off_b[st.q0];
    p.sb = off_b[st.q0 + st.n] - p.rb;
    long long t_b;
    if (st.kind == SK_CLOSED) {
        // the closing joins come last: elements 1..n-1, then 0
        const long long a0 = off_a[st.q0 + 1] - p.ra, b0 = off_b[st.q0 + 1] - p.rb;
        p.pos_a = k >= 1 ? off_a[q] - a0 : p.ra + p.sa - a0;
        t_b = k >= 1 ? off_b[q] - p.rb - b0 : p.sb - b0;
    } else {
        p.pos_a = off_a[q];
        t_b = off_b[q] - p.rb;
    }
    p.end_b = p.rb + p.sb - t_b;
    return p;
}

__global__ void ks_elem_emit(const SubpathDev *__restrict__ subs, const StrokeDev *__restrict__ strokes,
                             const PenVertex *__restrict__ pen, const SubState *__restrict__ sub,
                             const double2 *__restrict__ q_pt, const int32_t *__restrict__ q_sub,
                             const uint8_t *__restrict__ q_mode, const int32_t *__restrict__ kept_off, long long n_raw,
                             const long long *__restrict__ off_a, const long long *__restrict__ off_b,
                             double2 *__restrict__ pa, double2 *__restrict__ pb) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kept_off[n_raw]) return;
    const int32_t sp = q_sub[q];
    const SubState st = sub[sp];
    const int32_t k = (int32_t)(q - st.q0);
    const StrokeDev T = strokes[subs[sp].stroke];
    const Place pl = place(st, k, q, off_a, off_b);
    Out<true> o;
    o.pa = pa + pl.pos_a;
    o.pb_end = pb + pl.end_b;
    o.scale = T.scale;
    element(o, T, pen + T.pen_off, st, q_pt, q_mode, k);
}

// Polygon.addEdgesFromContour: every contour point to the next one (the
// last back to the first).  An open subpath's contour is its outer region
// followed by its inner region.
__global__ void ks_edges(const SubpathDev *__restrict__ subs, const StrokeDev *__restrict__ strokes,
                         const SubState *__restrict__ sub, const int32_t *__restrict__ q_sub,
                         const int32_t *__restrict__ kept_off, long long n_raw, const long long *__restrict__ cnt_a,
                         const long long *__restrict__ cnt_b, const long long *__restrict__ off_a,
                         const long long *__restrict__ off_b, const StrokeTot *__restrict__ tot,
                         const double2 *__restrict__ pa, const double2 *__restrict__ pb,
                         const FillCmd *__restrict__ fills, FillState *__restrict__ st_fill,
                         DEdge *__restrict__ edges) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = q < kept_off[n_raw];
    int32_t f = -1;
    double et = 0, eb = 0, el = 0, er = 0;
    bool any = false;
    if (live) {
        const int32_t sp = q_sub[q];
        const SubState st = sub[sp];
        const int32_t k = (int32_t)(q - st.q0);
        const int32_t s = subs[sp].stroke;
        f = strokes[s].fill;
        const FillCmd F = fills[f];
        const StrokeTot t = tot[s];
        const Place pl = place(st, k, q, off_a, off_b);
        DEdge *out = edges + st_fill[f].edge_base;
        const bool closed = st.kind == SK_CLOSED;
        const long long na = cnt_a[q], nb = cnt_b[q];
        for (long long i = 0; i < na; i++) {
            const long long pos = pl.pos_a + i;
            const double2 a = pa[pos];
            long long nx = pos + 1;
            double2 b;
            if (nx < pl.ra + pl.sa) b = pa[nx];
            else if (!closed && pl.sb > 0) b = pb[pl.rb];
            else b = pa[pl.ra];
            add_edge(F, out + (pos - t.a0), a.x, a.y, b.x, b.y, et, eb, el, er, any);
        }
        for (long long i = 0; i < nb; i++) {
            const long long pos = pl.end_b - nb + i;
            const double2 a = pb[pos];
            long long nx = pos + 1;
            double2 b;
            if (nx < pl.rb + pl.sb) b = pb[nx];
            else if (!closed) b = pa[pl.ra];
            else b = pb[pl.rb];
            add_edge(F, out + (t.na + pos - t.b0), a.x, a.y, b.x, b.y, et, eb, el, er, any);
        }
    }
    merge_extents(st_fill, f, any, et, eb, el, er);
}

// Host-built polygons: each warp takes 32 consecutive points; lane k
// finds its contour among the (at most 32) contours the chunk touches.
__global__ void kp_edges(PolyRun run, const FillCmd *__restrict__ fills, FillState *__restrict__ st_fill,
                         DEdge *__restrict__ edges) {
    const unsigned all = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const long long n_pts = run.n_points;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long base = ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < n_pts;
         base += warps * 32) {
        // the contour holding `base`: the last one starting at or before it
        int32_t c0 = 0;
        if (lane == 0) {
            int32_t lo = 0, hi = run.n_contours - 1;
            while (lo < hi) {
                const int32_t mid = (lo + hi + 1) >> 1;
                if (run.start[mid] <= base) lo = mid;
                else hi = mid - 1;
            }
            c0 = lo;
        }
        c0 = __shfl_sync(all, c0, 0);
        const int32_t ck = c0 + lane;
        const long long end_k = ck < run.n_contours ? run.start[ck] + run.n[ck] : 0x7FFFFFFFFFFFFFFFll;
        const long long pt = base + lane;
        int32_t my = c0;
#pragma unroll 8
        for (int k = 0; k < 32; k++) my += __shfl_sync(all, end_k, k) <= pt ? 1 : 0;
        int32_t f = -1;
        double et = 0, eb = 0, el = 0, er = 0;
        bool any = false;
        if (pt < n_pts) {
            const long long s0 = run.start[my];
            const int32_t n = run.n[my];
            f = run.fill[my];
            const long long nx = pt + 1 == s0 + n ? s0 : pt + 1;
            const double2 a = run.pts[pt], b = run.pts[nx];
            add_edge(fills[f], edges + st_fill[f].edge_base + run.edge_off[my] + (pt - s0), a.x, a.y, b.x, b.y, et, eb,
                     el, er, any);
        }
        merge_extents(st_fill, f, any, et, eb, el, er);
    }
}

inline unsigned blocks_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// carves aligned sub-buffers out of one allocation
struct Carve {
    size_t off = 0;
    template <class T>
    size_t take(long long count) {
        const size_t at = off;
        off = (off + sizeof(T) * (size_t)count + 255) & ~(size_t)255;
        return at;
    }
};

}  // namespace

int poly_emit(Ctx &c, const PolyRun &run, const FillCmd *d_fills, FillState *d_st, DEdge *d_edges) {
    if (run.n_points == 0 || run.n_contours == 0) return Z2D_OK;
    constexpr int T = 128;
    const unsigned blocks = (unsigned)std::min<long long>(blocks_for((run.n_points + 31) / 32, T / 32),
                                                          (long long)c.sm_count * 32);
    cudaEvent_t ts = c.timer_begin(c.t_stroke);
    kp_edges<<<blocks, T, 0, c.stream>>>(run, d_fills, d_st, d_edges);
    c.timer_end(c.t_stroke, ts);
    c.launches += 1;
    return Z2D_OK;
}

const long long *stroke_totals_dev(const StrokeRun &run) {
    return reinterpret_cast<const State *>(run.state)->totals;
}

int stroke_count(Ctx &c, StrokeRun &run, int32_t *d_status) {
    if (run.n_strokes == 0) return Z2D_OK;
    static thread_local State st;  // device pointers of this thread's current run
    st = State{};
    run.state = &st;
    constexpr int T = 128;
    // ---- buffers known before counting
    Carve ca;
    const size_t o_cnt = ca.take<long long>(run.n_local + 1), o_off = ca.take<long long>(run.n_local + 1);
    const size_t o_lsub = ca.take<int32_t>(run.n_local + 1), o_pen = ca.take<PenVertex>(run.n_pen + 1);
    const size_t o_sub = ca.take<SubState>(run.n_subs + 1), o_tot = ca.take<StrokeTot>(run.n_strokes + 1);
    const size_t o_edges = ca.take<int32_t>(run.n_strokes + 1), o_totals = ca.take<long long>(2);
    if (c.stroke_a.ensure(ca.off)) return Z2D_ERR_OUT_OF_MEMORY;
    uint8_t *A = c.stroke_a.as<uint8_t>();
    st.raw_cnt = reinterpret_cast<long long *>(A + o_cnt);
    st.raw_off = reinterpret_cast<long long *>(A + o_off);
    int32_t *local_sub = reinterpret_cast<int32_t *>(A + o_lsub);
    st.pen = reinterpret_cast<PenVertex *>(A + o_pen);
    st.sub = reinterpret_cast<SubState *>(A + o_sub);
    st.tot = reinterpret_cast<StrokeTot *>(A + o_tot);
    run.stroke_edges = reinterpret_cast<int32_t *>(A + o_edges);
    st.totals = reinterpret_cast<long long *>(A + o_totals);

    cudaEvent_t ts = c.timer_begin(c.t_stroke);
    ks_pen<<<blocks_for(run.n_strokes, T), T, 0, c.stream>>>(run.strokes, run.n_strokes, run.trig, st.pen);
    ks_local_sub<<<blocks_for(run.n_subs, T), T, 0, c.stream>>>(run.subs, run.n_subs, local_sub);
    ks_raw_count<<<blocks_for(run.n_local + 1, T), T, 0, c.stream>>>(run.nodes, run.subs, local_sub, run.strokes,
                                                                      run.n_local, st.raw_cnt, d_status);
    size_t tmp = 0;
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, st.raw_cnt, st.raw_off, run.n_local + 1, c.stream));
    if (c.scan_tmp.ensure(tmp + 16)) return Z2D_ERR_OUT_OF_MEMORY;
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(c.scan_tmp.ptr, tmp, st.raw_cnt, st.raw_off, run.n_local + 1, c.stream));
    c.launches += 4;
    long long *rb = nullptr;
    if (c.readback.ensure(64)) return Z2D_ERR_OUT_OF_MEMORY;
    rb = c.readback.as<long long>();
    Z2D_CUDA(cudaMemcpyAsync(rb, st.raw_off + run.n_local, sizeof(long long), cudaMemcpyDeviceToHost, c.stream));
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    const long long R = rb[0];
    if (R < 0 || R >= 0x7FFFFFFFll) {
        set_error("batch too large: more than 2^31 stroke points");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    run.raw = R;
    // ---- buffers sized by the point count
    Carve cb;
    const size_t o_rpt = cb.take<double2>(R + 1), o_rsub = cb.take<int32_t>(R + 1), o_rmode = cb.take<uint8_t>(R + 1);
    const size_t o_keep = cb.take<int32_t>(R + 1), o_kept = cb.take<int32_t>(R + 1);
    const size_t o_qpt = cb.take<double2>(R + 1), o_qsub = cb.take<int32_t>(R + 1), o_qmode = cb.take<uint8_t>(R + 1);
    const size_t o_ca = cb.take<long long>(R + 1), o_cb = cb.take<long long>(R + 1);
    const size_t o_oa = cb.take<long long>(R + 1), o_ob = cb.take<long long>(R + 1);
    if (c.stroke_b.ensure(cb.off)) return Z2D_ERR_OUT_OF_MEMORY;
    uint8_t *B = c.stroke_b.as<uint8_t>();
    st.raw_pt = reinterpret_cast<double2 *>(B + o_rpt);
    st.raw_sub = reinterpret_cast<int32_t *>(B + o_rsub);
    st.raw_mode = B + o_rmode;
    st.keep = reinterpret_cast<int32_t *>(B + o_keep);
    st.kept_off = reinterpret_cast<int32_t *>(B + o_kept);
    st.q_pt = reinterpret_cast<double2 *>(B + o_qpt);
    st.q_sub = reinterpret_cast<int32_t *>(B + o_qsub);
    st.q_mode = B + o_qmode;
    st.cnt_a = reinterpret_cast<long long *>(B + o_ca);
    st.cnt_b = reinterpret_cast<long long *>(B + o_cb);
    st.off_a = reinterpret_cast<long long *>(B + o_oa);
    st.off_b = reinterpret_cast<long long *>(B + o_ob);

    ks_raw_emit<<<blocks_for(run.n_local + 1, T), T, 0, c.stream>>>(run.nodes, run.subs, local_sub, run.strokes,
                                                                     run.n_local, st.raw_off, R, st.raw_pt, st.raw_sub,
                                                                     st.raw_mode, st.keep);
    size_t t1 = 0, t2 = 0;
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t1, st.keep, st.kept_off, R + 1, c.stream));
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t2, st.cnt_a, st.off_a, R + 1, c.stream));
    if (c.scan_tmp.ensure(std::max(t1, t2) + 16)) return Z2D_ERR_OUT_OF_MEMORY;
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(c.scan_tmp.ptr, t1, st.keep, st.kept_off, R + 1, c.stream));
    ks_compact<<<blocks_for(R, T), T, 0, c.stream>>>(st.raw_pt, st.raw_sub, st.raw_mode, st.keep, st.kept_off, R,
                                                      st.q_pt, st.q_sub, st.q_mode);
    ks_sub_setup<<<blocks_for(run.n_subs, T), T, 0, c.stream>>>(run.subs, run.n_subs, run.strokes, st.raw_off,
                                                                 st.kept_off, st.q_pt, st.sub);
    ks_elem_count<<<blocks_for(R + 1, T), T, 0, c.stream>>>(run.subs, run.strokes, st.pen, st.sub, st.q_pt, st.q_sub,
                                                             st.q_mode, st.kept_off, R, st.cnt_a, st.cnt_b);
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(c.scan_tmp.ptr, t2, st.cnt_a, st.off_a, R + 1, c.stream));
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(c.scan_tmp.ptr, t2, st.cnt_b, st.off_b, R + 1, c.stream));
    ks_stroke_tot<<<blocks_for(std::max(run.n_strokes, 1), T), T, 0, c.stream>>>(
        run.strokes, run.n_strokes, st.sub, st.off_a, st.off_b, R, st.tot, run.stroke_edges, st.totals);
    c.timer_end(c.t_stroke, ts);
    c.launches += 9;
    return Z2D_OK;
}

int stroke_emit(Ctx &c, StrokeRun &run, const FillCmd *d_fills, FillState *d_st, DEdge *d_edges) {
    if (run.n_strokes == 0) return Z2D_OK;
    State &st = *reinterpret_cast<State *>(run.state);
    if (run.n_a < 0 || run.n_b < 0 || run.n_a + run.n_b > 0x7FFFFFFFll) {
        set_error("batch too large: more than 2^31 stroke polygon points");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    Carve cc;
    const size_t o_pa = cc.take<double2>(run.n_a + 1), o_pb = cc.take<double2>(run.n_b + 1);
    if (c.stroke_c.ensure(cc.off)) return Z2D_ERR_OUT_OF_MEMORY;
    st.pa = reinterpret_cast<double2 *>(c.stroke_c.as<uint8_t>() + o_pa);
    st.pb = reinterpret_cast<double2 *>(c.stroke_c.as<uint8_t>() + o_pb);
    constexpr int T = 128;
    const long long R = run.raw;
    cudaEvent_t ts = c.timer_begin(c.t_stroke);
    ks_elem_emit<<<blocks_for(R, T), T, 0, c.stream>>>(run.subs, run.strokes, st.pen, st.sub, st.q_pt, st.q_sub,
                                                        st.q_mode, st.kept_off, R, st.off_a, st.off_b, st.pa, st.pb);
    ks_edges<<<blocks_for(R, T), T, 0, c.stream>>>(run.subs, run.strokes, st.sub, st.q_sub, st.kept_off, R, st.cnt_a,
                                                    st.cnt_b, st.off_a, st.off_b, st.tot, st.pa, st.pb, d_fills, d_st,
                                                    d_edges);
    c.timer_end(c.t_stroke, ts);
    c.launches += 2;
    return Z2D_OK;
}

}  // namespace z2dg
