// stroke_gpu.cuh -- painter.stroke's polygon built on the device.
//
// A stroke command keeps its path nodes on the device; the stroker expands
// them into the stroke polygon's edges in parallel (stroke_gpu.cu):
//   1. per node: the points stroke_plotter.Plotter receives (lineTo points,
//      curve subdivisions of Spline.zig), with their join mode
//   2. consecutive duplicates dropped (the degenerate-node check of
//      stroke_plotter.zig:110-112)
//   3. per kept point ("element"): its join (stroke_plotter.zig:405-545),
//      cap (Face.cap) or dot, counted, then emitted into the positions the
//      outer and inner contours of Polygon give them
//   4. per contour point: the edge to the next point (Polygon.addEdge)
// The host validates the options and the node sequence, splits each path
// into subpaths and computes the pen's cos/sin tables (the only
// transcendental functions of the tessellation).
#pragma once
#include <stdint.h>

#include <vector>

#include "fill.cuh"
#include "stroke.h"

namespace z2dg {

// One device-stroked command: stroke_plotter.PlotterOptions after
// painter.stroke's adjustments, the fill that draws the polygon, its
// subpaths and its pen.
struct StrokeDev {
    int32_t fill;          // index of the FillCmd drawing the polygon
    int32_t sub0, n_sub;   // subpaths [sub0, sub0 + n_sub)
    int32_t join, cap;
    int32_t pen_n;         // pen vertices (Pen.init)
    int32_t pen_tab;       // first (cos, sin) pair of the pen in the trig table
    int32_t pen_off;       // first vertex of the pen in the device pen array
    double thickness, miter_limit, tolerance, scale;
    double ctm[6];         // ax, by, cx, dy, tx, ty
};

// A subpath: a move_to followed by line_to / curve_to nodes.
struct SubpathDev {
    int32_t node0, n_nodes;  // nodes [node0, node0 + n_nodes) of the device node array
    int32_t local0;          // index of node0 in the concatenation of all subpaths' nodes
    int32_t stroke;
    int32_t closed;          // ended by close_path (else by move_to or the end of the path)
    int32_t _pad;
};

// What the host hands over: device-stroked commands with their subpaths and
// the pens' tables, and polygons built on the host (dashed strokes), each
// drawn by the fill whose `poly` names it.
struct StrokeSet {
    std::vector<StrokeDev> strokes;
    std::vector<SubpathDev> subs;
    std::vector<double> trig;  // (cos t, sin t) pairs
    int64_t n_local = 0;       // sum of the subpaths' node counts
    int64_t n_pen = 0;         // sum of the strokes' pen vertices
    std::vector<const stroke::Polygon *> polys;
    bool empty() const { return strokes.empty() && polys.empty(); }
};

// The contours of the host-built polygons on the device (structure of
// arrays over all contours, in order): contour k is points
// [start[k], start[k] + n[k]) of the point array, drawn by fill[k], its
// first edge at edge_off[k] within that fill's edges.
struct PolyRun {
    const double2 *pts = nullptr;
    const long long *start = nullptr;
    const int32_t *n = nullptr, *fill = nullptr, *edge_off = nullptr;
    int32_t n_contours = 0;
    long long n_points = 0;
};
// Writes the edges of every host-built polygon's contours (each point to
// the next, the last to the first) and merges the fills' extents.
int poly_emit(Ctx &c, const PolyRun &run, const FillCmd *d_fills, FillState *d_st, DEdge *d_edges);

// Hairline strokes (hairline.cu): per command its polylines (host-built by
// stroke::polyline), the FillCmd that carries its pattern, operator,
// precision and surface (job), and whether it draws without anti-aliasing.
struct HairSet {
    std::vector<const stroke::Polygon *> lines;
    std::vector<int32_t> fill;
    std::vector<int32_t> aa_none;
};
// Draws the hairlines in command order on the jobs' device surfaces
// (hairline.zig: Bresenham or Xiaolin Wu segments, single-pixel
// composites applied in path order).
int run_hairlines(Ctx &c, const std::vector<DevJob> &jobs, std::vector<FillCmd> &fills,
                  const std::vector<DevGradient> &grads, const std::vector<int32_t> &grad_of_fill, const HairSet &hs);

// Device side of a StrokeSet during one run_jobs call.
struct StrokeRun {
    const z2d_node *nodes = nullptr;
    const StrokeDev *strokes = nullptr;
    const SubpathDev *subs = nullptr;
    const double *trig = nullptr;
    int32_t n_strokes = 0, n_subs = 0;
    int64_t n_local = 0, n_pen = 0;
    int32_t *stroke_edges = nullptr;  // per stroke: edges of its polygon (read by k_fill_scan)
    long long raw = 0;                // points before deduplication
    long long n_a = 0, n_b = 0;       // outer / inner contour points of all strokes
    void *state = nullptr;            // internal device pointers (stroke_gpu.cu)
};

// Phase 1, before the fills' edge counts: counts every stroke polygon's
// edges into run.stroke_edges.  Reads back one count (synchronises).
int stroke_count(Ctx &c, StrokeRun &run, int32_t *d_status);
// The device address of the contour totals that the caller reads back with
// the edge count (two int64: outer and inner points).
const long long *stroke_totals_dev(const StrokeRun &run);
// Phase 2, after the edges are allocated: writes every stroke polygon's
// edges at its fill's edge_base and merges the fills' extents.
int stroke_emit(Ctx &c, StrokeRun &run, const FillCmd *d_fills, FillState *d_st, DEdge *d_edges);

}  // namespace z2dg
