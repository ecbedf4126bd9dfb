// stroke.h -- painter.stroke's polygon builder (stroke.cpp).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "../../include/z2dgpu.h"

namespace z2dg {
namespace stroke {

enum { kJoinMiter = Z2D_JOIN_MITER, kJoinRound = Z2D_JOIN_ROUND, kJoinBevel = Z2D_JOIN_BEVEL };
enum { kCapButt = Z2D_CAP_BUTT, kCapRound = Z2D_CAP_ROUND, kCapSquare = Z2D_CAP_SQUARE };
enum { kErrInvalidState = Z2D_ERR_INVALID_STATE };

// stroke_plotter.PlotterOptions (stroke_plotter.zig:28-38), after
// painter.stroke's adjustments (painter.zig:286-304).
struct Options {
    int cap, join;
    double ctm[6];  // ax, by, cx, dy, tx, ty
    double miter_limit;
    double scale;
    double thickness;
    double tolerance;
    const double *dashes;  // Dasher input (used when Dasher.validate accepts it)
    size_t n_dashes;
    double dash_offset;
};

// Dasher.validate: the dash array draws dashes (stroke_plotter.zig:40-44).
bool dashed(const Options &opts);

// Pen.init's vertex count for a pen of width `thickness` through the CTM m
// (ax, by, cx, dy, tx, ty) at `tolerance` (Pen.zig:25-60).
int32_t pen_vertex_count(double thickness, double tolerance, const double m[6]);
// The n (cos t, sin t) pairs of the pen's vertex angles t = 2 pi i / n,
// negated when the CTM reflects (Pen.zig:62-75).
void pen_trig(int32_t n, bool reflect, double *out);

// Transformation.inverse succeeds (painter.zig:231).
bool transformation_invertible(const double m[6]);

// A polygon as closed contours: contour k is points [ends[k-1], ends[k])
// of xy (x, y pairs), each point joined to the next and the last to the
// first.
struct Polygon {
    std::vector<double> xy;
    std::vector<uint64_t> ends;
    size_t points() const { return xy.size() / 2; }
    void clear() {
        xy.clear();
        ends.clear();
    }
};

// stroke_plotter.plot: the closed contours (points already multiplied by
// opts.scale) whose edges form the stroke polygon, in the order z2d adds
// them; empty contours are left out.  Returns Z2D_OK or an error code.
int plot(const z2d_node *nodes, size_t n_nodes, const Options &opts, Polygon &out);

// polyline_plotter.plot (polyline_plotter.zig:27-141), for hairline
// strokes: the path as open polylines (contours whose last point is not
// joined to the first), untransformed and unscaled, dashed when
// opts.dashes validates; opts.tolerance is used as given.
int polyline(const z2d_node *nodes, size_t n_nodes, const Options &opts, Polygon &out);

}  // namespace stroke
}  // namespace z2dg
