// fill.cuh -- device structures of the fill pipeline (fill.cu).
#pragma once
#include <stdint.h>

#include "z2d_internal.h"

namespace z2dg {

constexpr int kSplineStack = 48;  // subdivision depth bound (coordinates are bounded)
constexpr int32_t kSplineMaxSplits = 1 << 22;  // subdivisions per curve before giving up
constexpr int kTileRows = 4;      // pixel rows per band / tile
constexpr int kTileCols = 256;    // pixels per tile row
constexpr int kRasterThreads = 32 * kTileRows;  // one warp per tile row
constexpr int32_t kMaxBandEdges = 32000;  // edges of one fill in one band (16-bit winding counters)

// One fill command, prepared on the host.
struct FillCmd {
    int32_t node_off, n_nodes;
    int32_t aa;         // Z2D_AA_NONE, Z2D_AA_MULTISAMPLE_4X or Z2D_AA_SUPERSAMPLE_4X
    int32_t rule, op;
    int32_t precision;  // after the float upgrade of multisample.zig:36 / direct.zig:25
    int32_t pattern_kind;
    int32_t reduces;    // pixel pattern whose operator reduces to the source (shared.zig:111-117)
    int32_t fast_kind;  // FAST_* specialisation the rasteriser may use
    int32_t job;        // index of the surface (job) the fill draws on
    int32_t stroke;     // device-stroked command whose polygon this fill draws, or -1
    int32_t poly;       // host-built polygon this fill draws, or -1
    double tol;         // max(tolerance, 0.001) (painter.zig:103)
    double scale;       // 4 for multisample / supersample, 1 for none (painter.zig:93-97)
    double edge_scale;  // multiplier of node coordinates in Polygon.addEdge: scale, or 1 for
                        // stroke contours whose points are already scaled
    DevSrc src;         // the pattern as a compositor source
    Px px_paint;        // pattern pixel converted to the surface format (paintStride)
    I16 px_rgba;        // RGBA.fromPixel lanes of the pattern pixel (compositeStride)
};

// Per-node results of the flatten passes.
struct NodeInfo {
    double sx, sy;  // start point (the buffer's last point before the node)
    double ex, ey;  // close_path: the subpath's first point
    int32_t n_emit; // edges emitted (one per lineTo the reference issues)
    int32_t n_added;
    int32_t edge_off;
    int32_t chords; // curve whose edges are its subdivision leaves' chords (see k_node_emit_w)
    int32_t pool;   // first of its leaves' points in the curve pool, or -1 (see k_curve_count_w)
    int32_t _pad;
};

// Polygon.Edge plus its rounded active range: the edge is active on sample
// row y exactly when rt <= y < rb (top < y+0.5 <= bottom, Polygon.zig:284-285).
// fxs/fxi/ftp are x_start/x_inc/top rounded to f32 for crossing_f32; the
// first 16 bytes load as one vector.
struct DEdge {
    float fxs, fxi, ftp;
    int32_t dir;  // -1 down, +1 up, 0 horizontal (dropped)
    int32_t rt, rb;
    double x_start, x_inc, top;
};

static_assert(sizeof(DEdge) == 48, "DEdge layout: 16-byte f32 block, ranges, f64 fields");

// The crossing of an edge with sample row sr is
//   X = round(x_start + x_inc * ((sr + 0.5) - top))      (Polygon.zig:272-276)
// in f64, rounded half away from zero.  crossing_f32 evaluates the same
// expression in f32 from the f32-rounded inputs (s = sr + 0.5, exact) and
// bounds its distance from the f64 value.  With u = 2^-24 and every f32
// operation correctly rounded, to first order
//   |fv - v| <= u * (|fv| + |fxs| + |fp| + |fxi| * (|ftp| + 2|ft|))
// (input roundings of x_start, x_inc and top, then one rounding per
// operation); the f64 evaluation's own error is ~2^-29 of that.  The bound
// used is 1.25x the first-order one.  When fv is farther than the bound
// from the nearest half-integer, the f64 value lies on the same side of it
// and rounds to the same integer; otherwise the caller evaluates in f64.
// Returns false when the f32 result does not decide X.
Z2D_HD bool crossing_f32(float fxs, float fxi, float ftp, float s, int32_t &X) {
    const float ft = s - ftp;
    const float fp = fxi * ft;
    const float fv = fxs + fp;
    const float bound =
        (fabsf(fv) + fabsf(fxs) + fabsf(fp) + fabsf(fxi) * (fabsf(ftp) + 2.0f * fabsf(ft))) * 7.450580596923828e-8f;
    const float fl = floorf(fv);
    const float h = fl + 0.5f;
    if (!(fabsf(fv - h) > bound) || !(fabsf(fv) < 4194304.0f)) return false;  // NaN/inf fail here too
    X = (int32_t)fl + (fv > h ? 1 : 0);
    return true;
}

enum : int32_t {
    FAST_NONE = 0,
    FAST_PIXEL_SRC_OVER = 1,  // pixel pattern, integer precision, src_over
};

enum : int32_t {
    FILL_OPEN_CHAIN = 1,  // an open 2-point subpath: rows may be unbalanced
    FILL_EXACT = 2,       // rasterised by k_exact
    FILL_SS_ZERO = 4,     // supersample mask too small to downsample: all zero
};

struct FillState {
    int32_t edge_base, n_edges, flags, has_edges;
    unsigned long long ext[4];  // top(min), bottom(max), left(min), right(max) as ordered keys
    int32_t active;             // inBox passed
    int32_t start_y, end_y;     // draw rows [start_y, end_y] (supersample: the composite region)
    int32_t start_x, end_x;     // draw columns [start_x, end_x)
    int32_t band0, band1;       // bands the fill touches
    int32_t fb_base;            // first (fill, band) slot
    int32_t mask_w, mask_x0;
    long long mask_base;        // exact-path action mask offset (bytes)
    int32_t cull_x0, cull_x1;   // columns a tile must overlap to be affected
};

// What k_raster reads of a fill on its common path, in two 16-byte loads
// (written by k_fill_setup from the FillCmd and FillState).
struct RasterFill {
    int32_t start_x, end_x, start_y, end_y;  // FillState's draw box
    uint32_t meta;  // RF_* fields below
    uint32_t px;    // pattern pixel's RGBA lanes (FillCmd.px_rgba), one byte each: r | g << 8 | b << 16 | a << 24
    int32_t _pad[2];
};
static_assert(sizeof(RasterFill) == 32, "RasterFill: two 16-byte loads");
enum : uint32_t {
    RF_OP_MASK = 0x1F,        // operator
    RF_AA_SHIFT = 5,          // anti-aliasing mode, 2 bits
    RF_EVEN_ODD = 1u << 7,    // fill rule
    RF_FAST_SHIFT = 8,        // FillCmd.fast_kind, 2 bits
    RF_EXACT = 1u << 10,      // FILL_EXACT
    RF_SS_ZERO = 1u << 11,    // FILL_SS_ZERO
    RF_BOUNDED = 1u << 12,    // the operator is bounded
};

// counters (int32 slots; the mask byte count is a 64-bit pair)
enum : int32_t {
    CNT_EDGES = 0,
    CNT_FILL_BANDS = 1,
    CNT_MASK_LO = 2,  // + CNT_MASK_HI = 3
    CNT_EXACT = 4,
    CNT_STATUS = 5,
    CNT_CURVES = 6,       // curves queued by k_node_count_w
    CNT_CURVES_EMIT = 7,  // curves queued by k_node_emit_w
    CNT_POOL = 8,         // points asked of the curve pool (64-bit pair, + 9)
    CNT_QUEUE = 10,       // k_raster's work-queue counter (64-bit pair, + 11)
    CNT_COUNT = 12
};

// action-mask byte of the exact path: bit 7 = clear first, bits 0-4 = coverage
constexpr uint8_t kMaskClear = 0x80;

// One surface of a batch with the contiguous range of its fills.  The host
// sets sfc and fill0/fill1; k_fill_setup widens the touched band and tile
// column ranges; the host then lays out global bands, tiles and band-list
// storage job after job.
struct DevJob {
    DevSurface sfc;
    int32_t fill0, fill1;      // fills [fill0, fill1), in call order
    int32_t band_lo, band_hi;  // 4-row bands touched (band_hi < band_lo: none)
    int32_t tcol_lo, tcol_hi;  // 256-pixel tile columns touched
    int32_t gband_base;        // first global band of the job
    int32_t tile_base;         // first CTA of the job in k_raster's grid
    long long list_base;       // first band-list entry (one slot per fill and band)
};

// Runs ordered lists of fills on device surfaces (one list per job; jobs are
// independent).  `fills` hold the prepared commands grouped by job (node
// offsets into `nodes`, host memory; the fills' node ranges are disjoint);
// grad_of_fill[i] >= 0 names the gradient of fill i in `grads`.
// Nodes that no fill owns are skipped; device-stroked
// commands (`strokes`, fills with stroke >= 0) read their nodes from the
// same array; fills with poly >= 0 draw a host-built polygon of `strokes`.
// A call with few short fills, on one surface or many, in a single upload
// and a single launch: the host flattens the paths (fill_plotter.plot,
// Spline.decompose, Polygon.addEdge), sets the fills up (inBox,
// multisample.run's draw box), bins their edges and lays out the band
// lists; the rasteriser draws the tiles.  Sets `done` = false without
// touching the device when the call is not one it takes (another
// anti-aliasing mode, strokes, an open two-point chain, more nodes, edges or
// bands than its limits, a packed surface, a gradient with a stop table),
// and the caller runs the full pipeline.
int run_small_jobs(Ctx &c, std::vector<DevJob> &jobs, const z2d_node *nodes, const std::vector<FillCmd> &fills,
                   const std::vector<DevGradient> &grads, const std::vector<int32_t> &grad_of_fill, bool &done);

struct StrokeSet;
int run_jobs(Ctx &c, std::vector<DevJob> &jobs, const z2d_node *nodes, int32_t n_nodes, std::vector<FillCmd> &fills,
             const std::vector<DevGradient> &grads,
             const std::vector<int32_t> &grad_of_fill, const StrokeSet *strokes = nullptr);

}  // namespace z2dg
