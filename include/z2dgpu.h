/*
 * z2dgpu.h -- C ABI of the GB300-native fill-and-composite path.
 *
 * This is the drop-in boundary for z2d's painter.fill / SurfaceCompositor.run
 * hot path.  Every entry point is plain C: pointers, sizes and small POD
 * structs, no C++ or torch types.  Status codes mirror z2d's error sets.
 *
 * Reference interfaces replaced (paths are inside the z2d project):
 *   z2dgpu_fill        <- painter.fill                  src/painter.zig:66-72
 *   z2dgpu_fill_batch  <- N x painter.fill, same surface src/painter.zig:66-143
 *                         (Context.fill loop, src/Context.zig:592-607)
 *   z2dgpu_fill_jobs   <- the same over many surfaces
 *   z2dgpu_stroke      <- painter.stroke                src/painter.zig:214-344
 *   z2dgpu_composite   <- compositor.SurfaceCompositor.run
 *                                                       src/compositor.zig:302-309
 *                         (and Surface.composite,       src/surface.zig:225-241)
 *   z2d_surface        <- surface.Surface               src/surface.zig:74-83
 *   z2d_node           <- PathNode                      src/internal/path_nodes.zig:16-41
 *   z2d_pattern        <- pattern.Pattern               src/pattern.zig:32-36
 *   z2d_gradient       <- gradient.Gradient             src/gradient.zig:42-95
 *   z2d_fill_opts      <- painter.FillOptions           src/painter.zig:28-48
 *   z2d_operation      <- SurfaceCompositor.Operation   src/compositor.zig:223-284
 *
 * Memory layout of surface data (identical to z2d's in-memory layout):
 *   ARGB  4 B/px, bytes B,G,R,A        RGBA 4 B/px, bytes R,G,B,A
 *   XRGB  4 B/px, bytes B,G,R,pad      RGB  4 B/px, bytes R,G,B,pad
 *   ALPHA8 1 B/px
 *   ALPHA4/2/1 packed: pixel i (flat index w*y+x) occupies bits
 *     [i*bits, i*bits+bits) little-endian (LSB first); rows are NOT byte
 *     aligned.  Buffer length ceil(w*h*bits/8), host or device.  (Pixels
 *     are updated with 32-bit word atomics; a device buffer whose length is
 *     not a multiple of 4 bytes is drawn on a padded copy and copied back,
 *     so nothing past its length is touched.)
 *
 * Threading: a context owns one CUDA stream and device scratch; calls on one
 * context must not overlap.  Use one context per host thread.
 */
#ifndef Z2DGPU_H
#define Z2DGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define Z2D_EXTERN extern "C"
#else
#define Z2D_EXTERN extern
#endif
#define Z2D_API Z2D_EXTERN __attribute__((visibility("default")))

/* ---- status codes (src/painter.zig:54-63, src/surface.zig:85-91) ---- */
enum {
    Z2D_OK = 0,
    Z2D_ERR_PATH_NOT_CLOSED = 1,          /* FillError.PathNotClosed */
    Z2D_ERR_PIXEL_NOT_PREMULTIPLIED = 2,  /* FillError.PixelSourceNotPreMultiplied */
    Z2D_ERR_INVALID_DIMENSIONS = 3,       /* Surface.Error.InvalidWidth/InvalidHeight */
    Z2D_ERR_INVALID_STATE = 4,            /* InternalError.InvalidState */
    Z2D_ERR_OUT_OF_MEMORY = 5,            /* Allocator.Error.OutOfMemory */
    Z2D_ERR_CUDA = 6,                     /* CUDA runtime failure (see z2dgpu_last_error) */
    Z2D_ERR_TIMEOUT = 7,                  /* a bounded device wait gave up */
    Z2D_ERR_INVALID_ARGUMENT = 8          /* malformed descriptor */
};

/* ---- pixel formats (src/pixel.zig:47-56) ---- */
enum {
    Z2D_FORMAT_ARGB = 0,
    Z2D_FORMAT_XRGB = 1,
    Z2D_FORMAT_RGB = 2,
    Z2D_FORMAT_RGBA = 3,
    Z2D_FORMAT_ALPHA8 = 4,
    Z2D_FORMAT_ALPHA4 = 5,
    Z2D_FORMAT_ALPHA2 = 6,
    Z2D_FORMAT_ALPHA1 = 7
};

/* where z2d_surface.data lives */
enum { Z2D_MEM_HOST = 0, Z2D_MEM_DEVICE = 1 };

/* operators (src/compositor.zig:46-158), same order */
enum {
    Z2D_OP_CLEAR = 0, Z2D_OP_SRC, Z2D_OP_DST, Z2D_OP_SRC_OVER, Z2D_OP_DST_OVER,
    Z2D_OP_SRC_IN, Z2D_OP_DST_IN, Z2D_OP_SRC_OUT, Z2D_OP_DST_OUT, Z2D_OP_SRC_ATOP,
    Z2D_OP_DST_ATOP, Z2D_OP_XOR, Z2D_OP_PLUS, Z2D_OP_MULTIPLY, Z2D_OP_SCREEN,
    Z2D_OP_OVERLAY, Z2D_OP_DARKEN, Z2D_OP_LIGHTEN, Z2D_OP_COLOR_DODGE,
    Z2D_OP_COLOR_BURN, Z2D_OP_HARD_LIGHT, Z2D_OP_SOFT_LIGHT, Z2D_OP_DIFFERENCE,
    Z2D_OP_EXCLUSION, Z2D_OP_HUE, Z2D_OP_SATURATION, Z2D_OP_COLOR,
    Z2D_OP_LUMINOSITY,
    Z2D_OP_COUNT
};

enum { Z2D_PRECISION_INTEGER = 0, Z2D_PRECISION_FLOAT = 1 };  /* src/compositor.zig:214 */
enum { Z2D_FILL_NON_ZERO = 0, Z2D_FILL_EVEN_ODD = 1 };         /* src/options.zig:23-37 */
enum {                                                         /* src/options.zig:73-91 */
    Z2D_AA_NONE = 0, Z2D_AA_DEFAULT = 1, Z2D_AA_MULTISAMPLE_4X = 2, Z2D_AA_SUPERSAMPLE_4X = 3
};

/* A pixel value in its own format.  For ALPHA4/2/1 `a` holds the raw
 * 4/2/1-bit value.  For XRGB/RGB `a` is ignored. */
typedef struct z2d_pixel {
    int32_t format;
    uint8_t r, g, b, a;
} z2d_pixel;

typedef struct z2d_surface {
    int32_t format;
    int32_t width;
    int32_t height;
    int32_t location;   /* Z2D_MEM_HOST or Z2D_MEM_DEVICE */
    void *data;
} z2d_surface;

/* path nodes (src/internal/path_nodes.zig:9-14) */
enum { Z2D_MOVE_TO = 0, Z2D_LINE_TO = 1, Z2D_CURVE_TO = 2, Z2D_CLOSE_PATH = 3 };

/* options.JoinMode / options.CapMode (src/options.zig:40-70) */
enum { Z2D_JOIN_MITER = 0, Z2D_JOIN_ROUND = 1, Z2D_JOIN_BEVEL = 2 };
enum { Z2D_CAP_BUTT = 0, Z2D_CAP_ROUND = 1, Z2D_CAP_SQUARE = 2 };

/* move_to/line_to: point = (p[0], p[1]).  curve_to: p1 = (p[0], p[1]),
 * p2 = (p[2], p[3]), p3 = (p[4], p[5]).  Device-space coordinates, as held
 * by z2d's Path after transformation and clamping. 56 bytes. */
typedef struct z2d_node {
    int32_t tag;
    int32_t _pad;
    double p[6];
} z2d_node;

/* colors (src/color.zig:41-93); values are stored as after Color.init */
enum { Z2D_COLOR_LINEAR_RGB = 0, Z2D_COLOR_SRGB = 1, Z2D_COLOR_HSL = 2 };
typedef struct z2d_color {
    int32_t space;
    float c[4];         /* r,g,b,a or h,s,l,a */
} z2d_color;

/* gradient stop; offsets in insertion order, clamped to [0,1] and stably
 * sorted by the library exactly as Stop.List.addAssumeCapacity does
 * (src/gradient.zig:797-811). */
typedef struct z2d_stop {
    float offset;
    z2d_color color;
} z2d_stop;

enum { Z2D_GRADIENT_LINEAR = 0, Z2D_GRADIENT_RADIAL = 1, Z2D_GRADIENT_CONIC = 2 };
enum {  /* InterpolationMethod (src/color.zig:111-135) */
    Z2D_INTERP_LINEAR_RGB = 0, Z2D_INTERP_SRGB = 1,
    Z2D_INTERP_HSL_SHORTER = 2, Z2D_INTERP_HSL_LONGER = 3,
    Z2D_INTERP_HSL_INCREASING = 4, Z2D_INTERP_HSL_DECREASING = 5
};

typedef struct z2d_gradient {
    int32_t type;
    int32_t method;
    int32_t n_stops;
    int32_t _pad;
    /* linear: x0,y0,x1,y1; radial: inner_x,inner_y,inner_r,outer_x,outer_y,
     * outer_r; conic: x,y,angle (radians, un-normalised) */
    double geom[6];
    /* the device->pattern matrix as stored by setTransformation (already
     * inverted): ax, by, cx, dy, tx, ty.  Identity means "no transform". */
    double transform[6];
    const z2d_stop *stops;
} z2d_gradient;

/* pattern (src/pattern.zig:32) and dither (src/Dither.zig:28-70) */
enum { Z2D_PATTERN_PIXEL = 0, Z2D_PATTERN_GRADIENT = 1, Z2D_PATTERN_DITHER = 2 };
enum { Z2D_DITHER_NONE = 0, Z2D_DITHER_BAYER = 1, Z2D_DITHER_BLUE_NOISE = 2 };
enum { Z2D_DITHER_SRC_PIXEL = 0, Z2D_DITHER_SRC_COLOR = 1, Z2D_DITHER_SRC_GRADIENT = 2 };

typedef struct z2d_pattern {
    int32_t kind;              /* Z2D_PATTERN_* */
    z2d_pixel pixel;           /* PIXEL, or dither source pixel */
    const z2d_gradient *gradient; /* GRADIENT, or dither source gradient */
    int32_t dither_type;       /* DITHER: Z2D_DITHER_* */
    int32_t dither_source;     /* DITHER: Z2D_DITHER_SRC_* */
    int32_t dither_scale;      /* DITHER: bits per channel of the target (1..15) */
    int32_t _pad;
    z2d_color dither_color;    /* DITHER with COLOR source */
} z2d_pattern;

typedef struct z2d_fill_opts {
    int32_t anti_aliasing;     /* Z2D_AA_* (default: Z2D_AA_DEFAULT) */
    int32_t fill_rule;         /* Z2D_FILL_* (default: NON_ZERO) */
    int32_t op;                /* Z2D_OP_* (default: SRC_OVER) */
    int32_t precision;         /* Z2D_PRECISION_* (default: INTEGER) */
    double tolerance;          /* default 0.1 */
} z2d_fill_opts;

/* Compositor parameters (SurfaceCompositor.Operation.Param) */
enum {
    Z2D_PARAM_NONE = 0, Z2D_PARAM_PIXEL = 1, Z2D_PARAM_GRADIENT = 2,
    Z2D_PARAM_DITHER = 3, Z2D_PARAM_SURFACE = 4
};
typedef struct z2d_param {
    int32_t kind;              /* Z2D_PARAM_* */
    int32_t _pad;
    z2d_pattern pattern;       /* PIXEL / GRADIENT / DITHER use the matching fields */
    const z2d_surface *surface;/* SURFACE */
} z2d_param;

typedef struct z2d_operation {
    int32_t op;
    int32_t _pad;
    z2d_param dst;
    z2d_param src;
} z2d_operation;

/* one fill of a batch: nodes[node_offset, node_offset+n_nodes) of the batch
 * node array, drawn with `pattern` and `opts` */
typedef struct z2d_fill_cmd {
    const z2d_pattern *pattern;
    uint64_t node_offset;
    uint64_t n_nodes;
    z2d_fill_opts opts;
} z2d_fill_cmd;

/* painter.StrokeOptions (src/painter.zig:145-195).  Defaults: AA default,
 * miter join, butt cap, line width 2, miter limit 10, tolerance 0.1,
 * identity transformation, no dashes, no hairline, src_over, integer. */
typedef struct z2d_stroke_opts {
    int32_t anti_aliasing;     /* Z2D_AA_* */
    int32_t line_join;         /* Z2D_JOIN_* */
    int32_t line_cap;          /* Z2D_CAP_* */
    int32_t op;                /* Z2D_OP_* */
    int32_t precision;         /* Z2D_PRECISION_* */
    int32_t hairline;          /* nonzero: hairline mode (1-pixel Bresenham / Wu lines) */
    double line_width;
    double miter_limit;
    double tolerance;
    double dash_offset;
    double transformation[6];  /* ax, by, cx, dy, tx, ty (Transformation.zig) */
    const double *dashes;      /* dash array (Dasher.zig); ignored unless it has a positive entry and no negative one */
    uint64_t n_dashes;
} z2d_stroke_opts;

/* one drawing operation of a mixed batch: painter.fill (kind FILL, `fill`
 * options) or painter.stroke (kind STROKE, `stroke` options) of
 * nodes[node_offset, node_offset+n_nodes) with `pattern` */
enum { Z2D_DRAW_FILL = 0, Z2D_DRAW_STROKE = 1 };
typedef struct z2d_draw_cmd {
    int32_t kind;
    int32_t _pad;
    const z2d_pattern *pattern;
    uint64_t node_offset;
    uint64_t n_nodes;
    z2d_fill_opts fill;
    z2d_stroke_opts stroke;
} z2d_draw_cmd;

/* one surface of a multi-surface batch: cmds[cmd_offset, cmd_offset+n_cmds)
 * of the batch command array, drawn in order on `surface` */
typedef struct z2d_job {
    z2d_surface surface;
    uint64_t cmd_offset;
    uint64_t n_cmds;
} z2d_job;

typedef struct z2dgpu_ctx z2dgpu_ctx;

/* ---- library / context ---- */
Z2D_API const char *z2dgpu_version(void);
/* Message of the last failing call on this thread ("" if none). */
Z2D_API const char *z2dgpu_last_error(void);
/* Creates a context on `device`.  `stream` is a cudaStream_t to run on, or
 * NULL for a context-owned stream. */
Z2D_API int z2dgpu_ctx_create(z2dgpu_ctx **out, int device, void *stream);
Z2D_API int z2dgpu_ctx_destroy(z2dgpu_ctx *ctx);
/* Blocks until all work queued on the context's stream has finished. */
Z2D_API int z2dgpu_ctx_synchronize(z2dgpu_ctx *ctx);
/* Number of kernels this context has launched since creation. */
Z2D_API uint64_t z2dgpu_ctx_launch_count(const z2dgpu_ctx *ctx);

/* Kernel timing: when enabled, the context brackets its dominant kernels
 * (the fill rasteriser "raster" and the compositor "composite") with CUDA
 * events on its stream and accumulates their device time.  Reading a time
 * synchronizes the context.  No reference counterpart (instrumentation). */
Z2D_API int z2dgpu_ctx_set_timing(z2dgpu_ctx *ctx, int enable);
/* The rasteriser's schedule on this context (no counterpart in z2d).  By
 * default an autotuner picks it per kind of pass (one surface or many, its
 * number of tiles, the mean fills per band) by timing the candidates on the
 * first passes of each kind, and caches its choices in raster_tune.json
 * beside the library (Z2D_TUNE_FILE overrides the path; Z2D_TUNE=off keeps
 * the default schedule).  ctas_per_sm >= -1 forces a schedule: the grid
 * (-1 = one CTA per tile, not persistent; 0 = a persistent grid of as many
 * resident CTAs as fit; n = n per SM), the queue order (0 = tile order, 1 =
 * tiles of the bands with the most fills first) and the queue item (1 = a
 * whole 4-row tile per CTA, 0 = one tile row per warp); ctas_per_sm = -2
 * returns to the tuner.  Every schedule draws the same pixels. */
Z2D_API int z2dgpu_ctx_set_raster(z2dgpu_ctx *ctx, int32_t ctas_per_sm, int32_t order,
                                  int32_t tile_items);
/* The tuner's state for the kind of pass this context drew last: *decided =
 * 1 with its schedule, 0 while candidates are still being timed, -1 when
 * tuning is off. */
Z2D_API int z2dgpu_ctx_raster_tuning(z2dgpu_ctx *ctx, int32_t *decided, int32_t *ctas_per_sm,
                                     int32_t *order, int32_t *tile_items);
/* Accumulated milliseconds and launch count of a stage since timing was
 * enabled: "raster" (k_raster), "composite" (compositor kernels), "flatten"
 * (path flattening, stroking and fill setup, two intervals per fill call),
 * "stroke" (the stroke kernels, a share of "flatten"), "bins" (edge
 * binning, band lists and the exact path) or "export" (the PNG encoding
 * kernel).  Returns -1 for an unknown name. */
Z2D_API double z2dgpu_ctx_kernel_ms(z2dgpu_ctx *ctx, const char *kernel, uint64_t *launches);

/* Bytes of pixel storage for a surface (src/surface.zig:382-395, 621-635). */
Z2D_API size_t z2dgpu_surface_bytes(int32_t format, int32_t width, int32_t height);

/* painter.fill (src/painter.zig:66-143).  Synchronous for host surfaces;
 * for device surfaces the work is queued on the context stream and the call
 * returns after launch (validation errors are still reported). */
Z2D_API int z2dgpu_fill(z2dgpu_ctx *ctx, z2d_surface *surface,
                        const z2d_pattern *pattern, const z2d_node *nodes,
                        size_t n_nodes, const z2d_fill_opts *opts);

/* Equivalent to calling painter.fill for cmds[0..n_cmds) in order on one
 * surface; the fills are flattened, binned and composited in one device
 * pass that keeps per-pixel order.  `nodes` is the node array the commands
 * index into. */
Z2D_API int z2dgpu_fill_batch(z2dgpu_ctx *ctx, z2d_surface *surface,
                              const z2d_node *nodes, size_t n_nodes,
                              const z2d_fill_cmd *cmds, size_t n_cmds);

/* painter.stroke (src/painter.zig:214-344): the stroke polygon z2d's stroke
 * plotter builds (joins, caps, pens, dashes), filled with the non-zero rule
 * by the GPU rasterisers.  Solid strokes are tessellated on the device;
 * dashed ones on the host; hairlines are drawn by the hairline rasteriser
 * (hairline.zig).  A transformation that cannot be inverted returns
 * Z2D_ERR_INVALID_ARGUMENT (Transformation.Error.InvalidMatrix); a
 * line_to / curve_to without a current point or a non-finite coordinate
 * returns Z2D_ERR_INVALID_STATE. */
Z2D_API int z2dgpu_stroke(z2dgpu_ctx *ctx, z2d_surface *surface,
                          const z2d_pattern *pattern, const z2d_node *nodes,
                          size_t n_nodes, const z2d_stroke_opts *opts);

/* Host only (no device work): the polygon painter.stroke would rasterise
 * for a surface of `surface_format`, as closed contours of points already
 * multiplied by the rasteriser scale (written to *scale).  For hairline
 * strokes: the open polylines of polyline_plotter, scale 1.  points receives
 * x, y pairs, contour_ends[k] the index one past contour k's last point.
 * The counts are returned even when the capacities are too small. */
Z2D_API int z2dgpu_stroke_contours(const z2d_node *nodes, size_t n_nodes,
                                   const z2d_stroke_opts *opts, int32_t surface_format,
                                   double *points, size_t cap_points, uint64_t *n_points,
                                   uint64_t *contour_ends, size_t cap_contours,
                                   uint64_t *n_contours, double *scale);

/* ---- Path building on the device (src/Path.zig, src/internal/arc.zig,
 * src/internal/Glyph.zig) ----
 * A path program is the sequence of Path calls that builds one path, with
 * the Path's transformation and tolerance at its start.  The device runs
 * each program as z2d's Path would and writes the device-space nodes it
 * would hold: user points clamped to the i24 range and mapped by the
 * transformation, a move_to to the point of a trailing move_to dropped,
 * close as close_path plus a move_to back to the subpath's start, rel*
 * points relative to the current point mapped back through the inverse
 * transformation, arcs as arc.zig's cubic splines (Zig's f64 sin / cos /
 * tan), glyph outlines as Outline.init + appendToPath. */
enum {
    Z2D_PATH_MOVE_TO = 0,           /* v: x, y */
    Z2D_PATH_LINE_TO = 1,           /* v: x, y */
    Z2D_PATH_CURVE_TO = 2,          /* v: x1, y1, x2, y2, x3, y3 */
    Z2D_PATH_REL_MOVE_TO = 3,       /* v: dx, dy */
    Z2D_PATH_REL_LINE_TO = 4,       /* v: dx, dy */
    Z2D_PATH_REL_CURVE_TO = 5,      /* v: dx1, dy1, dx2, dy2, dx3, dy3 */
    Z2D_PATH_ARC = 6,               /* v: xc, yc, radius, angle1, angle2 (Path.arc) */
    Z2D_PATH_ARC_NEGATIVE = 7,      /* v: as ARC (Path.arcNegative) */
    Z2D_PATH_CLOSE = 8,
    Z2D_PATH_SET_TRANSFORMATION = 9,/* v: ax, by, cx, dy, tx, ty (Path.transformation = v) */
    Z2D_PATH_SET_TOLERANCE = 10,    /* v: tolerance (Path.tolerance) */
    Z2D_PATH_RESET = 11,            /* Path.reset: clears the nodes and the points */
    Z2D_PATH_GLYPH = 12             /* v: first point, points, first contour end, contours,
                                     *    units per em: a simple glyph's outline (Glyph.zig
                                     *    runOutline) appended with the current transformation */
};
typedef struct z2d_path_cmd {
    int32_t op;
    int32_t _pad;
    double v[6];
} z2d_path_cmd;
typedef struct z2d_path_program {
    uint64_t cmd_offset, n_cmds;  /* the program's commands in the command array */
    double transformation[6];     /* ax, by, cx, dy, tx, ty at the start */
    double tolerance;             /* Path.tolerance at the start (z2d's default: 0.1) */
} z2d_path_program;
/* A glyph outline point (TrueType simple glyph): font units; bit 0 of
 * flags = on-curve.  Contours are given by the index of their last point. */
typedef struct z2d_glyph_point {
    int16_t x, y;
    uint16_t flags;
    uint16_t _pad;
} z2d_glyph_point;
/* Runs every program and writes its nodes, program after program, to
 * `nodes` (host or device memory, cap_nodes entries): program p's nodes are
 * nodes[offsets[p] .. offsets[p+1]) (offsets has n_programs + 1 entries and
 * is filled even when the nodes do not fit, which returns
 * Z2D_ERR_OUT_OF_MEMORY).  status[p] (may be NULL) is 0 or the program's
 * first error, where it stopped: Z2D_ERR_INVALID_STATE for NoCurrentPoint
 * (curve_to / rel* without a current point), Z2D_ERR_INVALID_ARGUMENT for
 * InvalidMatrix (rel* or a glyph with a transformation that cannot be
 * inverted), a malformed glyph, an unknown command, an arc angle beyond
 * 2^20 * pi/2 or arc angles so far apart that whole turns no longer change
 * them (z2d would loop there).  Its nodes up to the error are kept. */
Z2D_API int z2dgpu_build_paths(z2dgpu_ctx *ctx, const z2d_path_program *programs, size_t n_programs,
                               const z2d_path_cmd *cmds, size_t n_cmds, const z2d_glyph_point *glyph_points,
                               size_t n_glyph_points, const uint16_t *glyph_ends, size_t n_glyph_ends,
                               z2d_node *nodes, size_t cap_nodes, uint64_t *offsets, int32_t *status);

/* Gradient.getOffset (gradient.zig:239-243) of the w x h pixels from
 * (x0, y0), row-major into the host array `offsets`, exactly as the fill
 * and compositor kernels evaluate them (-1 = no colour).  *n_f64, when not
 * NULL, receives how many of them the double-word evaluation left to the
 * f64 code.  A diagnostic for the offsets; w * h <= 2^28. */
Z2D_API int z2dgpu_gradient_offsets(z2dgpu_ctx *ctx, const z2d_gradient *gradient, int32_t x0, int32_t y0, int32_t w,
                                    int32_t h, float *offsets, int64_t *n_f64);

/* ---- PNG export (src/export_png.zig) ---- */
enum { Z2D_PROFILE_NONE = -1, Z2D_PROFILE_LINEAR = 0, Z2D_PROFILE_SRGB = 1 };
/* png_exporter.writeToPNGFile (export_png.zig:56-87) to memory: the PNG file
 * of a surface (host or device memory) with the exporter's encoding
 * (demultiplied RGBA/RGB, alpha as grayscale, packed alpha4/2/1), a gAMA
 * chunk and the sRGB gamma on the pixels when color_profile asks for them.
 * The bytes are allocated by the library: *out, *out_len; release them with
 * z2dgpu_free.  The IDAT stream is zlib's default compression where the
 * library was built with zlib, stored deflate blocks otherwise (the decoded
 * image is the same). */
Z2D_API int z2dgpu_png_encode(z2dgpu_ctx *ctx, const z2d_surface *surface, int32_t color_profile, uint8_t **out,
                              size_t *out_len);
/* The PNG's uncompressed image data: per row a filter byte (0) followed by
 * the row's encoded pixels (writePNGIDATStream, export_png.zig:153-311).
 * Allocated like z2dgpu_png_encode's output. */
Z2D_API int z2dgpu_png_scanlines(z2dgpu_ctx *ctx, const z2d_surface *surface, int32_t color_profile, uint8_t **out,
                                 size_t *out_len);
/* Releases memory the library returned. */
Z2D_API void z2dgpu_free(void *p);

/* Many independent surfaces in one device pass: for every job, the
 * equivalent of calling painter.fill for its commands in order on its
 * surface (z2d's callers loop over surfaces; there is no batch call in z2d
 * itself).  Surfaces must be in device memory and distinct; the commands
 * index one shared node array.  The work is queued on the context stream and
 * the call returns after launch. */
Z2D_API int z2dgpu_fill_jobs(z2dgpu_ctx *ctx, const z2d_job *jobs, size_t n_jobs,
                             const z2d_node *nodes, size_t n_nodes,
                             const z2d_fill_cmd *cmds, size_t n_cmds);

/* z2dgpu_fill_jobs with fills and strokes mixed: each job's commands are
 * drawn in order on its surface (job.cmd_offset / n_cmds index `cmds`).
 * Stroke polygons are built on the host (in parallel across commands),
 * then every job is drawn in one device pass. */
Z2D_API int z2dgpu_draw_jobs(z2dgpu_ctx *ctx, const z2d_job *jobs, size_t n_jobs,
                             const z2d_node *nodes, size_t n_nodes,
                             const z2d_draw_cmd *cmds, size_t n_cmds);

/* SurfaceCompositor.run (src/compositor.zig:302-440) with 1 or 2 operations.
 * Source/destination surfaces must live where `dst` lives. */
Z2D_API int z2dgpu_composite(z2dgpu_ctx *ctx, z2d_surface *dst, int32_t dst_x,
                             int32_t dst_y, int32_t n_ops,
                             const z2d_operation *ops, int32_t precision);

/* z2dgpu_composite for callers that may not allocate device memory, such as
 * a plugin whose host owns every device allocation, or a per-frame loop in
 * which a cudaMalloc/cudaFree would synchronise the whole device.  It has no
 * counterpart in z2d.  It takes no context: the work is queued on `stream`
 * (a cudaStream_t; NULL = the default stream) of `device`, and the call
 * returns after launch.  `dst` and every surface param must be in device
 * memory (packed formats of any length).  Gradient
 * descriptors go to a fixed device array inside the library, so one call
 * takes at most 4 gradient params (pattern gradients and gradient-sourced
 * dithers); more are rejected with Z2D_ERR_INVALID_ARGUMENT.  Each call
 * writes every descriptor it reads, so nothing has to start at zero.  The
 * array is shared by all calls on a device: calls whose GPU work overlaps
 * (other streams, other threads) race on it, while calls queued in order on
 * one stream do not.  The first call on a device looks up the array's
 * device address, so make that call before any stream capture; the address
 * is kept for the life of the process, so do not use this entry point on a
 * device after cudaDeviceReset there.  A call with gradient params is
 * rejected with Z2D_ERR_INVALID_ARGUMENT while `stream` is capturing: their
 * descriptors are copied from memory that does not outlive the call. */
Z2D_API int z2dgpu_composite_noalloc(int device, void *stream, z2d_surface *dst,
                                     int32_t dst_x, int32_t dst_y, int32_t n_ops,
                                     const z2d_operation *ops, int32_t precision);

/* ---------------------------------------------------------------- serving
 * Continuous batching in front of z2dgpu_fill_jobs, for callers that submit
 * fills for many surfaces from many threads (no counterpart in z2d, whose
 * painter.fill is one synchronous call, src/painter.zig:66-72).  The server
 * runs `lanes` workers, each with its own context and stream: a free lane
 * takes the requests queued at that moment (after at most `max_wait_us` of
 * batching window, up to `max_batch_jobs`) and draws them in one pass, while
 * the other lanes take the requests that keep arriving, so several batches
 * are on the GPU at once.  A request draws either on a caller-owned device
 * surface (z2dgpu_server_submit) or on a surface the server allocates from
 * its device pool (z2dgpu_server_submit_new).  The pool is one allocation
 * made at creation: `pool_bytes`, at most 40 GB and at most 7/8 of the HBM
 * the driver reports free (cudaMemGetInfo); a pool request is admitted into
 * a batch once the pool can hold its surface, in arrival order.  Requests on
 * the same caller-owned surface are drawn in submission order.  Requests are
 * copied at submit, so the caller's node/command/pattern/initial-pixel
 * buffers can be reused when submit returns; caller-owned surfaces and
 * `out` buffers must stay valid until the request completes. */
typedef struct z2dgpu_server z2dgpu_server;

typedef struct z2dgpu_server_opts {
    int32_t max_batch_jobs; /* requests per pass, >= 1 */
    int32_t max_wait_us;    /* batching window after the oldest queued request, >= 0 */
    int32_t lanes;          /* workers drawing batches concurrently, 1..16 */
    int64_t pool_bytes;     /* device surface pool for z2dgpu_server_submit_new; 0 = none */
} z2dgpu_server_opts;

typedef struct z2dgpu_server_stats_t {
    uint64_t batches, requests;
    uint64_t deferred;         /* times a pool request waited for pool space */
    double busy_ms;            /* time the lanes spent drawing, summed */
    int32_t lanes, max_inflight; /* most batches that were being drawn at once */
    int64_t pool_bytes, pool_peak_bytes;
} z2dgpu_server_stats_t;

Z2D_API int z2dgpu_server_create2(z2dgpu_server **server, int device, const z2dgpu_server_opts *opts);
/* z2dgpu_server_create2 with 2 lanes and no pool. */
Z2D_API int z2dgpu_server_create(z2dgpu_server **server, int device, int32_t max_batch_jobs,
                                 int32_t max_wait_us);
/* Queues painter.fill for cmds[0..n_cmds) in order on `surface` (device
 * memory); *ticket identifies the request. */
Z2D_API int z2dgpu_server_submit(z2dgpu_server *server, const z2d_surface *surface,
                                 const z2d_node *nodes, size_t n_nodes,
                                 const z2d_fill_cmd *cmds, size_t n_cmds, uint64_t *ticket);
/* Queues painter.fill for cmds[0..n_cmds) on a new width x height surface
 * of `format` from the server's pool, initialised from `init` (host memory
 * in z2d's layout; NULL: cleared to zero).  When the request completes the
 * drawn pixels are in `out` (host memory, z2d's layout and length; NULL:
 * not read back).  The pool block is released at completion.  A surface
 * larger than the whole pool is Z2D_ERR_OUT_OF_MEMORY; a server without a
 * pool is Z2D_ERR_INVALID_STATE. */
Z2D_API int z2dgpu_server_submit_new(z2dgpu_server *server, int32_t format, int32_t width,
                                     int32_t height, const void *init, void *out,
                                     const z2d_node *nodes, size_t n_nodes,
                                     const z2d_fill_cmd *cmds, size_t n_cmds, uint64_t *ticket);
/* Waits for a request (timeout_ms < 0: no limit) and returns its status, or
 * Z2D_ERR_TIMEOUT if it is still pending (the ticket stays valid).
 * *latency_us (optional) = completion time - submit time. */
Z2D_API int z2dgpu_server_wait(z2dgpu_server *server, uint64_t ticket, int32_t timeout_ms,
                               double *latency_us);
/* Passes run, requests completed and lane busy time so far. */
Z2D_API int z2dgpu_server_stats(z2dgpu_server *server, uint64_t *batches, uint64_t *requests,
                                double *busy_ms);
/* All counters, including the overlap of batches and the pool's use. */
Z2D_API int z2dgpu_server_info(z2dgpu_server *server, z2dgpu_server_stats_t *out);
/* Draws every queued request, then stops the lanes and frees the server. */
Z2D_API int z2dgpu_server_destroy(z2dgpu_server *server);

#endif /* Z2DGPU_H */
