// z2d_internal.h -- host-side internals shared by the library's .cu files:
// the context (stream, device arena, pinned staging), error reporting and
// conversion of C ABI descriptors into device descriptors.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/z2dgpu.h"
#include "stroke.h"
#include "z2d_pixel.cuh"

namespace z2dg {

// thread-local message behind z2dgpu_last_error()
void set_error(const char *msg);
void set_errorf(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

#define Z2D_CUDA(call)                                        \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

// A growable device buffer.
struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    void release();
    template <class T>
    T *as() const { return reinterpret_cast<T *>(ptr); }
};
// A growable pinned host buffer.
struct HostBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    void release();
    template <class T>
    T *as() const { return reinterpret_cast<T *>(ptr); }
};

// The rasteriser's schedule tuner (tune.cu): a pass is keyed by whether it
// draws one surface or many, log2 of its tiles and log2 of the mean fills
// per band list.
struct TuneKey {
    int multi, tiles, load;
    bool operator<(const TuneKey &o) const {
        return multi != o.multi ? multi < o.multi : tiles != o.tiles ? tiles < o.tiles : load < o.load;
    }
};
struct RasterPlan {
    int ctas;       // resident CTAs per SM, 0 = as many as fit
    int order;      // 0 tile order, 1 longest bands first
    int cta_items;  // 1: a queue item is a tile (one CTA), 0: a tile row (one warp)
    int candidate;  // the tuner's candidate being measured, or -1
};
struct TunePending {
    TuneKey key;
    int candidate;
    cudaEvent_t start, stop;
};
TuneKey tune_key(int32_t n_jobs, long long n_tiles, long long n_slots, long long n_gbands);
RasterPlan tune_pick(const TuneKey &k);
void tune_report(const TuneKey &k, int candidate, float ms);
// 1: decided (ctas, order set), 0: still exploring, -1: tuning off
int tune_state(const TuneKey &k, int *ctas, int *order, int *cta_items);

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint64_t launches = 0;
    int sm_count = 0;
    // device scratch, reused across calls on this context
    DevBuf params;      // descriptors uploaded per call (patterns, gradients, fills)
    DevBuf nodes;       // path nodes
    DevBuf node_info;   // per-node flatten info
    DevBuf edges;       // flattened edges
    DevBuf fill_state;  // per-fill device state
    DevBuf counters;    // small counters read back by the host
    DevBuf band_fills;  // ordered fill lists per band
    DevBuf bins;        // per (fill, band) edge lists
    DevBuf bin_offsets; // per (fill, band) offsets/cursors
    DevBuf masks;       // exact-path action masks
    DevBuf surface;     // staging copy of host surfaces
    DevBuf surface2;    // staging for a second host surface (compositor params)
    DevBuf surface3;
    DevBuf scan_tmp;    // temporary storage of device-wide scans
    DevBuf stroke_a;    // device stroker: per node / subpath / stroke state
    DevBuf stroke_b;    // device stroker: per point state
    DevBuf stroke_c;    // device stroker: contour points
    DevBuf curve_pool;  // leaf points of flattened curves (count pass -> emit pass)
    long long pool_demand = 0;  // curve-pool points the last flatten asked for
    // k_raster's schedule when forced by z2dgpu_ctx_set_raster (otherwise the
    // tuner's): resident CTAs per SM (0: as many as fit), queue order (0
    // tile order, 1 longest bands first) and item size (1 tile, 0 tile row)
    bool raster_forced = false;
    int raster_ctas_per_sm = 0;
    int raster_order = 0;
    int raster_cta_items = 1;
    std::vector<TunePending> tune_pending;  // tuner measurements not yet read
    TuneKey last_key{-1, 0, 0};             // key of the last pass
    void tune_collect(bool wait);
    DevBuf tile_order;          // cost-ordered queue: keys, indices, sorted copies, sort scratch
    DevBuf pad_buf;             // padded copies of packed surfaces (PackedPads)
    // dashed strokes' polygons of z2dgpu_draw_jobs, kept with their
    // capacity across calls (building them then touches no fresh pages)
    std::vector<stroke::Polygon> poly_cache;
    HostBuf staging;    // pinned upload staging
    HostBuf readback;   // pinned readback
    // the one-upload path of few short fills (fill.cu, run_small_jobs):
    // two pinned staging slots, each free again once its upload event has
    // passed, and the device copy of the latest upload (stream ordered)
    HostBuf small_stage[2];
    cudaEvent_t small_done[2] = {nullptr, nullptr};
    int small_slot = 0;
    DevBuf small_params;
    cudaEvent_t done = nullptr;
    // upload of a host surface overlapping the flatten kernels: the copy runs
    // on copy_stream after call_start (the call's first point on `stream`);
    // `stream` waits for surface_ready before the first kernel that reads the
    // surface (surface_pending says whether that wait is still owed)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t call_start = nullptr, surface_ready = nullptr;
    bool surface_pending = false;
    // Makes `stream` wait for a pending surface upload (no-op otherwise).
    int await_surface();
    // kernel timing (z2dgpu_ctx_set_timing)
    bool timing = false;
    struct Timer {
        std::vector<cudaEvent_t> pending;  // start/stop pairs not yet read
        double ms = 0;
        uint64_t n = 0;
    } t_raster, t_composite, t_flatten, t_bins, t_stroke, t_export;
    cudaEvent_t timer_begin(Timer &t);
    void timer_end(Timer &t, cudaEvent_t start);
    void timer_collect(Timer &t);
};

}  // namespace z2dg

namespace z2dg {
// The PNG exporter (png.cu): the unfiltered scanline stream of a device
// surface as export_png.zig encodes it, and the whole PNG file.
int png_scanlines(Ctx &c, const DevSurface &s, int profile, std::vector<uint8_t> &raw);
int png_file(Ctx &c, const DevSurface &s, int profile, std::vector<uint8_t> &png);
}  // namespace z2dg

// The opaque handle of include/z2dgpu.h is a context.
struct z2dgpu_ctx : public z2dg::Ctx {};

namespace z2dg {
// Packed (alpha4 / alpha2 / alpha1) pixels are updated with 32-bit word
// atomics, which would reach up to 3 bytes past a surface buffer of z2d's
// exact length (ceil(w * h * bits / 8)).  Such a surface -- packed, its
// length not a whole number of words, not already in one of the context's
// padded staging buffers -- is drawn on a padded copy in c.pad_buf: copied
// in when the guard starts, its own length copied back by finish(), which
// also points the surface back at the caller's buffer.  An error path that
// never calls finish() leaves the caller's surface as it was.
struct PackedPads {
    struct Entry {
        uint8_t *orig, *pad;
        size_t len;
        DevSurface *sfc;
    };
    std::vector<Entry> list;
    template <class SfcOf>
    int begin(Ctx &c, size_t n, SfcOf sfc_of) {
        auto staged = [&](const uint8_t *p) {
            for (DevBuf *b : {&c.surface, &c.surface2, &c.surface3})
                if (b->ptr && p >= b->as<uint8_t>() && p < b->as<uint8_t>() + b->cap) return true;
            return false;
        };
        size_t total = 0;
        for (size_t j = 0; j < n; j++) {
            DevSurface &s = sfc_of(j);
            const size_t len = ((size_t)s.w * (size_t)s.h * (size_t)fmt_bits(s.fmt) + 7) / 8;
            if (!fmt_packed(s.fmt) || len % 4 == 0 || staged(s.data)) continue;
            list.push_back(Entry{s.data, nullptr, len, &s});
            total += (len + 255) & ~(size_t)255;
        }
        if (list.empty()) return Z2D_OK;
        if (c.pad_buf.ensure(total)) return Z2D_ERR_OUT_OF_MEMORY;
        size_t off = 0;
        for (Entry &e : list) {
            e.pad = c.pad_buf.as<uint8_t>() + off;
            const cudaError_t r = cudaMemcpyAsync(e.pad, e.orig, e.len, cudaMemcpyDeviceToDevice, c.stream);
            if (r != cudaSuccess) return cuda_fail(r, "cudaMemcpyAsync (padded surface)");
            e.sfc->data = e.pad;
            off += (e.len + 255) & ~(size_t)255;
        }
        return Z2D_OK;
    }
    int finish(Ctx &c) {
        for (const Entry &e : list) {
            e.sfc->data = e.orig;
            const cudaError_t r = cudaMemcpyAsync(e.orig, e.pad, e.len, cudaMemcpyDeviceToDevice, c.stream);
            if (r != cudaSuccess) return cuda_fail(r, "cudaMemcpyAsync (padded surface)");
        }
        list.clear();
        return Z2D_OK;
    }
};
}  // namespace z2dg

namespace z2dg {

// -------------------------------------------------- descriptor conversion
// Fills `out` for a pattern or compositor param.  Gradients are written to
// `grad_host` (the caller uploads them and patches DevSrc::grad).
// Returns Z2D_OK or an error code.
int make_dev_gradient(const z2d_gradient &g, DevGradient &out);
// Stop tables of the gradients with more than kMaxStops stops: their size,
// and put_ext_stops, which writes them at `host` (to be uploaded to `dev`)
// and points each such gradient of g[0..n) (the copy being uploaded) at its
// table; the caller's gradient descriptions must still be valid.
inline size_t ext_table_bytes(int n_stops) {
    return ((sizeof(float) * (size_t)n_stops + 15) & ~(size_t)15) + sizeof(RGBf) * (size_t)n_stops;
}
size_t ext_stops_bytes(const DevGradient *g, size_t n);
void put_ext_stops(DevGradient *g, size_t n, uint8_t *host, uint8_t *dev);
int make_dev_src_from_pattern(int param_kind, const z2d_pattern &p, DevSrc &out, bool &needs_grad,
                              DevGradient &grad_out);

// --------------------------------------------------------------- kernels
struct CompOp {
    int32_t op;
    DevSrc dst;  // kind SRC_NONE => the destination surface
    DevSrc src;  // kind SRC_NONE => previous result
};
struct CompJob {
    DevSurface dst;
    int32_t n_ops, precision;
    int32_t dst_x, dst_y;   // batch origin
    int32_t dsx;            // first destination column
    int32_t y0, y1;         // destination rows [y0, y1)
    int32_t line_w;         // pixels per row
    CompOp ops[2];
};
int launch_composite(Ctx &c, const CompJob &job);
// z2dgpu_fill_jobs on a context (capi.cu); the caller has made c's device current.
int fill_jobs(Ctx &c, const z2d_job *jobs, size_t n_jobs, const z2d_node *nodes, size_t n_nodes,
              const z2d_fill_cmd *cmds, size_t n_cmds);
// Message of the last failing call on this thread.
const char *last_error();
// Launches the whole-surface mask batch [dst_in(pixel, alpha8 mask), op]
// when J has that shape (composite_mask.cu); returns false otherwise.
bool try_mask_batch(Ctx &c, const CompJob &J, bool flat);
// The same batch in float precision (4-byte formats, alpha8) and on the
// packed alpha formats in integer precision (composite_fused.cu); false
// when the surface does not fit the kernel's layout.
bool launch_mask_float(Ctx &c, uint8_t *dst, int fmt, const uint8_t *mask, size_t px, int op, const F4 &spf);
bool launch_mask_packed(Ctx &c, uint8_t *dst, int fmt, const uint8_t *mask, size_t px, int op, const I16 &spx);
// The same batch with a gradient or dithered-gradient source on the 4-byte
// formats in integer precision (composite_grad.cu).
bool try_mask_grad(Ctx &c, const CompJob &J, bool flat);
// Path programs built on the device (path_build.cu).
int build_paths(Ctx &c, const z2d_path_program *progs, size_t n_progs, const z2d_path_cmd *cmds, size_t n_cmds,
                const z2d_glyph_point *gpts, size_t n_gpts, const uint16_t *gends, size_t n_gends, z2d_node *nodes,
                size_t cap_nodes, uint64_t *offsets, int32_t *status);

}  // namespace z2dg
