// capi.cu -- the C ABI of include/z2dgpu.h: contexts, validation that
// mirrors painter.fill's error checks, descriptor preparation, host <->
// device staging, and dispatch into the fill and compositor kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fill.cuh"
#include "host_pool.h"
#include "stroke.h"
#include "stroke_gpu.cuh"
#include "z2d_internal.h"

namespace z2dg {

// Message of the last failing call on this thread.  A fixed buffer, so that
// reporting an error never allocates.
static thread_local char g_err[256];

void set_error(const char *msg) { set_errorf("%s", msg); }
void set_errorf(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}
const char *last_error() { return g_err; }
int cuda_fail(cudaError_t e, const char *what) {
    set_errorf("%s: %s", what, cudaGetErrorString(e));
    return Z2D_ERR_CUDA;
}

int DevBuf::ensure(size_t bytes) {
    if (bytes <= cap) return 0;
    size_t n = std::max(bytes, cap + cap / 2);
    n = (n + 4095) & ~(size_t)4095;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    if (cudaMalloc(&ptr, n) != cudaSuccess) {
        ptr = nullptr;
        set_errorf("device allocation of %zu bytes failed", n);
        return 1;
    }
    cap = n;
    return 0;
}
void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
}
int HostBuf::ensure(size_t bytes) {
    if (bytes <= cap) return 0;
    size_t n = std::max(bytes, cap + cap / 2);
    n = (n + 4095) & ~(size_t)4095;
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    cap = 0;
    if (cudaMallocHost(&ptr, n) != cudaSuccess) {
        ptr = nullptr;
        set_error("pinned host allocation failed");
        return 1;
    }
    cap = n;
    return 0;
}
void HostBuf::release() {
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    cap = 0;
}

cudaEvent_t Ctx::timer_begin(Timer &t) {
    if (!timing) return nullptr;
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    cudaEventRecord(e, stream);
    return e;
}
void Ctx::timer_end(Timer &t, cudaEvent_t start) {
    if (!start) return;
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaEventDestroy(start);
        return;
    }
    cudaEventRecord(e, stream);
    t.pending.push_back(start);
    t.pending.push_back(e);
}
void Ctx::timer_collect(Timer &t) {
    for (size_t i = 0; i + 1 < t.pending.size(); i += 2) {
        float ms = 0;
        cudaEventSynchronize(t.pending[i + 1]);
        if (cudaEventElapsedTime(&ms, t.pending[i], t.pending[i + 1]) == cudaSuccess) {
            t.ms += ms;
            t.n++;
        }
        cudaEventDestroy(t.pending[i]);
        cudaEventDestroy(t.pending[i + 1]);
    }
    t.pending.clear();
}

// ---------------------------------------------- descriptor preparation
// The double-word constants of the gradient's fast offsets (grad_fast.cuh):
// each f64 value split into float hi + lo.  The fast path is left off when
// a constant is not finite or a nonzero one lies outside [2^-60, 2^60]
// (both words of every split are then normal floats).
static void fast_constants(DevGradient &d) {
    GradFast &F = d.fz;
    F.mode = kFastNone;
    bool sane = true;
    auto split = [&](double v) {
        if (!std::isfinite(v) || (v != 0.0 && (std::fabs(v) < 0x1p-60 || std::fabs(v) > 0x1p60))) sane = false;
        DW w;
        w.h = (float)v;
        w.l = std::isfinite(v) ? (float)(v - (double)w.h) : 0.0f;
        return w;
    };
    if (d.has_tf)
        for (int i = 0; i < 6; i++) F.tf[i] = split(d.tf[i]);
    F.g0 = split(d.g[0]);
    F.g1 = split(d.g[1]);
    if (d.type == Z2D_GRADIENT_LINEAR) {
        if (d.lin_zero) {
            F.mode = kFastVoid;
            return;
        }
        F.k[0] = split(d.lin_dx);
        F.k[1] = split(d.lin_dy);
        F.k[2] = split(d.lin_inv);
        if (sane) F.mode = kFastLinear;
    } else if (d.type == Z2D_GRADIENT_RADIAL) {
        if (d.inner_r == 0.0 && d.outer_r == 0.0) {
            F.mode = kFastVoid;
            return;
        }
        // the per-pixel products of the f64 code, formed the same way
        const double ir_dr = d.inner_r * d.dr, nir2 = -d.inner_r * d.inner_r;
        const double k[8] = {d.cdx, d.cdy, ir_dr, nir2, d.a, d.inv_a, d.dr, d.min_dr};
        for (int i = 0; i < 8; i++) F.k[i] = split(k[i]);
        if (sane) F.mode = d.a == 0.0 ? kFastRadialA0 : kFastRadial;
    } else {
        F.k[0] = split(d.angle);
        if (sane) F.mode = kFastConic;
    }
}

int make_dev_gradient(const z2d_gradient &g, DevGradient &out) {
    memset(&out, 0, sizeof(out));
    if (g.n_stops < 0 || (g.n_stops > 0 && !g.stops)) {
        set_error("gradient: bad stop list");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (g.type < Z2D_GRADIENT_LINEAR || g.type > Z2D_GRADIENT_CONIC || g.method < 0 || g.method > Z2D_INTERP_HSL_DECREASING) {
        set_error("gradient: bad type or interpolation method");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    out.type = g.type;
    out.method = g.method;
    out.n_stops = g.n_stops;
    static const double ident[6] = {1, 0, 0, 1, 0, 0};
    out.has_tf = 0;
    for (int i = 0; i < 6; i++) {
        out.g[i] = g.geom[i];
        out.tf[i] = g.transform[i];
        if (!(g.transform[i] == ident[i])) out.has_tf = 1;  // Transformation.equal
    }
    // Stop.List.addAssumeCapacity: clamp, then order by (offset, insertion)
    struct S {
        float off;
        int idx;
    };
    if (g.n_stops > kMaxStops) {
        out.src = &g;  // the table is built where the descriptors are uploaded (put_ext_stops)
    }
    S order[kMaxStops];  // stable insertion sort on the stack (no allocation)
    for (int i = 0; i < g.n_stops && i < kMaxStops && g.n_stops <= kMaxStops; i++) {
        const S v{std::fmax(0.0f, std::fmin(g.stops[i].offset, 1.0f)), i};
        int j = i;
        for (; j > 0 && v.off < order[j - 1].off; j--) order[j] = order[j - 1];
        order[j] = v;
    }
    for (int i = 0; i < g.n_stops && g.n_stops <= kMaxStops; i++) {
        const z2d_color &col = g.stops[order[i].idx].color;
        out.offsets[i] = order[i].off;
        out.prep[i] = prepare_stop(g.method, col);
    }
    if (g.type == Z2D_GRADIENT_LINEAR) {  // Linear.getOffset's per-gradient terms (src/gradient.zig:355-359)
        out.lin_dx = g.geom[2] - g.geom[0];
        out.lin_dy = g.geom[3] - g.geom[1];
        double dist = 0.0;
        dist += out.lin_dx * out.lin_dx;
        dist += out.lin_dy * out.lin_dy;
        out.lin_zero = dist == 0.0;
        out.lin_inv = out.lin_zero ? 0.0 : 1.0 / dist;
    }
    if (g.type == Z2D_GRADIENT_RADIAL) {  // Radial.initBuffer (src/gradient.zig:401-438)
        const double ir = std::fmax(0.0, g.geom[2]), orr = std::fmax(0.0, g.geom[5]);
        out.inner_r = ir;
        out.outer_r = orr;
        out.cdx = g.geom[3] - g.geom[0];
        out.cdy = g.geom[4] - g.geom[1];
        out.dr = orr - ir;
        out.min_dr = -ir;
        double a = 0;
        a += out.cdx * out.cdx;
        a += out.cdy * out.cdy;
        a += out.dr * -out.dr;
        out.a = a;
        out.inv_a = (a != 0) ? 1 / a : 0;
    } else if (g.type == Z2D_GRADIENT_CONIC) {  // Conic.initBuffer (:666-681)
        const double twopi = 6.283185307179586;
        const double r = std::fmod(g.geom[2], twopi);
        out.angle = g.geom[2] < 0.0 ? std::fmod(r + twopi, twopi) : r;
    }
    fast_constants(out);
    return Z2D_OK;
}

size_t ext_stops_bytes(const DevGradient *g, size_t n) {
    size_t b = 0;
    for (size_t i = 0; i < n; i++)
        if (g[i].n_stops > kMaxStops) b += ext_table_bytes(g[i].n_stops);
    return b;
}

void put_ext_stops(DevGradient *g, size_t n, uint8_t *host, uint8_t *dev) {
    size_t off = 0;
    std::vector<std::pair<float, int>> order;
    for (size_t i = 0; i < n; i++) {
        DevGradient &d = g[i];
        if (d.n_stops <= kMaxStops || !d.src) continue;
        const z2d_gradient &src = *d.src;
        // Stop.List.addAssumeCapacity (src/gradient.zig:797-811): clamped
        // offsets in ascending order, equal offsets in insertion order
        order.resize((size_t)src.n_stops);
        for (int k = 0; k < src.n_stops; k++)
            order[(size_t)k] = {std::fmax(0.0f, std::fmin(src.stops[k].offset, 1.0f)), k};
        std::stable_sort(order.begin(), order.end(),
                         [](const std::pair<float, int> &a, const std::pair<float, int> &b) { return a.first < b.first; });
        const size_t o_off = off, o_prep = off + ((sizeof(float) * (size_t)src.n_stops + 15) & ~(size_t)15);
        float *ho = reinterpret_cast<float *>(host + o_off);
        RGBf *hp = reinterpret_cast<RGBf *>(host + o_prep);
        for (int k = 0; k < src.n_stops; k++) {
            ho[k] = order[(size_t)k].first;
            hp[k] = prepare_stop(src.method, src.stops[order[(size_t)k].second].color);
        }
        d.ext_off = reinterpret_cast<const float *>(dev + o_off);
        d.ext_prep = reinterpret_cast<const RGBf *>(dev + o_prep);
        off += ext_table_bytes(src.n_stops);
    }
}

static bool valid_format(int f) { return f >= Z2D_FORMAT_ARGB && f <= Z2D_FORMAT_ALPHA1; }

static int check_pixel(const z2d_pixel &p) {
    if (!valid_format(p.format)) {
        set_error("pixel: bad format");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (fmt_packed(p.format) && p.a > fmt_max(p.format)) {
        set_error("pixel: alpha out of range for its format");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    return Z2D_OK;
}

int make_dev_src_from_pattern(int param_kind, const z2d_pattern &p, DevSrc &out, bool &needs_grad, DevGradient &grad_out) {
    memset(&out, 0, sizeof(out));
    needs_grad = false;
    out.kind = param_kind == Z2D_PARAM_PIXEL ? SRC_PIXEL : param_kind == Z2D_PARAM_GRADIENT ? SRC_GRADIENT : SRC_DITHER;
    if (out.kind == SRC_PIXEL || (out.kind == SRC_DITHER && p.dither_source == Z2D_DITHER_SRC_PIXEL)) {
        const int rc = check_pixel(p.pixel);
        if (rc) return rc;
        out.px = Px{p.pixel.format, p.pixel.r, p.pixel.g, p.pixel.b, p.pixel.a};
        out.pix = i16_from_pixel(out.px);
        out.pixf = F4{(float)out.pix.r / 255.0f, (float)out.pix.g / 255.0f, (float)out.pix.b / 255.0f, (float)out.pix.a / 255.0f};
    }
    if (out.kind == SRC_GRADIENT || (out.kind == SRC_DITHER && p.dither_source == Z2D_DITHER_SRC_GRADIENT)) {
        if (!p.gradient) {
            set_error("pattern: gradient missing");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
        const int rc = make_dev_gradient(*p.gradient, grad_out);
        if (rc) return rc;
        needs_grad = true;
        out.grad_type = grad_out.type;
        out.grad_method = grad_out.method;
    }
    if (out.kind == SRC_DITHER) {
        if (p.dither_type < Z2D_DITHER_NONE || p.dither_type > Z2D_DITHER_BLUE_NOISE || p.dither_scale < 1 || p.dither_scale > 15 ||
            p.dither_source < Z2D_DITHER_SRC_PIXEL || p.dither_source > Z2D_DITHER_SRC_GRADIENT) {
            set_error("dither: bad type, source or scale");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
        out.dither_type = p.dither_type;
        out.dither_source = p.dither_source;
        out.dither_scale = p.dither_scale;
        if (p.dither_source == Z2D_DITHER_SRC_PIXEL) {
            // LinearRGB.decodeRGBA: integer demultiply, then /255 (src/color.zig:261-269)
            I16 v = out.pix;
            if (v.a == 0) v = I16{0, 0, 0, 0};
            else v = I16{(v.r * 255 / v.a) & 0xFFu, (v.g * 255 / v.a) & 0xFFu, (v.b * 255 / v.a) & 0xFFu, v.a};
            out.dither_base = RGBf{(float)v.r / 255.0f, (float)v.g / 255.0f, (float)v.b / 255.0f, (float)v.a / 255.0f};
        } else if (p.dither_source == Z2D_DITHER_SRC_COLOR) {
            // LinearRGB.fromColor (src/color.zig:227-249), same arithmetic
            // on the host (compiled without FP contraction)
            if (p.dither_color.space < Z2D_COLOR_LINEAR_RGB || p.dither_color.space > Z2D_COLOR_HSL) {
                set_error("dither: bad color space");
                return Z2D_ERR_INVALID_ARGUMENT;
            }
            out.dither_base = linear_from_color(p.dither_color);
        }
    }
    return Z2D_OK;
}

static bool pixel_premultiplied(const z2d_pixel &p) {  // canDemultiply (src/pixel.zig:504-514)
    if (p.format != Z2D_FORMAT_ARGB && p.format != Z2D_FORMAT_RGBA) return true;
    if (p.a == 0) return true;
    const int ch[3] = {p.r, p.g, p.b};
    for (int v : ch)
        if (v * 255 / p.a > 255) return false;
    return true;
}

// The node checks of painter.fill in one pass: PathNode.isClosedNodeSet
// (src/internal/path_nodes.zig:23-36), then per node in order its tag, a
// current point for line_to / curve_to (fill_plotter.zig reports
// InvalidState), finite coordinates and z2d's +-2^24 coordinate range.
// PathNotClosed takes precedence over the per-node errors.
static int check_nodes(const z2d_node *nodes, size_t n) {
    bool closed = false, closed_ok = true, seen_move = false;
    size_t bad = n;  // first node failing a per-node check
    for (size_t i = 0; i < n; i++) {
        const z2d_node &nd = nodes[i];
        const int32_t tag = nd.tag;
        if (tag == Z2D_MOVE_TO) {
            if (!closed && i != 0) closed_ok = false;
            seen_move = true;
        } else if (tag == Z2D_CLOSE_PATH) {
            closed = true;
        } else {
            closed = false;
        }
        if (bad < n) continue;
        if (tag < Z2D_MOVE_TO || tag > Z2D_CLOSE_PATH || ((tag == Z2D_LINE_TO || tag == Z2D_CURVE_TO) && !seen_move)) {
            bad = i;
            continue;
        }
        // |p| <= 2^24 is false for NaN and the infinities as well
        const int np = tag == Z2D_CURVE_TO ? 6 : tag == Z2D_CLOSE_PATH ? 0 : 2;
        bool ok = true;
        for (int k = 0; k < np; k++) ok &= std::fabs(nd.p[k]) <= 16777216.0;
        if (!ok) bad = i;
    }
    if (!closed_ok || !closed) {
        set_error("PathNotClosed");
        return Z2D_ERR_PATH_NOT_CLOSED;
    }
    if (bad == n) return Z2D_OK;
    const z2d_node &nd = nodes[bad];
    if (nd.tag < Z2D_MOVE_TO || nd.tag > Z2D_CLOSE_PATH) {
        set_error("node: bad tag");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (nd.tag == Z2D_LINE_TO || nd.tag == Z2D_CURVE_TO) {
        bool moved = false;
        for (size_t i = 0; i < bad && !moved; i++) moved = nodes[i].tag == Z2D_MOVE_TO;
        if (!moved) {
            set_error("InvalidState: line_to/curve_to without a current point");
            return Z2D_ERR_INVALID_STATE;
        }
    }
    const int np = nd.tag == Z2D_CURVE_TO ? 6 : 2;
    for (int k = 0; k < np; k++) {
        if (!std::isfinite(nd.p[k])) {
            set_error("InvalidState: non-finite coordinate");
            return Z2D_ERR_INVALID_STATE;
        }
        if (std::fabs(nd.p[k]) > 16777216.0) break;
    }
    set_error("coordinate outside +-2^24 (z2d's Path clamps to the i24 range)");
    return Z2D_ERR_INVALID_ARGUMENT;
}

// The validation of painter.fill (src/painter.zig:73-91) plus the
// conditions under which fill_plotter.plot reports InvalidState.
static int check_fill(const z2d_pattern &p, const z2d_node *nodes, size_t n, const z2d_fill_opts &o) {
    if (p.kind == Z2D_PATTERN_PIXEL) {
        const int rc = check_pixel(p.pixel);
        if (rc) return rc;
        if (!pixel_premultiplied(p.pixel)) {
            set_error("PixelSourceNotPreMultiplied");
            return Z2D_ERR_PIXEL_NOT_PREMULTIPLIED;
        }
    } else if (p.kind != Z2D_PATTERN_GRADIENT && p.kind != Z2D_PATTERN_DITHER) {
        set_error("pattern: bad kind");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (o.op < 0 || o.op >= Z2D_OP_COUNT || (o.fill_rule != Z2D_FILL_NON_ZERO && o.fill_rule != Z2D_FILL_EVEN_ODD) ||
        o.anti_aliasing < Z2D_AA_NONE || o.anti_aliasing > Z2D_AA_SUPERSAMPLE_4X ||
        (o.precision != Z2D_PRECISION_INTEGER && o.precision != Z2D_PRECISION_FLOAT) || !(o.tolerance == o.tolerance)) {
        set_error("fill options out of range");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return Z2D_OK;
    if (!nodes) return Z2D_ERR_INVALID_ARGUMENT;
    return check_nodes(nodes, n);
}

static int check_surface(const z2d_surface *s) {
    if (!s) return Z2D_ERR_INVALID_ARGUMENT;
    if (!valid_format(s->format)) {
        set_error("surface: bad format");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (s->width < 1 || s->height < 1) {
        set_error(s->width < 1 ? "InvalidWidth" : "InvalidHeight");
        return Z2D_ERR_INVALID_DIMENSIONS;
    }
    if (!s->data || (s->location != Z2D_MEM_HOST && s->location != Z2D_MEM_DEVICE)) return Z2D_ERR_INVALID_ARGUMENT;
    if (s->location == Z2D_MEM_DEVICE && fmt_bits(s->format) >= 32 && (reinterpret_cast<uintptr_t>(s->data) & 3)) {
        set_error("surface: device data of 32-bit formats must be 4-byte aligned");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (s->location == Z2D_MEM_DEVICE && fmt_packed(s->format) && (reinterpret_cast<uintptr_t>(s->data) & 3)) {
        set_error("surface: device data of packed formats must be 4-byte aligned");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    return Z2D_OK;
}

static size_t sfc_bytes(const z2d_surface &s) { return ((size_t)s.width * (size_t)s.height * (size_t)fmt_bits(s.format) + 7) / 8; }

// A packed device surface whose length is not a whole number of 32-bit
// words: its word atomics need a padded copy (see PackedPads).
static bool needs_pad(const z2d_surface &s) {
    return s.location == Z2D_MEM_DEVICE && fmt_packed(s.format) && sfc_bytes(s) % 4 != 0;
}

// Device view of a surface; host surfaces, and packed device surfaces of an
// odd length, are staged through `buf` (sized up to a 16-byte multiple so
// packed word atomics stay in bounds).
static int stage_in(Ctx &c, const z2d_surface &s, DevBuf &buf, DevSurface &out) {
    out.fmt = s.format;
    out.w = s.width;
    out.h = s.height;
    if (s.location == Z2D_MEM_DEVICE && !needs_pad(s)) {
        out.data = reinterpret_cast<uint8_t *>(s.data);
        return Z2D_OK;
    }
    const size_t bytes = sfc_bytes(s);
    if (buf.ensure(((bytes + 15) & ~(size_t)15) + 16)) return Z2D_ERR_OUT_OF_MEMORY;
    Z2D_CUDA(cudaMemcpyAsync(buf.ptr, s.data, bytes,
                             s.location == Z2D_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c.stream));
    out.data = buf.as<uint8_t>();
    return Z2D_OK;
}
// stage_in with the copy on the context's copy stream, so that it overlaps
// the work queued on c.stream before the first await_surface().
static int stage_in_async(Ctx &c, const z2d_surface &s, DevBuf &buf, DevSurface &out) {
    if (s.location == Z2D_MEM_DEVICE) return stage_in(c, s, buf, out);
    if (!c.copy_stream) {
        Z2D_CUDA(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
        Z2D_CUDA(cudaEventCreateWithFlags(&c.call_start, cudaEventDisableTiming));
        Z2D_CUDA(cudaEventCreateWithFlags(&c.surface_ready, cudaEventDisableTiming));
    }
    out.fmt = s.format;
    out.w = s.width;
    out.h = s.height;
    const size_t bytes = sfc_bytes(s);
    if (buf.ensure(((bytes + 15) & ~(size_t)15) + 16)) return Z2D_ERR_OUT_OF_MEMORY;
    // after everything already queued on c.stream (earlier users of buf)
    Z2D_CUDA(cudaEventRecord(c.call_start, c.stream));
    Z2D_CUDA(cudaStreamWaitEvent(c.copy_stream, c.call_start, 0));
    Z2D_CUDA(cudaMemcpyAsync(buf.ptr, s.data, bytes, cudaMemcpyHostToDevice, c.copy_stream));
    Z2D_CUDA(cudaEventRecord(c.surface_ready, c.copy_stream));
    c.surface_pending = true;
    out.data = buf.as<uint8_t>();
    return Z2D_OK;
}
int Ctx::await_surface() {
    if (!surface_pending) return Z2D_OK;
    surface_pending = false;
    Z2D_CUDA(cudaStreamWaitEvent(stream, surface_ready, 0));
    return Z2D_OK;
}
// Ends a call that staged its surface with stage_in_async: on every path
// out of the call the upload is awaited (the caller's host memory must not be
// read after the call returns).
struct SurfaceUploadGuard {
    Ctx &c;
    ~SurfaceUploadGuard() {
        if (c.surface_pending) {
            c.surface_pending = false;
            cudaEventSynchronize(c.surface_ready);
        }
    }
};

static int stage_out(Ctx &c, const z2d_surface &s, const DevSurface &d) {
    if (s.location == Z2D_MEM_DEVICE) {
        if (needs_pad(s))  // back from the padded copy, in stream order
            Z2D_CUDA(cudaMemcpyAsync(s.data, d.data, sfc_bytes(s), cudaMemcpyDeviceToDevice, c.stream));
        return Z2D_OK;
    }
    {
        const int rc = c.await_surface();
        if (rc) return rc;
    }
    Z2D_CUDA(cudaMemcpyAsync(s.data, d.data, sfc_bytes(s), cudaMemcpyDeviceToHost, c.stream));
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    return Z2D_OK;
}

// One fill command prepared for the device: painter.fill's checks, its
// anti-aliasing, precision and tolerance adjustments, and the pattern as a
// compositor source (grad receives a gradient's table when needs_grad).
static int prepare_fill(const z2d_surface &s, int32_t job, const z2d_node *nodes, size_t n_nodes,
                        const z2d_fill_cmd &cm, FillCmd &F, DevGradient &grad, bool &needs_grad) {
    needs_grad = false;
    if (!cm.pattern) return Z2D_ERR_INVALID_ARGUMENT;
    if (cm.node_offset > n_nodes || cm.n_nodes > n_nodes - cm.node_offset) {
        set_error("fill command outside the node array");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    int rc = check_fill(*cm.pattern, nodes + cm.node_offset, cm.n_nodes, cm.opts);
    if (rc || cm.n_nodes == 0) return rc;  // painter.fill returns early on an empty path
    // painter.fill's AA choice (painter.zig:86-97): alpha1 surfaces
    // always draw without anti-aliasing; default is multisample
    const int aa = (s.format == Z2D_FORMAT_ALPHA1) ? Z2D_AA_NONE : cm.opts.anti_aliasing;
    memset(&F, 0, sizeof(F));
    F.node_off = (int32_t)cm.node_offset;
    F.n_nodes = (int32_t)cm.n_nodes;
    F.job = job;
    F.stroke = -1;
    F.poly = -1;
    F.aa = (aa == Z2D_AA_NONE || aa == Z2D_AA_SUPERSAMPLE_4X) ? aa : Z2D_AA_MULTISAMPLE_4X;
    F.rule = cm.opts.fill_rule;
    F.op = cm.opts.op;
    F.precision = requires_float(F.op) ? Z2D_PRECISION_FLOAT : cm.opts.precision;
    F.tol = std::fmax(cm.opts.tolerance, 0.001);
    F.scale = F.aa == Z2D_AA_NONE ? 1.0 : 4.0;
    F.edge_scale = F.scale;
    F.pattern_kind = cm.pattern->kind;
    const int pk = cm.pattern->kind == Z2D_PATTERN_PIXEL      ? Z2D_PARAM_PIXEL
                   : cm.pattern->kind == Z2D_PATTERN_GRADIENT ? Z2D_PARAM_GRADIENT
                                                              : Z2D_PARAM_DITHER;
    rc = make_dev_src_from_pattern(pk, *cm.pattern, F.src, needs_grad, grad);
    if (rc) return rc;
    if (F.pattern_kind == Z2D_PATTERN_PIXEL) {
        const Px px = F.src.px;
        bool opaque = (px.fmt == Z2D_FORMAT_XRGB || px.fmt == Z2D_FORMAT_RGB) ? true : px.a == fmt_max(px.fmt);
        F.reduces = (F.op == Z2D_OP_SRC) || (F.op == Z2D_OP_SRC_OVER && opaque);
        F.px_paint = convert_px(px, s.format);
        F.px_rgba = to_i16(convert_px(px, Z2D_FORMAT_RGBA));
        if (F.op == Z2D_OP_SRC_OVER && F.precision == Z2D_PRECISION_INTEGER) F.fast_kind = FAST_PIXEL_SRC_OVER;
    }
    return Z2D_OK;
}

// Appends the prepared commands of a list of fills on surface `s` (job
// `job` of the batch), skipping empty paths.  Large lists are prepared on
// the host pool, 64 commands per task; the first failing command in list
// order decides the error.
static int prepare_fills(const z2d_surface &s, int32_t job, const z2d_node *nodes, size_t n_nodes,
                         const z2d_fill_cmd *cmds, size_t n_cmds, std::vector<FillCmd> &fills,
                         std::vector<DevGradient> &grads, std::vector<int32_t> &grad_of_fill) {
    if (n_nodes > 0x7FFFFFFF || n_cmds > 0x7FFFFFF || fills.size() + n_cmds > 0x7FFFFFF) {
        set_error("batch too large");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    constexpr size_t kTask = 64;
    if (n_cmds < 2 * kTask) {
        for (size_t i = 0; i < n_cmds; i++) {
            FillCmd F;
            DevGradient g;
            bool needs_grad;
            const int rc = prepare_fill(s, job, nodes, n_nodes, cmds[i], F, g, needs_grad);
            if (rc) return rc;
            if (cmds[i].n_nodes == 0) continue;
            grad_of_fill.push_back(needs_grad ? (int32_t)grads.size() : -1);
            if (needs_grad) grads.push_back(g);
            fills.push_back(F);
        }
        return Z2D_OK;
    }
    // commands are prepared in place at fills[base + i]; a gradient table
    // can only come from a command whose pattern is not a pixel, and goes
    // to its slot among those
    const size_t base = fills.size(), gbase = grads.size();
    std::vector<int32_t> slot(n_cmds);
    size_t n_slots = 0;
    for (size_t i = 0; i < n_cmds; i++)
        slot[i] = (cmds[i].pattern && cmds[i].pattern->kind != Z2D_PATTERN_PIXEL) ? (int32_t)n_slots++ : -1;
    fills.resize(base + n_cmds);
    grads.resize(gbase + n_slots);
    std::vector<uint8_t> NG(n_cmds);
    std::vector<int> RC(n_cmds, 0);
    HostPool::get().run((n_cmds + kTask - 1) / kTask, [&](size_t t) {
        DevGradient scratch;
        for (size_t i = t * kTask, e = std::min(n_cmds, i + kTask); i < e; i++) {
            bool needs_grad = false;
            DevGradient &g = slot[i] >= 0 ? grads[gbase + (size_t)slot[i]] : scratch;
            RC[i] = prepare_fill(s, job, nodes, n_nodes, cmds[i], fills[base + i], g, needs_grad);
            NG[i] = needs_grad && slot[i] >= 0;
            if (needs_grad && slot[i] < 0) RC[i] = Z2D_ERR_INVALID_ARGUMENT;  // not reached: pixels need no table
        }
    });
    // keep the non-empty commands and the tables they use, in order
    size_t nf = base, ng = gbase;
    for (size_t i = 0; i < n_cmds; i++) {
        if (RC[i]) {  // again on this thread, for its message
            fills.resize(base);
            grads.resize(gbase);
            FillCmd f;
            DevGradient g;
            bool needs_grad;
            const int rc = prepare_fill(s, job, nodes, n_nodes, cmds[i], f, g, needs_grad);
            return rc ? rc : Z2D_ERR_INVALID_ARGUMENT;
        }
        if (cmds[i].n_nodes == 0) continue;
        if (NG[i]) {
            if (ng != gbase + (size_t)slot[i]) grads[ng] = grads[gbase + (size_t)slot[i]];
            grad_of_fill.push_back((int32_t)ng++);
        } else {
            grad_of_fill.push_back(-1);
        }
        if (nf != base + i) fills[nf] = fills[base + i];
        nf++;
    }
    fills.resize(nf);
    grads.resize(ng);
    return Z2D_OK;
}

// painter.fill draws each path from its own nodes: the node ranges of the
// fills (stroke fills own none) must not overlap.
static int check_fills_disjoint(const std::vector<FillCmd> &fills) {
    bool sorted = true;
    int64_t end = 0;
    for (const FillCmd &F : fills) {
        if (F.n_nodes == 0) continue;
        if (F.node_off < end) {
            sorted = false;
            break;
        }
        end = (int64_t)F.node_off + F.n_nodes;
    }
    if (sorted) return Z2D_OK;
    std::vector<std::pair<int32_t, int32_t>> r;
    r.reserve(fills.size());
    for (const FillCmd &F : fills)
        if (F.n_nodes > 0) r.emplace_back(F.node_off, F.n_nodes);
    std::sort(r.begin(), r.end());
    for (size_t i = 1; i < r.size(); i++)
        if ((int64_t)r[i - 1].first + r[i - 1].second > r[i].first) {
            set_error("fill commands must not share nodes");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
    return Z2D_OK;
}

static int do_fill_batch(Ctx &c, z2d_surface *surface, const z2d_node *nodes, size_t n_nodes, const z2d_fill_cmd *cmds,
                         size_t n_cmds) {
    int rc = check_surface(surface);
    if (rc) return rc;
    if (n_cmds > 0 && !cmds) return Z2D_ERR_INVALID_ARGUMENT;
    std::vector<FillCmd> fills;
    std::vector<int32_t> grad_of_fill;
    std::vector<DevGradient> grads;
    rc = prepare_fills(*surface, 0, nodes, n_nodes, cmds, n_cmds, fills, grads, grad_of_fill);
    if (rc) return rc;
    if (fills.empty()) return Z2D_OK;
    rc = check_fills_disjoint(fills);
    if (rc) return rc;
    std::vector<DevJob> jobs(1);
    memset(jobs.data(), 0, sizeof(DevJob));
    SurfaceUploadGuard guard{c};
    rc = stage_in_async(c, *surface, c.surface, jobs[0].sfc);
    if (rc) return rc;
    jobs[0].fill0 = 0;
    jobs[0].fill1 = (int32_t)fills.size();
    const DevSurface ds = jobs[0].sfc;
    rc = run_jobs(c, jobs, nodes, (int32_t)n_nodes, fills, grads, grad_of_fill);
    if (rc) return rc;
    return stage_out(c, *surface, ds);
}

// Many surfaces, each with its own ordered fill commands (device surfaces).
int fill_jobs(Ctx &c, const z2d_job *jobs_in, size_t n_jobs, const z2d_node *nodes, size_t n_nodes,
                        const z2d_fill_cmd *cmds, size_t n_cmds) {
    if ((n_jobs > 0 && !jobs_in) || (n_cmds > 0 && !cmds) || (n_nodes > 0 && !nodes)) return Z2D_ERR_INVALID_ARGUMENT;
    if (n_jobs > 0x7FFFFFF) {
        set_error("batch too large");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    std::vector<FillCmd> fills;
    std::vector<int32_t> grad_of_fill;
    std::vector<DevGradient> grads;
    std::vector<DevJob> jobs(n_jobs);
    if (n_jobs > 0) memset(jobs.data(), 0, sizeof(DevJob) * n_jobs);
    for (size_t j = 0; j < n_jobs; j++) {
        const z2d_job &jb = jobs_in[j];
        int rc = check_surface(&jb.surface);
        if (rc) return rc;
        if (jb.surface.location != Z2D_MEM_DEVICE) {
            set_error("fill_jobs: surfaces must be in device memory");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
        if (jb.cmd_offset > n_cmds || jb.n_cmds > n_cmds - jb.cmd_offset) {
            set_error("fill_jobs: job commands outside the command array");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
        jobs[j].sfc = DevSurface{reinterpret_cast<uint8_t *>(jb.surface.data), jb.surface.format, jb.surface.width,
                                 jb.surface.height};
        jobs[j].fill0 = (int32_t)fills.size();
        rc = prepare_fills(jb.surface, (int32_t)j, nodes, n_nodes, cmds + jb.cmd_offset, jb.n_cmds, fills, grads,
                           grad_of_fill);
        if (rc) return rc;
        jobs[j].fill1 = (int32_t)fills.size();
    }
    if (fills.empty()) return Z2D_OK;
    const int rc = check_fills_disjoint(fills);
    if (rc) return rc;
    return run_jobs(c, jobs, nodes, (int32_t)n_nodes, fills, grads, grad_of_fill);
}

// ------------------------------------------------------------------ strokes
// painter.stroke's option handling (painter.zig:221-304) and the stroke
// polygon.  aa receives the anti-aliasing mode actually used.
// painter.stroke's option checks and adjustments (painter.zig:228-304):
// the rasteriser's AA mode and scale, and the plotter options.
static int stroke_options(const z2d_stroke_opts &o, int32_t surface_format, int &aa, stroke::Options &so) {
    if (o.line_join < Z2D_JOIN_MITER || o.line_join > Z2D_JOIN_BEVEL || o.line_cap < Z2D_CAP_BUTT ||
        o.line_cap > Z2D_CAP_SQUARE || o.anti_aliasing < Z2D_AA_NONE || o.anti_aliasing > Z2D_AA_SUPERSAMPLE_4X ||
        !(o.line_width == o.line_width) || !(o.tolerance == o.tolerance) || (o.n_dashes > 0 && !o.dashes)) {
        set_error("stroke options out of range");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (!stroke::transformation_invertible(o.transformation)) {
        set_error("InvalidMatrix: the stroke transformation cannot be inverted");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    aa = (surface_format == Z2D_FORMAT_ALPHA1) ? Z2D_AA_NONE : o.anti_aliasing;
    const bool wide = o.line_width >= 2;
    so.cap = wide ? o.line_cap : Z2D_CAP_BUTT;
    so.join = wide ? o.line_join : Z2D_JOIN_MITER;
    so.miter_limit = wide ? o.miter_limit : 10.0;
    for (int k = 0; k < 6; k++) so.ctm[k] = o.transformation[k];
    so.scale = aa == Z2D_AA_NONE ? 1.0 : 4.0;
    so.thickness = o.line_width >= 0.00390625 ? o.line_width : 0.00390625;
    so.tolerance = std::fmax(o.tolerance, 0.001);
    so.dashes = o.dashes;
    so.n_dashes = (size_t)o.n_dashes;
    so.dash_offset = o.dash_offset;
    return Z2D_OK;
}

// The checks of a non-empty stroke's path and dashes.
static int stroke_checks(const z2d_node *nodes, size_t n_nodes, const z2d_stroke_opts &o) {
    if (!nodes) return Z2D_ERR_INVALID_ARGUMENT;
    for (uint64_t i = 0; i < o.n_dashes; i++)
        if (!(o.dashes[i] == o.dashes[i]) || !(o.dash_offset == o.dash_offset)) {
            set_error("stroke dashes must be numbers");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
    for (size_t i = 0; i < n_nodes; i++)
        if (nodes[i].tag < Z2D_MOVE_TO || nodes[i].tag > Z2D_CLOSE_PATH) {
            set_error("node: bad tag");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
    return Z2D_OK;
}

static int stroke_polygon(const z2d_node *nodes, size_t n_nodes, const z2d_stroke_opts &o, int32_t surface_format,
                          int &aa, stroke::Polygon &contours, double &scale) {
    stroke::Options so;
    contours.clear();
    int rc = stroke_options(o, surface_format, aa, so);
    if (rc) return rc;
    scale = so.scale;
    if (n_nodes == 0) return Z2D_OK;
    rc = stroke_checks(nodes, n_nodes, o);
    if (rc) return rc;
    if (o.hairline) {  // the polylines of polyline_plotter, unscaled
        so.tolerance = o.tolerance;
        scale = 1.0;
        rc = stroke::polyline(nodes, n_nodes, so, contours);
    } else {
        rc = stroke::plot(nodes, n_nodes, so, contours);
    }
    if (rc) set_error("InvalidState: stroke path node sequence");
    return rc;
}

// The device stroker's input for one solid stroke: the subpaths the
// plotter walks (node indices relative to the stroke's nodes) and the pen.
// The node sequence is checked the way the plotter does: line_to /
// curve_to need a current point (stroke_plotter.zig:104-150), and after
// close_path only move_to or close_path may follow.
struct StrokePrep {
    std::vector<SubpathDev> subs;
    int64_t n_local = 0;
    int32_t pen_n = 0;
    bool reflect = false;
};
static int stroke_prepare(const z2d_node *nodes, size_t n_nodes, const stroke::Options &so, StrokePrep &out) {
    out.subs.clear();
    out.n_local = 0;
    SubpathDev cur{};
    bool open = false;
    auto end = [&](bool closed) {
        cur.closed = closed ? 1 : 0;
        out.n_local += cur.n_nodes;
        out.subs.push_back(cur);
        open = false;
    };
    if (n_nodes > 0x7FFFFFFF) return Z2D_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < n_nodes; i++) {
        const z2d_node &nd = nodes[i];
        const int np = nd.tag == Z2D_CURVE_TO ? 6 : nd.tag == Z2D_CLOSE_PATH ? 0 : 2;
        for (int k = 0; k < np; k++)
            if (!std::isfinite(nd.p[k])) {
                set_error("InvalidState: non-finite coordinate");
                return Z2D_ERR_INVALID_STATE;
            }
        switch (nd.tag) {
            case Z2D_MOVE_TO:
                if (open) end(false);
                cur = SubpathDev{};
                cur.node0 = (int32_t)i;
                cur.n_nodes = 1;
                open = true;
                break;
            case Z2D_LINE_TO:
            case Z2D_CURVE_TO:
                if (!open) {
                    set_error("InvalidState: stroke path node sequence");
                    return Z2D_ERR_INVALID_STATE;
                }
                cur.n_nodes++;
                break;
            default:
                if (open) end(true);
                break;
        }
    }
    if (open) end(false);
    out.pen_n = stroke::pen_vertex_count(so.thickness, so.tolerance, so.ctm);
    out.reflect = so.ctm[0] * so.ctm[3] - so.ctm[1] * so.ctm[2] < 0;
    return Z2D_OK;
}

// The fill command of a polygon drawn with a pattern and options (the
// pattern part of prepare_fill), for polygons that come from elsewhere than
// nodes: non-zero rule, points already scaled.
static int prepare_polygon_fill_one(const z2d_surface &s, int32_t job, const z2d_pattern *pattern, int aa,
                                    int32_t op, int32_t precision, double tolerance, FillCmd &F, DevGradient &grad,
                                    bool &needs_grad) {
    z2d_fill_cmd fc;
    memset(&fc, 0, sizeof(fc));
    fc.pattern = pattern;
    fc.opts.anti_aliasing = aa;
    fc.opts.fill_rule = Z2D_FILL_NON_ZERO;  // painter.zig:306-341
    fc.opts.op = op;
    fc.opts.precision = precision;
    fc.opts.tolerance = tolerance;
    // a placeholder closed path so that prepare_fill keeps the command
    z2d_node nd[2];
    memset(nd, 0, sizeof(nd));
    nd[0].tag = Z2D_MOVE_TO;
    nd[1].tag = Z2D_CLOSE_PATH;
    fc.n_nodes = 2;
    const int rc = prepare_fill(s, job, nd, 2, fc, F, grad, needs_grad);
    if (rc) return rc;
    F.node_off = 0;
    F.n_nodes = 0;
    F.edge_scale = 1.0;  // the stroker's points are already scaled
    return Z2D_OK;
}

// A prepared fill drawing a pattern with given options (the pattern part
// of prepare_fills), for polygons that come from elsewhere than nodes.
static int prepare_polygon_fill(const z2d_surface &s, int32_t job, const z2d_pattern *pattern, int aa, int32_t op,
                                int32_t precision, double tolerance, std::vector<FillCmd> &fills,
                                std::vector<DevGradient> &grads, std::vector<int32_t> &grad_of_fill) {
    z2d_fill_cmd fc;
    memset(&fc, 0, sizeof(fc));
    fc.pattern = pattern;
    fc.opts.anti_aliasing = aa;
    fc.opts.fill_rule = Z2D_FILL_NON_ZERO;  // painter.zig:306-341
    fc.opts.op = op;
    fc.opts.precision = precision;
    fc.opts.tolerance = tolerance;
    // one placeholder node so that prepare_fills keeps the command
    z2d_node nd[2];
    memset(nd, 0, sizeof(nd));
    nd[0].tag = Z2D_MOVE_TO;
    nd[1].tag = Z2D_CLOSE_PATH;
    fc.n_nodes = 2;
    const int rc = prepare_fills(s, job, nd, 2, &fc, 1, fills, grads, grad_of_fill);
    if (rc) return rc;
    fills.back().node_off = 0;
    fills.back().n_nodes = 0;
    fills.back().edge_scale = 1.0;  // the stroker's points are already scaled
    return Z2D_OK;
}

// Fills and strokes over many device surfaces.  Solid strokes are
// tessellated on the device from the caller's nodes; dashed strokes are
// built on host threads (each command independently) and uploaded as
// their polygons' points (already scaled); fills use the caller's nodes.
// The caller's node array is uploaded as it is.
// draw_jobs without hairline commands (the caller has checked the
// arguments and the command kinds).
static int draw_core(Ctx &c, const z2d_job *jobs_in, size_t n_jobs, const z2d_node *nodes, size_t n_nodes,
                     const z2d_draw_cmd *cmds, size_t n_cmds) {
    std::vector<size_t> strokes;
    // the surface format decides the stroke's anti-aliasing (alpha1: none)
    std::vector<int32_t> cmd_fmt(n_cmds, Z2D_FORMAT_RGBA);
    for (size_t j = 0; j < n_jobs; j++) {
        const z2d_job &jb = jobs_in[j];
        for (uint64_t k = 0; k < jb.n_cmds; k++) {
            cmd_fmt[jb.cmd_offset + k] = jb.surface.format;
            if (cmds[jb.cmd_offset + k].kind == Z2D_DRAW_STROKE) strokes.push_back(jb.cmd_offset + k);
        }
    }
    // per stroke: options, then the device stroker's input (solid) or the
    // host-built polygon (dashed), in parallel
    const size_t ns = strokes.size();
    if (c.poly_cache.size() < ns) c.poly_cache.resize(ns);
    std::vector<stroke::Polygon> &polys = c.poly_cache;
    std::vector<StrokePrep> preps(ns);
    std::vector<stroke::Options> sopts(ns);
    std::vector<uint8_t> on_device(ns, 0);
    std::vector<int> aas(ns, 0), rcs(ns, 0);
    std::vector<std::string> errs(ns);
    {
        // on the host pool, 16 strokes per task (the pool's threads keep
        // their point arenas between calls)
        constexpr size_t kTask = 16;
        auto work = [&](size_t t) {
            for (size_t k = t * kTask, k1 = std::min(ns, k + kTask); k < k1; k++) {
                polys[k].clear();  // (an earlier call's polygon)
                const z2d_draw_cmd &cm = cmds[strokes[k]];
                if (!cm.pattern || cm.node_offset > n_nodes || cm.n_nodes > n_nodes - cm.node_offset) {
                    rcs[k] = Z2D_ERR_INVALID_ARGUMENT;
                    errs[k] = "stroke command outside the node array";
                    continue;
                }
                const z2d_node *nd = nodes + cm.node_offset;
                int rc = stroke_options(cm.stroke, cmd_fmt[strokes[k]], aas[k], sopts[k]);
                if (!rc && cm.n_nodes > 0) rc = stroke_checks(nd, cm.n_nodes, cm.stroke);
                if (!rc && cm.n_nodes > 0) {
                    if (stroke::dashed(sopts[k])) {
                        rc = stroke::plot(nd, cm.n_nodes, sopts[k], polys[k]);
                        if (rc) set_error("InvalidState: stroke path node sequence");
                    } else {
                        on_device[k] = 1;
                        rc = stroke_prepare(nd, cm.n_nodes, sopts[k], preps[k]);
                    }
                }
                rcs[k] = rc;
                if (rc) errs[k] = last_error();
            }
        };
        HostPool::get().run((ns + kTask - 1) / kTask, work);
        for (size_t k = 0; k < ns; k++)
            if (rcs[k]) {
                set_error(errs[k].c_str());
                return rcs[k];
            }
    }
    std::vector<int64_t> stroke_of(n_cmds, -1);
    for (size_t k = 0; k < ns; k++) stroke_of[strokes[k]] = (int64_t)k;
    // Every (job, command) entry in job order is prepared on the host pool:
    // its fill command (a fill's, or the fill drawing a stroke's polygon)
    // and gradient table; the loop below then assembles them in order, and
    // the first failing entry (or job) in that order decides the error.
    std::vector<int> job_rc(n_jobs, 0);
    std::vector<size_t> ent_job, ent_cmd;
    ent_job.reserve(n_cmds);
    ent_cmd.reserve(n_cmds);
    for (size_t j = 0; j < n_jobs; j++) {
        const z2d_job &jb = jobs_in[j];
        job_rc[j] = check_surface(&jb.surface);
        if (!job_rc[j] && jb.surface.location != Z2D_MEM_DEVICE) job_rc[j] = -1;  // reported below
        if (job_rc[j]) continue;
        for (uint64_t q = 0; q < jb.n_cmds; q++) {
            ent_job.push_back(j);
            ent_cmd.push_back(jb.cmd_offset + q);
        }
    }
    const size_t n_ent = ent_cmd.size();
    std::vector<FillCmd> ent_fill(n_ent);
    std::vector<int32_t> ent_slot(n_ent, -1);  // gradient slot (patterns other than pixels)
    int32_t n_slots = 0;
    for (size_t e = 0; e < n_ent; e++)
        if (cmds[ent_cmd[e]].pattern && cmds[ent_cmd[e]].pattern->kind != Z2D_PATTERN_PIXEL) ent_slot[e] = n_slots++;
    std::vector<DevGradient> ent_grad((size_t)n_slots);
    std::vector<uint8_t> ent_drawn(n_ent, 0), ent_ng(n_ent, 0);
    std::vector<int> ent_rc(n_ent, 0);
    // prepares entry e into the slots above; `scratch` takes a gradient a
    // pixel pattern would never ask for
    auto prepare_entry = [&](size_t e, DevGradient &scratch) -> int {
        const size_t j = ent_job[e], i = ent_cmd[e];
        const z2d_job &jb = jobs_in[j];
        const z2d_draw_cmd &cm = cmds[i];
        DevGradient &g = ent_slot[e] >= 0 ? ent_grad[(size_t)ent_slot[e]] : scratch;
        bool ng = false;
        int rc;
        if (cm.kind == Z2D_DRAW_FILL) {
            z2d_fill_cmd fc;
            fc.pattern = cm.pattern;
            fc.node_offset = cm.node_offset;
            fc.n_nodes = cm.n_nodes;
            fc.opts = cm.fill;
            rc = prepare_fill(jb.surface, (int32_t)j, nodes, n_nodes, fc, ent_fill[e], g, ng);
            if (!rc && cm.n_nodes > 0) ent_drawn[e] = 1;
        } else {
            const size_t k = (size_t)stroke_of[i];
            if (cm.pattern->kind == Z2D_PATTERN_PIXEL && !pixel_premultiplied(cm.pattern->pixel)) {
                set_error("PixelSourceNotPreMultiplied");
                return Z2D_ERR_PIXEL_NOT_PREMULTIPLIED;
            }
            const bool drawn = on_device[k] ? !preps[k].subs.empty() : polys[k].points() > 0;
            if (!drawn) return Z2D_OK;  // nothing is drawn
            rc = prepare_polygon_fill_one(jb.surface, (int32_t)j, cm.pattern, aas[k], cm.stroke.op,
                                          cm.stroke.precision, cm.stroke.tolerance, ent_fill[e], g, ng);
            if (!rc) ent_drawn[e] = 1;
        }
        ent_ng[e] = ng && ent_slot[e] >= 0;
        if (ng && ent_slot[e] < 0) rc = Z2D_ERR_INVALID_ARGUMENT;  // not reached: pixels need no table
        return rc;
    };
    constexpr size_t kTask = 256;
    HostPool::get().run((n_ent + kTask - 1) / kTask, [&](size_t t) {
        DevGradient scratch;
        for (size_t e = t * kTask, e1 = std::min(n_ent, e + kTask); e < e1; e++) ent_rc[e] = prepare_entry(e, scratch);
    });
    std::vector<FillCmd> fills;
    std::vector<int32_t> grad_of_fill;
    std::vector<DevGradient> grads;
    fills.reserve(n_ent);
    grad_of_fill.reserve(n_ent);
    std::vector<DevJob> jobs(n_jobs);
    if (n_jobs > 0) memset(jobs.data(), 0, sizeof(DevJob) * n_jobs);
    StrokeSet sset;
    std::vector<std::pair<int32_t, int32_t>> trig_keys;  // (n, reflect) of each table, in trig order
    std::vector<int32_t> trig_at;
    size_t e = 0;
    for (size_t j = 0; j < n_jobs; j++) {
        const z2d_job &jb = jobs_in[j];
        if (job_rc[j]) {
            if (job_rc[j] > 0) return check_surface(&jb.surface);  // again on this thread, for its message
            set_error("draw_jobs: surfaces must be in device memory");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
        jobs[j].sfc = DevSurface{reinterpret_cast<uint8_t *>(jb.surface.data), jb.surface.format, jb.surface.width,
                                 jb.surface.height};
        jobs[j].fill0 = (int32_t)fills.size();
        for (uint64_t q = 0; q < jb.n_cmds; q++, e++) {
            const size_t i = jb.cmd_offset + q;
            const z2d_draw_cmd &cm = cmds[i];
            if (ent_rc[e]) {  // again on this thread, for its message
                DevGradient scratch;
                const int rc = prepare_entry(e, scratch);
                return rc ? rc : ent_rc[e];
            }
            if (!ent_drawn[e]) continue;
            grad_of_fill.push_back(ent_ng[e] ? (int32_t)grads.size() : -1);
            if (ent_ng[e]) grads.push_back(ent_grad[(size_t)ent_slot[e]]);
            fills.push_back(ent_fill[e]);
            if (cm.kind == Z2D_DRAW_FILL) continue;
            const size_t k = (size_t)stroke_of[i];
            if (!on_device[k]) {  // a host-built polygon
                fills.back().poly = (int32_t)sset.polys.size();
                sset.polys.push_back(&polys[k]);
                continue;
            }
            // a device-stroked command
            StrokePrep &pr = preps[k];
            const stroke::Options &so = sopts[k];
            StrokeDev S;
            memset(&S, 0, sizeof(S));
            S.fill = (int32_t)fills.size() - 1;
            fills.back().stroke = (int32_t)sset.strokes.size();
            S.sub0 = (int32_t)sset.subs.size();
            S.n_sub = (int32_t)pr.subs.size();
            S.join = so.join;
            S.cap = so.cap;
            S.pen_n = pr.pen_n;
            S.pen_off = (int32_t)sset.n_pen;
            S.thickness = so.thickness;
            S.miter_limit = so.miter_limit;
            S.tolerance = so.tolerance;
            S.scale = so.scale;
            for (int t = 0; t < 6; t++) S.ctm[t] = so.ctm[t];
            // the pen's cos/sin table, shared by pens of the same size and handedness
            int32_t tab = -1;
            for (size_t t = 0; t < trig_keys.size(); t++)
                if (trig_keys[t].first == pr.pen_n && trig_keys[t].second == (int32_t)pr.reflect) {
                    tab = trig_at[t];
                    break;
                }
            if (tab < 0) {
                tab = (int32_t)(sset.trig.size() / 2);
                trig_keys.emplace_back(pr.pen_n, (int32_t)pr.reflect);
                trig_at.push_back(tab);
                sset.trig.resize(sset.trig.size() + 2 * (size_t)pr.pen_n);
                stroke::pen_trig(pr.pen_n, pr.reflect, sset.trig.data() + 2 * (size_t)tab);
            }
            S.pen_tab = tab;
            sset.n_pen += pr.pen_n;
            for (SubpathDev sp : pr.subs) {
                sp.node0 += (int32_t)cm.node_offset;
                sp.local0 = (int32_t)sset.n_local;
                sp.stroke = (int32_t)sset.strokes.size();
                sset.n_local += sp.n_nodes;
                sset.subs.push_back(sp);
            }
            sset.strokes.push_back(S);
            if (sset.n_local > 0x7FFFFFFF || sset.n_pen > 0x7FFFFFFF) {
                set_error("batch too large");
                return Z2D_ERR_INVALID_ARGUMENT;
            }
        }
        jobs[j].fill1 = (int32_t)fills.size();
    }
    if (fills.empty()) return Z2D_OK;
    const int rc = check_fills_disjoint(fills);
    if (rc) return rc;
    return run_jobs(c, jobs, nodes, (int32_t)n_nodes, fills, grads, grad_of_fill, &sset);
}

static bool is_hairline(const z2d_draw_cmd &cm) { return cm.kind == Z2D_DRAW_STROKE && cm.stroke.hairline != 0; }

// Hairline strokes: for every job, the hairline commands
// [ranges[j].first, ranges[j].second) of its command list, in order
// (painter.zig:245-262).  The polylines are built on host threads.
static int draw_hairlines(Ctx &c, const z2d_job *jobs_in, size_t n_jobs,
                          const std::vector<std::pair<uint64_t, uint64_t>> &ranges, const z2d_node *nodes,
                          size_t n_nodes, const z2d_draw_cmd *cmds) {
    std::vector<size_t> hc;   // command index
    std::vector<int32_t> hj;  // its job
    for (size_t j = 0; j < n_jobs; j++)
        for (uint64_t k = ranges[j].first; k < ranges[j].second; k++) {
            hc.push_back(jobs_in[j].cmd_offset + k);
            hj.push_back((int32_t)j);
        }
    const size_t nh = hc.size();
    if (nh == 0) return Z2D_OK;
    std::vector<stroke::Polygon> lines(nh);
    std::vector<int> rcs(nh, 0);
    std::vector<std::string> errs(nh);
    {
        const size_t nt = std::max<size_t>(1, std::min<size_t>(std::thread::hardware_concurrency(), nh / 256 + 1));
        std::atomic<size_t> next{0};
        auto work = [&] {
            for (size_t k; (k = next.fetch_add(1)) < nh;) {
                const z2d_draw_cmd &cm = cmds[hc[k]];
                if (!cm.pattern || cm.node_offset > n_nodes || cm.n_nodes > n_nodes - cm.node_offset) {
                    rcs[k] = Z2D_ERR_INVALID_ARGUMENT;
                    errs[k] = "stroke command outside the node array";
                    continue;
                }
                const z2d_node *nd = nodes + cm.node_offset;
                int aa = 0;
                stroke::Options so;
                int rc = stroke_options(cm.stroke, jobs_in[hj[k]].surface.format, aa, so);
                if (!rc && cm.n_nodes > 0) rc = stroke_checks(nd, cm.n_nodes, cm.stroke);
                if (!rc && cm.n_nodes > 0) {
                    so.tolerance = cm.stroke.tolerance;  // the polyline plotter takes it as given
                    rc = stroke::polyline(nd, cm.n_nodes, so, lines[k]);
                    if (rc) set_error("InvalidState: stroke path node sequence");
                    for (double v : lines[k].xy)
                        if (!rc && !(std::fabs(v) < 1073741824.0)) {
                            set_error("InvalidState: hairline coordinate out of range");
                            rc = Z2D_ERR_INVALID_STATE;
                        }
                }
                rcs[k] = rc;
                if (rc) errs[k] = last_error();
            }
        };
        std::vector<std::thread> pool;
        for (size_t t = 1; t < nt; t++) pool.emplace_back(work);
        work();
        for (auto &t : pool) t.join();
        for (size_t k = 0; k < nh; k++)
            if (rcs[k]) {
                set_error(errs[k].c_str());
                return rcs[k];
            }
    }
    std::vector<DevJob> jobs(n_jobs);
    if (n_jobs > 0) memset(jobs.data(), 0, sizeof(DevJob) * n_jobs);
    for (size_t j = 0; j < n_jobs; j++) {
        const z2d_job &jb = jobs_in[j];
        jobs[j].sfc = DevSurface{reinterpret_cast<uint8_t *>(jb.surface.data), jb.surface.format, jb.surface.width,
                                 jb.surface.height};
    }
    std::vector<FillCmd> fills;
    std::vector<DevGradient> grads;
    std::vector<int32_t> grad_of_fill;
    HairSet hs;
    for (size_t k = 0; k < nh; k++) {
        const z2d_draw_cmd &cm = cmds[hc[k]];
        if (cm.pattern->kind == Z2D_PATTERN_PIXEL && !pixel_premultiplied(cm.pattern->pixel)) {
            set_error("PixelSourceNotPreMultiplied");
            return Z2D_ERR_PIXEL_NOT_PREMULTIPLIED;
        }
        if (lines[k].points() == 0) continue;
        const int rc = prepare_polygon_fill(jobs_in[hj[k]].surface, hj[k], cm.pattern, cm.stroke.anti_aliasing,
                                            cm.stroke.op, cm.stroke.precision, cm.stroke.tolerance, fills, grads,
                                            grad_of_fill);
        if (rc) return rc;
        hs.lines.push_back(&lines[k]);
        hs.fill.push_back((int32_t)fills.size() - 1);
        hs.aa_none.push_back(cm.stroke.anti_aliasing == Z2D_AA_NONE ? 1 : 0);
    }
    return run_hairlines(c, jobs, fills, grads, grad_of_fill, hs);
}

// Fills and strokes over many device surfaces, in order per surface.
// Hairline strokes draw as single-pixel composites outside the fill
// pipeline, so a job list with hairlines runs in phases: the commands up to
// each job's next hairlines, then those hairlines, and so on.
static int draw_jobs(Ctx &c, const z2d_job *jobs_in, size_t n_jobs, const z2d_node *nodes, size_t n_nodes,
                     const z2d_draw_cmd *cmds, size_t n_cmds) {
    if ((n_jobs > 0 && !jobs_in) || (n_cmds > 0 && !cmds) || (n_nodes > 0 && !nodes)) return Z2D_ERR_INVALID_ARGUMENT;
    if (n_jobs > 0x7FFFFFF || n_cmds > 0x7FFFFFF || n_nodes > 0x7FFFFFFF) {
        set_error("batch too large");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    bool any_hairline = false;
    for (size_t i = 0; i < n_cmds; i++) {
        if (cmds[i].kind != Z2D_DRAW_STROKE && cmds[i].kind != Z2D_DRAW_FILL) {
            set_error("draw command: bad kind");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
        any_hairline = any_hairline || is_hairline(cmds[i]);
    }
    for (size_t j = 0; j < n_jobs; j++) {
        const z2d_job &jb = jobs_in[j];
        if (jb.cmd_offset > n_cmds || jb.n_cmds > n_cmds - jb.cmd_offset) {
            set_error("draw_jobs: job commands outside the command array");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
    }
    if (!any_hairline) return draw_core(c, jobs_in, n_jobs, nodes, n_nodes, cmds, n_cmds);
    std::vector<uint64_t> cursor(n_jobs, 0);
    std::vector<z2d_job> phase(jobs_in, jobs_in + n_jobs);
    std::vector<std::pair<uint64_t, uint64_t>> hair(n_jobs);
    while (true) {
        bool any = false;
        for (size_t j = 0; j < n_jobs; j++) {  // commands up to the next hairline
            uint64_t e = cursor[j];
            while (e < jobs_in[j].n_cmds && !is_hairline(cmds[jobs_in[j].cmd_offset + e])) e++;
            phase[j].cmd_offset = jobs_in[j].cmd_offset + cursor[j];
            phase[j].n_cmds = e - cursor[j];
            any = any || e > cursor[j];
            cursor[j] = e;
        }
        if (any) {
            const int rc = draw_core(c, phase.data(), n_jobs, nodes, n_nodes, cmds, n_cmds);
            if (rc) return rc;
        }
        bool more = false;
        for (size_t j = 0; j < n_jobs; j++) {  // then the hairlines that follow
            uint64_t e = cursor[j];
            while (e < jobs_in[j].n_cmds && is_hairline(cmds[jobs_in[j].cmd_offset + e])) e++;
            hair[j] = {cursor[j], e};
            more = more || e > cursor[j];
            cursor[j] = e;
        }
        if (!more) break;
        const int rc = draw_hairlines(c, jobs_in, n_jobs, hair, nodes, n_nodes, cmds);
        if (rc) return rc;
    }
    return Z2D_OK;
}

static int do_stroke(Ctx &c, z2d_surface *surface, const z2d_pattern *pattern, const z2d_node *nodes, size_t n_nodes,
                     const z2d_stroke_opts &o) {
    int rc = check_surface(surface);
    if (rc) return rc;
    if (pattern->kind == Z2D_PATTERN_PIXEL) {  // painter.zig:221-227
        rc = check_pixel(pattern->pixel);
        if (rc) return rc;
        if (!pixel_premultiplied(pattern->pixel)) {
            set_error("PixelSourceNotPreMultiplied");
            return Z2D_ERR_PIXEL_NOT_PREMULTIPLIED;
        }
    }
    int aa = 0;
    stroke::Options so;
    rc = stroke_options(o, surface->format, aa, so);
    if (rc || n_nodes == 0) return rc;
    rc = stroke_checks(nodes, n_nodes, o);
    if (rc) return rc;
    // one job on the (staged) surface
    DevSurface ds;
    rc = stage_in(c, *surface, c.surface, ds);
    if (rc) return rc;
    z2d_job jb;
    memset(&jb, 0, sizeof(jb));
    jb.surface = *surface;
    jb.surface.location = Z2D_MEM_DEVICE;
    jb.surface.data = ds.data;
    jb.cmd_offset = 0;
    jb.n_cmds = 1;
    z2d_draw_cmd cm;
    memset(&cm, 0, sizeof(cm));
    cm.kind = Z2D_DRAW_STROKE;
    cm.pattern = pattern;
    cm.node_offset = 0;
    cm.n_nodes = n_nodes;
    cm.stroke = o;
    rc = draw_jobs(c, &jb, 1, nodes, n_nodes, &cm, 1);
    if (rc) return rc;
    return stage_out(c, *surface, ds);
}

// SurfaceCompositor.run's precision upgrade and bounds
// (src/compositor.zig:310-387): fills the geometry of J and sets `empty`
// when nothing is drawn.
static int composite_region(const z2d_surface *dst, int32_t dst_x, int32_t dst_y, int32_t n_ops,
                            const z2d_operation *ops, int32_t precision, CompJob &J, bool &empty) {
    memset(&J, 0, sizeof(J));
    empty = true;
    if (n_ops == 0) return Z2D_OK;
    if (dst_x >= dst->width || dst_y >= dst->height) return Z2D_OK;
    int prec = precision;
    for (int k = 0; k < n_ops; k++) {
        if (ops[k].op < 0 || ops[k].op >= Z2D_OP_COUNT) return Z2D_ERR_INVALID_ARGUMENT;
        if (requires_float(ops[k].op)) prec = Z2D_PRECISION_FLOAT;
    }
    int32_t sw, sh;
    const z2d_param &s0 = ops[0].src;
    if (s0.kind == Z2D_PARAM_NONE) return Z2D_OK;
    if (s0.kind == Z2D_PARAM_SURFACE) {
        const int rc = check_surface(s0.surface);
        if (rc) return rc;
        sw = s0.surface->width;
        sh = s0.surface->height;
    } else {
        if (dst_x != 0 || dst_y != 0) return Z2D_OK;
        sw = dst->width;
        sh = dst->height;
    }
    const int32_t ssx = dst_x < 0 ? -dst_x : 0, ssy = dst_y < 0 ? -dst_y : 0;
    const int32_t width = (sw + dst_x > dst->width) ? dst->width - dst_x : sw;
    const int32_t height = (sh + dst_y > dst->height) ? dst->height - dst_y : sh;
    if (ssx >= width || ssy >= height) return Z2D_OK;
    J.n_ops = n_ops;
    J.precision = prec;
    J.dst_x = dst_x;
    J.dst_y = dst_y;
    J.dsx = ssx + dst_x;
    J.y0 = ssy + dst_y;
    J.y1 = std::max(ssy, height) + dst_y;
    J.line_w = std::max(0, width - ssx);
    empty = false;
    return Z2D_OK;
}

// z2d leaves surface params smaller than the batch region undefined; the
// GPU path rejects them instead of reading out of bounds.
static int check_param_bounds(const CompJob &J) {
    for (int k = 0; k < J.n_ops; k++) {
        const DevSrc &ds = J.ops[k].dst, &ss = J.ops[k].src;
        if (ds.kind == SRC_SURFACE && ((int64_t)ds.sfc.w < (int64_t)J.dsx + J.line_w || ds.sfc.h < J.y1)) {
            set_error("composite: destination surface param smaller than the region");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
        if (ss.kind == SRC_SURFACE &&
            ((int64_t)ss.sfc.w < (int64_t)(J.dsx - J.dst_x) + J.line_w || ss.sfc.h < J.y1 - J.dst_y)) {
            set_error("composite: source surface param smaller than the region");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
    }
    return Z2D_OK;
}

// ------------------------------------------------- allocation-free compositing
// Scratch of z2dgpu_composite_noalloc: the gradient descriptors its
// operations read.  File-scope device memory, so no call allocates; every
// GPU that loads the library holds it until the process exits.
constexpr int kNoAllocGradients = 4;
static __device__ __align__(256) DevGradient g_noalloc_gradients[kNoAllocGradients];

// Device address of g_noalloc_gradients per device, looked up once per
// device (the name is only a host-side stand-in in host code).
constexpr int kMaxDevices = 64;
static DevGradient *g_noalloc_addr[kMaxDevices];
static std::mutex g_noalloc_mu;

static int noalloc_scratch(int device, DevGradient **out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_gradients);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_gradients)");
        g_noalloc_addr[device] = static_cast<DevGradient *>(p);
    }
    *out = g_noalloc_addr[device];
    return Z2D_OK;
}

}  // namespace z2dg

using namespace z2dg;


extern "C" {

Z2D_API const char *z2dgpu_version(void) { return "z2dgpu 0.1.0 (sm_103a)"; }

Z2D_API const char *z2dgpu_last_error(void) { return g_err; }

Z2D_API int z2dgpu_ctx_create(z2dgpu_ctx **out, int device, void *stream) {
    if (!out) return Z2D_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    Z2D_CUDA(cudaSetDevice(device));
    z2dgpu_ctx *c = new z2dgpu_ctx();
    c->device = device;
    if (stream) {
        c->stream = reinterpret_cast<cudaStream_t>(stream);
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete c;
            return cuda_fail(e, "cudaStreamCreate");
        }
        c->own_stream = true;
    }
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (c->sm_count <= 0) c->sm_count = 1;
    *out = c;
    return Z2D_OK;
}

Z2D_API int z2dgpu_ctx_destroy(z2dgpu_ctx *c) {
    if (!c) return Z2D_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    DevBuf *bufs[] = {&c->params, &c->nodes, &c->node_info, &c->edges, &c->fill_state, &c->counters, &c->band_fills,
                      &c->bins, &c->bin_offsets, &c->masks, &c->surface, &c->surface2, &c->surface3, &c->scan_tmp,
                      &c->stroke_a, &c->stroke_b, &c->stroke_c, &c->curve_pool, &c->tile_order, &c->pad_buf,
                      &c->small_params};
    for (DevBuf *b : bufs) b->release();
    c->tune_collect(true);
    c->staging.release();
    c->readback.release();
    for (int i = 0; i < 2; i++) {
        c->small_stage[i].release();
        if (c->small_done[i]) cudaEventDestroy(c->small_done[i]);
    }
    for (Ctx::Timer *t : {&c->t_raster, &c->t_composite, &c->t_flatten, &c->t_bins, &c->t_stroke, &c->t_export}) c->timer_collect(*t);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
        cudaEventDestroy(c->call_start);
        cudaEventDestroy(c->surface_ready);
    }
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    return Z2D_OK;
}

Z2D_API int z2dgpu_ctx_synchronize(z2dgpu_ctx *c) {
    if (!c) return Z2D_ERR_INVALID_ARGUMENT;
    Z2D_CUDA(cudaStreamSynchronize(c->stream));
    return Z2D_OK;
}

Z2D_API uint64_t z2dgpu_ctx_launch_count(const z2dgpu_ctx *c) { return c ? c->launches : 0; }

Z2D_API int z2dgpu_ctx_set_timing(z2dgpu_ctx *c, int enable) {
    if (!c) return Z2D_ERR_INVALID_ARGUMENT;
    for (Ctx::Timer *t : {&c->t_raster, &c->t_composite, &c->t_flatten, &c->t_bins, &c->t_stroke, &c->t_export}) {
        c->timer_collect(*t);
        *t = Ctx::Timer{};
    }
    c->timing = enable != 0;
    return Z2D_OK;
}

Z2D_API int z2dgpu_ctx_set_raster(z2dgpu_ctx *c, int32_t ctas_per_sm, int32_t order, int32_t tile_items) {
    // ctas_per_sm: -2 = the tuner, -1 = one CTA per tile, 0.. = persistent
    if (!c || ctas_per_sm < -2 || ctas_per_sm > 64 ||
        (ctas_per_sm >= -1 && (order < 0 || order > 1 || tile_items < 0 || tile_items > 1)))
        return Z2D_ERR_INVALID_ARGUMENT;
    c->raster_forced = ctas_per_sm >= -1;
    c->raster_ctas_per_sm = ctas_per_sm >= -1 ? ctas_per_sm : 0;
    c->raster_order = ctas_per_sm >= -1 ? order : 0;
    c->raster_cta_items = ctas_per_sm >= -1 ? tile_items : 1;
    return Z2D_OK;
}

Z2D_API int z2dgpu_ctx_raster_tuning(z2dgpu_ctx *c, int32_t *decided, int32_t *ctas_per_sm, int32_t *order,
                                     int32_t *tile_items) {
    if (!c || !decided || !ctas_per_sm || !order || !tile_items) return Z2D_ERR_INVALID_ARGUMENT;
    c->tune_collect(true);
    int ct = 0, od = 0, it = 1;
    const int st = c->last_key.multi < 0 ? 0 : tune_state(c->last_key, &ct, &od, &it);
    *decided = st;
    *ctas_per_sm = ct;
    *order = od;
    *tile_items = it;
    return Z2D_OK;
}

Z2D_API double z2dgpu_ctx_kernel_ms(z2dgpu_ctx *c, const char *kernel, uint64_t *launches) {
    if (!c || !kernel) return -1.0;
    Ctx::Timer *t = nullptr;
    if (strcmp(kernel, "raster") == 0) t = &c->t_raster;
    else if (strcmp(kernel, "composite") == 0) t = &c->t_composite;
    else if (strcmp(kernel, "flatten") == 0) t = &c->t_flatten;
    else if (strcmp(kernel, "bins") == 0) t = &c->t_bins;
    else if (strcmp(kernel, "stroke") == 0) t = &c->t_stroke;
    else if (strcmp(kernel, "export") == 0) t = &c->t_export;
    if (!t) return -1.0;
    c->timer_collect(*t);
    if (launches) *launches = t->n;
    return t->ms;
}

Z2D_API size_t z2dgpu_surface_bytes(int32_t format, int32_t width, int32_t height) {
    if (!valid_format(format) || width < 1 || height < 1) return 0;
    return ((size_t)width * (size_t)height * (size_t)fmt_bits(format) + 7) / 8;
}

Z2D_API int z2dgpu_fill(z2dgpu_ctx *c, z2d_surface *surface, const z2d_pattern *pattern, const z2d_node *nodes, size_t n_nodes,
                        const z2d_fill_opts *opts) {
    if (!c || !pattern || !opts) return Z2D_ERR_INVALID_ARGUMENT;
    Z2D_CUDA(cudaSetDevice(c->device));
    z2d_fill_cmd cmd;
    cmd.pattern = pattern;
    cmd.node_offset = 0;
    cmd.n_nodes = n_nodes;
    cmd.opts = *opts;
    return do_fill_batch(*c, surface, nodes, n_nodes, &cmd, 1);
}

Z2D_API int z2dgpu_fill_batch(z2dgpu_ctx *c, z2d_surface *surface, const z2d_node *nodes, size_t n_nodes,
                              const z2d_fill_cmd *cmds, size_t n_cmds) {
    if (!c) return Z2D_ERR_INVALID_ARGUMENT;
    Z2D_CUDA(cudaSetDevice(c->device));
    return do_fill_batch(*c, surface, nodes, n_nodes, cmds, n_cmds);
}

Z2D_API int z2dgpu_stroke(z2dgpu_ctx *c, z2d_surface *surface, const z2d_pattern *pattern, const z2d_node *nodes,
                          size_t n_nodes, const z2d_stroke_opts *opts) {
    if (!c || !pattern || !opts) return Z2D_ERR_INVALID_ARGUMENT;
    Z2D_CUDA(cudaSetDevice(c->device));
    return do_stroke(*c, surface, pattern, nodes, n_nodes, *opts);
}

Z2D_API int z2dgpu_stroke_contours(const z2d_node *nodes, size_t n_nodes, const z2d_stroke_opts *opts,
                                   int32_t surface_format, double *points, size_t cap_points, uint64_t *n_points,
                                   uint64_t *contour_ends, size_t cap_contours, uint64_t *n_contours, double *scale) {
    if (!opts) return Z2D_ERR_INVALID_ARGUMENT;
    stroke::Polygon poly;
    int aa = 0;
    double sc = 1;
    const int rc = stroke_polygon(nodes, n_nodes, *opts, surface_format, aa, poly, sc);
    if (rc) return rc;
    const uint64_t np = poly.points(), nc = poly.ends.size();
    if (points) memcpy(points, poly.xy.data(), sizeof(double) * 2 * std::min<uint64_t>(np, cap_points));
    if (contour_ends) memcpy(contour_ends, poly.ends.data(), sizeof(uint64_t) * std::min<uint64_t>(nc, cap_contours));
    if (n_points) *n_points = np;
    if (n_contours) *n_contours = nc;
    if (scale) *scale = sc;
    return Z2D_OK;
}

static int png_common(z2dgpu_ctx *c, const z2d_surface *surface, int32_t profile, bool file, uint8_t **out,
                      size_t *out_len) {
    if (!c || !out || !out_len) return Z2D_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    *out_len = 0;
    int rc = check_surface(surface);
    if (rc) return rc;
    if (profile != Z2D_PROFILE_NONE && profile != Z2D_PROFILE_LINEAR && profile != Z2D_PROFILE_SRGB) {
        set_error("png: bad color profile");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    Z2D_CUDA(cudaSetDevice(c->device));
    DevSurface ds;
    rc = stage_in(*c, *surface, c->surface, ds);
    if (rc) return rc;
    std::vector<uint8_t> bytes;
    rc = file ? png_file(*c, ds, profile, bytes) : png_scanlines(*c, ds, profile, bytes);
    if (rc) return rc;
    uint8_t *p = static_cast<uint8_t *>(malloc(std::max<size_t>(1, bytes.size())));
    if (!p) return Z2D_ERR_OUT_OF_MEMORY;
    if (!bytes.empty()) memcpy(p, bytes.data(), bytes.size());
    *out = p;
    *out_len = bytes.size();
    return Z2D_OK;
}

Z2D_API int z2dgpu_png_encode(z2dgpu_ctx *c, const z2d_surface *surface, int32_t color_profile, uint8_t **out,
                              size_t *out_len) {
    return png_common(c, surface, color_profile, true, out, out_len);
}

Z2D_API int z2dgpu_png_scanlines(z2dgpu_ctx *c, const z2d_surface *surface, int32_t color_profile, uint8_t **out,
                                 size_t *out_len) {
    return png_common(c, surface, color_profile, false, out, out_len);
}

Z2D_API void z2dgpu_free(void *p) { free(p); }

Z2D_API int z2dgpu_draw_jobs(z2dgpu_ctx *c, const z2d_job *jobs, size_t n_jobs, const z2d_node *nodes, size_t n_nodes,
                             const z2d_draw_cmd *cmds, size_t n_cmds) {
    if (!c) return Z2D_ERR_INVALID_ARGUMENT;
    Z2D_CUDA(cudaSetDevice(c->device));
    return draw_jobs(*c, jobs, n_jobs, nodes, n_nodes, cmds, n_cmds);
}

Z2D_API int z2dgpu_fill_jobs(z2dgpu_ctx *c, const z2d_job *jobs, size_t n_jobs, const z2d_node *nodes, size_t n_nodes,
                             const z2d_fill_cmd *cmds, size_t n_cmds) {
    if (!c) return Z2D_ERR_INVALID_ARGUMENT;
    Z2D_CUDA(cudaSetDevice(c->device));
    return fill_jobs(*c, jobs, n_jobs, nodes, n_nodes, cmds, n_cmds);
}

Z2D_API int z2dgpu_composite(z2dgpu_ctx *c, z2d_surface *dst, int32_t dst_x, int32_t dst_y, int32_t n_ops,
                             const z2d_operation *ops, int32_t precision) {
    if (!c) return Z2D_ERR_INVALID_ARGUMENT;
    int rc = check_surface(dst);
    if (rc) return rc;
    if (n_ops < 0 || n_ops > 2 || (n_ops > 0 && !ops)) {
        set_error("composite: 0..2 operations supported");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (precision != Z2D_PRECISION_INTEGER && precision != Z2D_PRECISION_FLOAT) return Z2D_ERR_INVALID_ARGUMENT;
    Z2D_CUDA(cudaSetDevice(c->device));
    CompJob J;
    bool empty = false;
    rc = composite_region(dst, dst_x, dst_y, n_ops, ops, precision, J, empty);
    if (rc || empty) return rc;
    // stage destination and surface params
    DevBuf *stage[3] = {&c->surface, &c->surface2, &c->surface3};
    int used = 0;
    rc = stage_in(*c, *dst, *stage[used++], J.dst);
    if (rc) return rc;
    std::vector<DevGradient> grads;
    std::vector<DevSrc *> grad_users;
    for (int k = 0; k < n_ops; k++) {
        J.ops[k].op = ops[k].op;
        const z2d_param *prm[2] = {&ops[k].dst, &ops[k].src};
        DevSrc *outs[2] = {&J.ops[k].dst, &J.ops[k].src};
        for (int j = 0; j < 2; j++) {
            const z2d_param &p = *prm[j];
            DevSrc &o = *outs[j];
            memset(&o, 0, sizeof(o));
            if (p.kind == Z2D_PARAM_NONE) {
                o.kind = SRC_NONE;
            } else if (p.kind == Z2D_PARAM_SURFACE) {
                rc = check_surface(p.surface);
                if (rc) return rc;
                if (p.surface->location != dst->location) {
                    set_error("composite: surface params must live where the destination lives");
                    return Z2D_ERR_INVALID_ARGUMENT;
                }
                o.kind = SRC_SURFACE;
                if (p.surface == dst || p.surface->data == dst->data) {
                    o.sfc = J.dst;
                } else {
                    if (used >= 3) {
                        set_error("composite: too many host surfaces");
                        return Z2D_ERR_INVALID_ARGUMENT;
                    }
                    rc = stage_in(*c, *p.surface, *stage[used++], o.sfc);
                    if (rc) return rc;
                }
            } else if (p.kind == Z2D_PARAM_PIXEL || p.kind == Z2D_PARAM_GRADIENT || p.kind == Z2D_PARAM_DITHER) {
                bool needs_grad = false;
                DevGradient g;
                rc = make_dev_src_from_pattern(p.kind, p.pattern, o, needs_grad, g);
                if (rc) return rc;
                if (needs_grad) {
                    grads.push_back(g);
                    grad_users.push_back(&o);
                }
            } else {
                return Z2D_ERR_INVALID_ARGUMENT;
            }
        }
    }
    if (!grads.empty()) {
        const size_t gbytes = (sizeof(DevGradient) * grads.size() + 255) & ~(size_t)255;
        const size_t bytes = gbytes + ext_stops_bytes(grads.data(), grads.size());
        if (c->params.ensure(bytes) || c->staging.ensure(bytes)) return Z2D_ERR_OUT_OF_MEMORY;
        Z2D_CUDA(cudaStreamSynchronize(c->stream));
        memcpy(c->staging.ptr, grads.data(), sizeof(DevGradient) * grads.size());
        put_ext_stops(c->staging.as<DevGradient>(), grads.size(), c->staging.as<uint8_t>() + gbytes,
                      c->params.as<uint8_t>() + gbytes);
        Z2D_CUDA(cudaMemcpyAsync(c->params.ptr, c->staging.ptr, bytes, cudaMemcpyHostToDevice, c->stream));
        for (size_t i = 0; i < grad_users.size(); i++) grad_users[i]->grad = c->params.as<DevGradient>() + i;
    }
    rc = check_param_bounds(J);
    if (rc) return rc;
    rc = launch_composite(*c, J);
    if (rc) return rc;
    return stage_out(*c, *dst, J.dst);
}

Z2D_API int z2dgpu_build_paths(z2dgpu_ctx *c, const z2d_path_program *programs, size_t n_programs,
                               const z2d_path_cmd *cmds, size_t n_cmds, const z2d_glyph_point *glyph_points,
                               size_t n_glyph_points, const uint16_t *glyph_ends, size_t n_glyph_ends,
                               z2d_node *nodes, size_t cap_nodes, uint64_t *offsets, int32_t *status) {
    if (!c) return Z2D_ERR_INVALID_ARGUMENT;
    Z2D_CUDA(cudaSetDevice(c->device));
    return build_paths(*c, programs, n_programs, cmds, n_cmds, glyph_points, n_glyph_points, glyph_ends,
                       n_glyph_ends, nodes, cap_nodes, offsets, status);
}

// Gradient offsets of a block of pixels, as the compositor and the
// rasteriser evaluate them; counts the pixels that took the f64 code.
__global__ void k_grad_offsets(const DevGradient *__restrict__ g, int32_t x0, int32_t y0, int32_t w, long long n,
                               float *__restrict__ out, unsigned long long *__restrict__ n_slow) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool slow = false;
    if (i < n) out[i] = grad_offset_ex(*g, x0 + (int32_t)(i % w), y0 + (int32_t)(i / w), slow);
    const unsigned b = __ballot_sync(0xffffffffu, slow);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(n_slow, (unsigned long long)__popc(b));
}

Z2D_API int z2dgpu_gradient_offsets(z2dgpu_ctx *c, const z2d_gradient *g, int32_t x0, int32_t y0, int32_t w, int32_t h,
                                    float *offsets, int64_t *n_f64) {
    if (!c || !g || !offsets || w <= 0 || h <= 0 || (long long)w * h > (1ll << 28)) return Z2D_ERR_INVALID_ARGUMENT;
    Z2D_CUDA(cudaSetDevice(c->device));
    DevGradient dg;
    const int rc = make_dev_gradient(*g, dg);
    if (rc) return rc;
    const long long n = (long long)w * h;
    const size_t o_out = 1024, o_cnt = o_out + ((sizeof(float) * (size_t)n + 255) & ~(size_t)255);
    if (c->params.ensure(o_cnt + 256) || c->staging.ensure(sizeof(DevGradient) + 16)) return Z2D_ERR_OUT_OF_MEMORY;
    static_assert(sizeof(DevGradient) <= 1024, "descriptor fits before the offsets");
    Z2D_CUDA(cudaStreamSynchronize(c->stream));
    memcpy(c->staging.ptr, &dg, sizeof(DevGradient));
    uint8_t *dv = c->params.as<uint8_t>();
    Z2D_CUDA(cudaMemcpyAsync(dv, c->staging.ptr, sizeof(DevGradient), cudaMemcpyHostToDevice, c->stream));
    Z2D_CUDA(cudaMemsetAsync(dv + o_cnt, 0, sizeof(unsigned long long), c->stream));
    k_grad_offsets<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(
        reinterpret_cast<const DevGradient *>(dv), x0, y0, w, n, reinterpret_cast<float *>(dv + o_out),
        reinterpret_cast<unsigned long long *>(dv + o_cnt));
    c->launches++;
    Z2D_CUDA(cudaGetLastError());
    unsigned long long slow = 0;
    Z2D_CUDA(cudaMemcpyAsync(offsets, dv + o_out, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    Z2D_CUDA(cudaMemcpyAsync(&slow, dv + o_cnt, sizeof(slow), cudaMemcpyDeviceToHost, c->stream));
    Z2D_CUDA(cudaStreamSynchronize(c->stream));
    if (n_f64) *n_f64 = (int64_t)slow;
    return Z2D_OK;
}

// SurfaceCompositor.run for callers that are not allowed to allocate device
// memory: the operations' gradient descriptors go to the file-scope
// g_noalloc_gradients instead of context scratch, and no context (with its
// own allocations) is involved.  The first call on a device looks up the
// scratch's device address; that call should come before any stream
// capture.  The address is kept for the life of the process, so the entry
// point must not be used on a device after cudaDeviceReset there.  Calls
// share the scratch: calls that overlap on the GPU race.  A call with
// gradient params is rejected while `stream` is capturing.
Z2D_API int z2dgpu_composite_noalloc(int device, void *stream, z2d_surface *dst, int32_t dst_x, int32_t dst_y,
                                     int32_t n_ops, const z2d_operation *ops, int32_t precision) {
    int rc = check_surface(dst);
    if (rc) return rc;
    if (dst->location != Z2D_MEM_DEVICE) {
        set_error("composite_noalloc: surfaces must be in device memory (host surfaces need staging buffers)");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (n_ops < 0 || n_ops > 2 || (n_ops > 0 && !ops)) {
        set_error("composite_noalloc: 0..2 operations supported");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (precision != Z2D_PRECISION_INTEGER && precision != Z2D_PRECISION_FLOAT) return Z2D_ERR_INVALID_ARGUMENT;
    if (device < 0 || device >= kMaxDevices) {
        set_errorf("composite_noalloc: device index must be in [0, %d)", kMaxDevices);
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    int prev = -1;
    Z2D_CUDA(cudaGetDevice(&prev));
    if (prev != device) Z2D_CUDA(cudaSetDevice(device));
    struct Restore {
        int prev, dev;
        ~Restore() {
            if (prev != dev) cudaSetDevice(prev);
        }
    } restore{prev, device};

    DevGradient *scratch = nullptr;
    rc = noalloc_scratch(device, &scratch);
    if (rc) return rc;
    CompJob J;
    bool empty = false;
    rc = composite_region(dst, dst_x, dst_y, n_ops, ops, precision, J, empty);
    if (rc || empty) return rc;
    J.dst = DevSurface{reinterpret_cast<uint8_t *>(dst->data), dst->format, dst->width, dst->height};
    DevGradient grads[kNoAllocGradients];
    int n_grads = 0;
    for (int k = 0; k < n_ops; k++) {
        J.ops[k].op = ops[k].op;
        const z2d_param *prm[2] = {&ops[k].dst, &ops[k].src};
        DevSrc *outs[2] = {&J.ops[k].dst, &J.ops[k].src};
        for (int j = 0; j < 2; j++) {
            const z2d_param &p = *prm[j];
            DevSrc &o = *outs[j];
            memset(&o, 0, sizeof(o));
            if (p.kind == Z2D_PARAM_NONE) {
                o.kind = SRC_NONE;
            } else if (p.kind == Z2D_PARAM_SURFACE) {
                rc = check_surface(p.surface);
                if (rc) return rc;
                if (p.surface->location != Z2D_MEM_DEVICE) {
                    set_error("composite_noalloc: surface params must be in device memory");
                    return Z2D_ERR_INVALID_ARGUMENT;
                }
                o.kind = SRC_SURFACE;
                o.sfc = DevSurface{reinterpret_cast<uint8_t *>(p.surface->data), p.surface->format, p.surface->width,
                                   p.surface->height};
            } else if (p.kind == Z2D_PARAM_PIXEL || p.kind == Z2D_PARAM_GRADIENT || p.kind == Z2D_PARAM_DITHER) {
                bool needs_grad = false;
                DevGradient g;
                rc = make_dev_src_from_pattern(p.kind, p.pattern, o, needs_grad, g);
                if (rc) return rc;
                if (needs_grad && g.n_stops > kMaxStops) {
                    set_errorf("composite_noalloc: at most %d stops per gradient", kMaxStops);
                    return Z2D_ERR_INVALID_ARGUMENT;
                }
                if (needs_grad) {
                    if (n_grads == kNoAllocGradients) {
                        set_errorf("composite_noalloc: at most %d gradient parameters per call", kNoAllocGradients);
                        return Z2D_ERR_INVALID_ARGUMENT;
                    }
                    grads[n_grads] = g;
                    o.grad = scratch + n_grads;
                    n_grads++;
                }
            } else {
                return Z2D_ERR_INVALID_ARGUMENT;
            }
        }
    }
    rc = check_param_bounds(J);
    if (rc) return rc;
    Ctx c;
    c.device = device;
    c.stream = reinterpret_cast<cudaStream_t>(stream);
    Z2D_CUDA(cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, device));
    // Every descriptor a kernel reads is written here, so nothing in the
    // scratch has to start at zero.  The copy reads `grads` before it returns.
    if (n_grads > 0) {
        // A capturing stream would record a copy node that reads `grads`
        // again at every replay, after this stack frame is gone.
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        Z2D_CUDA(cudaStreamIsCapturing(c.stream, &cap));
        if (cap != cudaStreamCaptureStatusNone) {
            set_error("composite_noalloc: gradient params cannot be used while the stream is capturing "
                      "(their descriptors are copied from memory that does not outlive the call)");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
        Z2D_CUDA(cudaMemcpyAsync(scratch, grads, sizeof(DevGradient) * (size_t)n_grads, cudaMemcpyHostToDevice, c.stream));
    }
    return launch_composite(c, J);
}

}  // extern "C"
