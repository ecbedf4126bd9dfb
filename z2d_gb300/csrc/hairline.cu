// hairline.cu -- painter.stroke's hairline mode on the device
// (src/internal/raster/hairline.zig).
//
// A hairline is a sequence of single-pixel composites: every polyline
// segment is drawn with Bresenham's (no anti-aliasing) or Xiaolin Wu's
// line algorithm, a lone point as one pixel, and z2d applies them one after
// the other, so pixels where segments meet or cross are composited more
// than once, in path order.  On the device:
//   kh_count  32 points per warp: each segment's pixel operations
//   (scan)    their positions in path order (the operation's sequence number)
//   kh_emit   every operation as (surface pixel key, sequence number) and
//             its opacity
//   (sort)    a stable radix sort by pixel key
//   kh_apply  one thread per touched pixel applies its operations in
//             sequence order
// Within one segment all pixels differ, so only operations of different
// segments ever meet on a pixel, and the sort keeps their order.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "raster_px.cuh"
#include "stroke_gpu.cuh"
#include "z2d_internal.h"

namespace z2dg {

namespace {

constexpr uint16_t kOpaque = 256;  // compositeOpaque; 0..255: compositeOpacity

// device view of one pass
struct HairArgs {
    const double2 *pts;
    const long long *start;  // per polyline: first point
    const int32_t *n;        // per polyline: points
    const int32_t *cmd;      // per polyline: its hairline command
    const int32_t *fill;     // per command: the FillCmd (pattern, operator, precision, job)
    const int32_t *aa_none;  // per command: Bresenham (1) or Wu (0)
    const FillCmd *fills;
    const DevJob *jobs;
    int32_t n_lines;
    long long n_points;
};

// hairline.zig deltaStep / errInc
__device__ __forceinline__ void delta_step(int32_t a, int32_t b, int32_t &d, int32_t &s) {
    const int32_t c = b - a;
    d = c < 0 ? -c : c;
    s = c < 0 ? -1 : 1;
}
__device__ __forceinline__ uint16_t err_inc(int32_t a, int32_t b) {
    if (a == b) return 0xFFFFu;
    return (uint16_t)(((uint32_t)a << 16) / (uint32_t)b);
}

// drawLine (hairline.zig:89-124) for the segment (x0, y0) -> (x1, y1) on a
// w x h surface: calls op(x, y, opacity) for every pixel composite in
// order.  Returns the count without calling op when COUNT.
template <bool COUNT, class Op>
__device__ __forceinline__ long long draw_line(int32_t w, int32_t h, bool aa_none, int32_t x0, int32_t y0, int32_t x1,
                                               int32_t y1, Op &&op) {
    // inBox (hairline.zig:396-406)
    if ((x0 < 0 || x0 >= w) && (x1 < 0 || x1 >= w)) return 0;
    if ((y0 < 0 || y0 >= h) && (y1 < 0 || y1 >= h)) return 0;
    const int32_t adx = abs(x1 - x0), ady = abs(y1 - y0);
    if (adx == 0) {  // drawVertical
        const int32_t sy = min(max(min(y0, y1), 0), h - 1), ey = min(max(max(y0, y1), 0), h - 1);
        if (COUNT) return (long long)(ey - sy + 1);
        for (int32_t y = sy; y <= ey; y++) op(x0, y, kOpaque);
        return 0;
    }
    if (ady == 0) {  // drawHorizontal: one compositeOpaque stride
        const int32_t sx = min(max(min(x0, x1), 0), w - 1), ex = min(max(max(x0, x1), 0), w - 1);
        const int32_t len = ex - sx + 1;
        if (len <= 0) return 0;
        if (COUNT) return len;
        for (int32_t x = sx; x <= ex; x++) op(x, y0, kOpaque);
        return 0;
    }
    const bool x_major = !(adx < ady);
    // the major axis runs forward (the reference swaps the endpoints)
    if (x_major ? x0 > x1 : y0 > y1) {
        int32_t t = x0;
        x0 = x1;
        x1 = t;
        t = y0;
        y0 = y1;
        y1 = t;
    }
    if (aa_none) {  // drawBresHorizontal / drawBresVertical
        if (COUNT) return (long long)(x_major ? x1 - x0 : y1 - y0) + 1;
        int32_t md, nd, ns;
        if (x_major) {
            md = x1 - x0;
            delta_step(y0, y1, nd, ns);
        } else {
            md = y1 - y0;
            delta_step(x0, x1, nd, ns);
        }
        int32_t x = x0, y = y0;
        int32_t d = 2 * nd - md;
        const int32_t d_inc = 2 * nd, d_dec = 2 * md;
        for (int32_t k = 0; k <= md; k++) {
            op(x, y, kOpaque);
            if (d > 0) {
                if (x_major) y += ns;
                else x += ns;
                d -= d_dec;
            }
            d += d_inc;
            if (x_major) x++;
            else y++;
        }
        return 0;
    }
    // drawWuHorizontal / drawWuVertical (hairline.zig:242-355)
    int32_t md, nd, ns;
    if (x_major) {
        md = x1 - x0;
        delta_step(y0, y1, nd, ns);
    } else {
        md = y1 - y0;
        delta_step(x0, x1, nd, ns);
    }
    if (COUNT) return 2 * (long long)md;
    const uint16_t inc = err_inc(nd, md);
    uint16_t err = 0;
    int32_t x = x0, y = y0;
    op(x, y, kOpaque);
    if (x_major) x++;
    else y++;
    for (int32_t k = 1; k < md; k++) {
        const uint32_t sum = (uint32_t)err + inc;
        err = (uint16_t)sum;
        if (sum > 0xFFFFu) {  // the error rolled over: step the minor axis
            if (x_major) y += ns;
            else x += ns;
        }
        const uint16_t comp = (uint16_t)(err >> 8);  // opacity complement
        op(x, y, (uint16_t)(comp ^ 0xFFu));
        if (x_major) op(x, y + ns, comp);
        else op(x + ns, y, comp);
        if (x_major) x++;
        else y++;
    }
    op(x1, y1, kOpaque);
    return 0;
}

// The polyline holding each of a warp's 32 consecutive points: the last one
// starting at or before the chunk, then the ends of the <= 32 that follow.
__device__ __forceinline__ int32_t line_of(const HairArgs &A, long long base, long long pt, int lane) {
    const unsigned all = 0xffffffffu;
    int32_t c0 = 0;
    if (lane == 0) {
        int32_t lo = 0, hi = A.n_lines - 1;
        while (lo < hi) {
            const int32_t mid = (lo + hi + 1) >> 1;
            if (A.start[mid] <= base) lo = mid;
            else hi = mid - 1;
        }
        c0 = lo;
    }
    c0 = __shfl_sync(all, c0, 0);
    const int32_t ck = c0 + lane;
    const long long end_k = ck < A.n_lines ? A.start[ck] + A.n[ck] : 0x7FFFFFFFFFFFFFFFll;
    int32_t my = c0;
#pragma unroll 8
    for (int k = 0; k < 32; k++) my += __shfl_sync(all, end_k, k) <= pt ? 1 : 0;
    return my;
}

// The operations point `pt` starts: a lone point's single pixel, or the
// segment to the next point of its polyline (hairline.zig:29-81).
template <bool COUNT, class Op>
__device__ __forceinline__ long long point_ops(const HairArgs &A, int32_t line, long long pt, Op &&op) {
    const long long s0 = A.start[line];
    const int32_t n = A.n[line], c = A.cmd[line];
    const FillCmd &F = A.fills[A.fill[c]];
    const DevSurface &S = A.jobs[F.job].sfc;
    const double2 p = A.pts[pt];
    if (n == 1) {
        if (COUNT) return 1;
        op((int32_t)round(p.x), (int32_t)round(p.y), kOpaque);
        return 0;
    }
    if (pt + 1 == s0 + n) return 0;  // the last point starts no segment
    const double2 q = A.pts[pt + 1];
    return draw_line<COUNT>(S.w, S.h, A.aa_none[c] != 0, (int32_t)round(p.x), (int32_t)round(p.y), (int32_t)round(q.x),
                            (int32_t)round(q.y), op);
}

__global__ void kh_count(HairArgs A, long long *__restrict__ cnt) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long base = ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < A.n_points;
         base += warps * 32) {
        const long long pt = base + lane;
        const int32_t line = line_of(A, base, pt, lane);
        if (pt < A.n_points) cnt[pt] = point_ops<true>(A, line, pt, [](int32_t, int32_t, uint16_t) {});
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[A.n_points] = 0;
}

__global__ void kh_emit(HairArgs A, const long long *__restrict__ off, unsigned long long invalid,
                        unsigned long long *__restrict__ keys, int32_t *__restrict__ seq, uint16_t *__restrict__ opv,
                        int32_t *__restrict__ fop) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long base = ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < A.n_points;
         base += warps * 32) {
        const long long pt = base + lane;
        const int32_t line = line_of(A, base, pt, lane);
        if (pt >= A.n_points) continue;
        const int32_t f = A.fill[A.cmd[line]];
        const int32_t job = A.fills[f].job;
        const DevSurface &S = A.jobs[job].sfc;
        long long k = off[pt];
        const long long k_end = off[pt + 1];
        point_ops<false>(A, line, pt, [&](int32_t x, int32_t y, uint16_t o) {
            if (k >= k_end) return;
            // out-of-range start co-ordinates are no-ops (surface.zig:509-544)
            const bool in = x >= 0 && y >= 0 && x < S.w && y < S.h;
            keys[k] = in ? (((unsigned long long)job << 32) | ((unsigned long long)y * (unsigned)S.w + (unsigned)x))
                         : invalid;
            seq[k] = (int32_t)k;
            opv[k] = o;
            fop[k] = f;
            k++;
        });
    }
}

__global__ void kh_apply(const unsigned long long *__restrict__ keys, const int32_t *__restrict__ seq,
                         const uint16_t *__restrict__ opv, const int32_t *__restrict__ fop, long long n_ops,
                         unsigned long long invalid, const FillCmd *__restrict__ fills,
                         const DevJob *__restrict__ jobs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_ops) return;
    const unsigned long long key = keys[i];
    if (key >= invalid || (i > 0 && keys[i - 1] == key)) return;  // not the first operation on its pixel
    const DevSurface S = jobs[key >> 32].sfc;
    const uint32_t idx = (uint32_t)key;
    const int32_t x = (int32_t)(idx % (uint32_t)S.w), y = (int32_t)(idx / (uint32_t)S.w);
    I16 d = raw_to_i16(load_raw(S, idx), S.fmt);
    for (long long j = i; j < n_ops && keys[j] == key; j++) {
        const int32_t s = seq[j];
        const FillCmd &F = fills[fop[s]];
        const uint16_t o = opv[s];
        d = o == kOpaque ? apply_fill(F, S.fmt, x, y, 1, 1, d) : apply_opacity(F, S.fmt, x, y, o, d);
    }
    store_raw(S, idx, i16_to_raw(d, S.fmt));
}

inline unsigned blocks_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

int run_hairlines(Ctx &c, const std::vector<DevJob> &jobs_in, std::vector<FillCmd> &fills,
                  const std::vector<DevGradient> &grads, const std::vector<int32_t> &grad_of_fill,
                  const HairSet &hs) {
    const size_t n_cmd = hs.lines.size();
    if (n_cmd == 0) return Z2D_OK;
    // packed surfaces of an odd length are drawn on padded copies
    std::vector<DevJob> jobs(jobs_in);
    PackedPads pads;
    {
        const int rc = pads.begin(c, jobs.size(), [&](size_t j) -> DevSurface & { return jobs[j].sfc; });
        if (rc) return rc;
    }
    long long n_pts = 0, n_lines = 0;
    for (size_t k = 0; k < n_cmd; k++) {
        n_pts += (long long)hs.lines[k]->points();
        n_lines += (long long)hs.lines[k]->ends.size();
    }
    if (n_pts == 0) return pads.finish(c);
    if (n_lines > 0x7FFFFFFFll || jobs.size() > 0x7FFFFFFFu) {
        set_error("batch too large");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    for (const DevJob &J : jobs)
        if ((unsigned long long)J.sfc.w * (unsigned long long)J.sfc.h > 0xFFFFFFFFull) {
            set_error("hairline strokes: surfaces of more than 2^32 pixels are not supported");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
    // ---- upload: gradients | fills | jobs | per command | per polyline | points
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t n_fills = fills.size(), n_jobs = jobs.size();
    const size_t o_grads = 0;
    const size_t o_ext = al(o_grads + sizeof(DevGradient) * grads.size());  // stop tables of long gradients
    const size_t o_fills = al(o_ext + ext_stops_bytes(grads.data(), grads.size()));
    const size_t o_jobs = al(o_fills + sizeof(FillCmd) * n_fills);
    const size_t o_cf = al(o_jobs + sizeof(DevJob) * n_jobs);
    const size_t o_ca = al(o_cf + sizeof(int32_t) * n_cmd);
    const size_t o_ls = al(o_ca + sizeof(int32_t) * n_cmd);
    const size_t o_ln = al(o_ls + sizeof(long long) * (size_t)n_lines);
    const size_t o_lc = al(o_ln + sizeof(int32_t) * (size_t)n_lines);
    const size_t o_pt = al(o_lc + sizeof(int32_t) * (size_t)n_lines);
    const size_t total = al(o_pt + sizeof(double) * 2 * (size_t)n_pts);
    if (c.params.ensure(total) || c.staging.ensure(total)) return Z2D_ERR_OUT_OF_MEMORY;
    uint8_t *h = c.staging.as<uint8_t>();
    uint8_t *dv = c.params.as<uint8_t>();
    const DevGradient *dgrads = reinterpret_cast<const DevGradient *>(dv + o_grads);
    for (size_t i = 0; i < n_fills; i++)
        if (grad_of_fill[i] >= 0) fills[i].src.grad = dgrads + grad_of_fill[i];
    Z2D_CUDA(cudaStreamSynchronize(c.stream));  // the staging buffer is free again
    if (!grads.empty()) {
        memcpy(h + o_grads, grads.data(), sizeof(DevGradient) * grads.size());
        put_ext_stops(reinterpret_cast<DevGradient *>(h + o_grads), grads.size(), h + o_ext, dv + o_ext);
    }
    memcpy(h + o_fills, fills.data(), sizeof(FillCmd) * n_fills);
    memcpy(h + o_jobs, jobs.data(), sizeof(DevJob) * n_jobs);
    memcpy(h + o_cf, hs.fill.data(), sizeof(int32_t) * n_cmd);
    memcpy(h + o_ca, hs.aa_none.data(), sizeof(int32_t) * n_cmd);
    {
        long long *ls = reinterpret_cast<long long *>(h + o_ls);
        int32_t *ln = reinterpret_cast<int32_t *>(h + o_ln), *lc = reinterpret_cast<int32_t *>(h + o_lc);
        double *hp = reinterpret_cast<double *>(h + o_pt);
        long long pt = 0, li = 0;
        for (size_t k = 0; k < n_cmd; k++) {
            const stroke::Polygon &P = *hs.lines[k];
            uint64_t prev = 0;
            for (uint64_t e : P.ends) {
                ls[li] = pt + (long long)prev;
                ln[li] = (int32_t)(e - prev);
                lc[li] = (int32_t)k;
                prev = e;
                li++;
            }
            if (!P.xy.empty()) memcpy(hp + 2 * pt, P.xy.data(), sizeof(double) * P.xy.size());
            pt += (long long)P.points();
        }
    }
    Z2D_CUDA(cudaMemcpyAsync(dv, h, total, cudaMemcpyHostToDevice, c.stream));
    HairArgs A;
    A.pts = reinterpret_cast<const double2 *>(dv + o_pt);
    A.start = reinterpret_cast<const long long *>(dv + o_ls);
    A.n = reinterpret_cast<const int32_t *>(dv + o_ln);
    A.cmd = reinterpret_cast<const int32_t *>(dv + o_lc);
    A.fill = reinterpret_cast<const int32_t *>(dv + o_cf);
    A.aa_none = reinterpret_cast<const int32_t *>(dv + o_ca);
    A.fills = reinterpret_cast<const FillCmd *>(dv + o_fills);
    A.jobs = reinterpret_cast<const DevJob *>(dv + o_jobs);
    A.n_lines = (int32_t)n_lines;
    A.n_points = n_pts;

    // ---- count, scan
    if (c.stroke_a.ensure(2 * sizeof(long long) * (size_t)(n_pts + 1) + 256)) return Z2D_ERR_OUT_OF_MEMORY;
    long long *cnt = c.stroke_a.as<long long>();
    long long *off = cnt + (n_pts + 1);
    constexpr int T = 128;
    const unsigned pt_blocks =
        (unsigned)std::min<long long>(blocks_for((n_pts + 31) / 32, T / 32), (long long)c.sm_count * 32);
    cudaEvent_t ts = c.timer_begin(c.t_stroke);
    kh_count<<<pt_blocks, T, 0, c.stream>>>(A, cnt);
    size_t tmp = 0;
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, cnt, off, n_pts + 1, c.stream));
    if (c.scan_tmp.ensure(tmp + 16)) return Z2D_ERR_OUT_OF_MEMORY;
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(c.scan_tmp.ptr, tmp, cnt, off, n_pts + 1, c.stream));
    c.timer_end(c.t_stroke, ts);
    if (c.readback.ensure(64)) return Z2D_ERR_OUT_OF_MEMORY;
    long long *rb = c.readback.as<long long>();
    Z2D_CUDA(cudaMemcpyAsync(rb, off + n_pts, sizeof(long long), cudaMemcpyDeviceToHost, c.stream));
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    const long long n_ops = rb[0];
    c.launches += 3;
    if (n_ops <= 0) return pads.finish(c);
    if (n_ops > 0x7FFFFFFFll) {
        set_error("batch too large: more than 2^31 hairline pixels");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    // ---- emit, sort, apply
    size_t o_k = 0, o_k2, o_s, o_s2, o_o, o_f, o_end;
    o_k2 = al(o_k + sizeof(unsigned long long) * (size_t)n_ops);
    o_s = al(o_k2 + sizeof(unsigned long long) * (size_t)n_ops);
    o_s2 = al(o_s + sizeof(int32_t) * (size_t)n_ops);
    o_o = al(o_s2 + sizeof(int32_t) * (size_t)n_ops);
    o_f = al(o_o + sizeof(uint16_t) * (size_t)n_ops);
    o_end = al(o_f + sizeof(int32_t) * (size_t)n_ops);
    if (c.stroke_b.ensure(o_end)) return Z2D_ERR_OUT_OF_MEMORY;
    uint8_t *B = c.stroke_b.as<uint8_t>();
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(B + o_k);
    unsigned long long *keys2 = reinterpret_cast<unsigned long long *>(B + o_k2);
    int32_t *seq = reinterpret_cast<int32_t *>(B + o_s), *seq2 = reinterpret_cast<int32_t *>(B + o_s2);
    uint16_t *opv = reinterpret_cast<uint16_t *>(B + o_o);
    int32_t *fop = reinterpret_cast<int32_t *>(B + o_f);
    const unsigned long long invalid = (unsigned long long)n_jobs << 32;
    int end_bit = 32;
    while (end_bit < 64 && ((invalid >> end_bit) != 0)) end_bit++;
    ts = c.timer_begin(c.t_stroke);
    kh_emit<<<pt_blocks, T, 0, c.stream>>>(A, off, invalid, keys, seq, opv, fop);
    size_t stmp = 0;
    Z2D_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, stmp, keys, keys2, seq, seq2, (int)n_ops, 0, end_bit, c.stream));
    if (c.scan_tmp.ensure(stmp + 16)) return Z2D_ERR_OUT_OF_MEMORY;
    Z2D_CUDA(cub::DeviceRadixSort::SortPairs(c.scan_tmp.ptr, stmp, keys, keys2, seq, seq2, (int)n_ops, 0, end_bit,
                                             c.stream));
    kh_apply<<<blocks_for(n_ops, T), T, 0, c.stream>>>(keys2, seq2, opv, fop, n_ops, invalid, A.fills, A.jobs);
    c.timer_end(c.t_stroke, ts);
    c.launches += 3;
    return pads.finish(c);
}

}  // namespace z2dg
