// fill.cu -- painter.fill on the GPU, for one fill or an ordered batch of
// fills on one surface.
//
// Pipeline (one launch each, all on the context stream):
//   k_node_count_w  32 nodes per warp: how many edges each line/curve
//                 emits (Bezier subdivision of Spline.zig:37-165; curves
//                 subdivided by the whole warp)
//   stroke_count  device-stroked commands (stroke_gpu.cu): their polygons'
//                 edge counts
//   k_fill_scan   warp per fill: the sequential part of fill_plotter.plot
//                 (fill_plotter.zig:21-97) -- start points, close_path edges,
//                 per-node edge offsets, open-chain detection
//   k_node_emit_w 32 nodes per warp: emits Polygon edges (Polygon.zig:61-109)
//                 and per-fill extents; stroke_emit does the same for the
//                 stroke polygons
//   k_fill_setup  thread per fill: Polygon.inBox and the draw box of
//                 multisample.run / direct.run
//   k_bin_count / k_bin_fill   (edge, 4-row band) lists per fill
//   k_band_lists  CTA per band: the fills touching the band, in call order
//   k_exact       thread per degenerate fill: literal restatement of the
//                 sorted-span rasteriser, writing a per-pixel action mask
//   k_raster      CTA per 4x256 tile: for each fill in order, winding deltas
//                 per sub-scanline in shared memory, a warp prefix scan per
//                 sub-scanline, coverage, then z2d's span compositing rules
//                 (raster/shared.zig) applied to the tile held in registers.
//
// Why the winding scan equals z2d's sorted spans: on every sub-scanline
// z2d sorts the active edges' rounded crossings, keeps the 0<->non-zero
// transitions (non-zero) or all of them (even-odd) and fills [x_{2k},
// x_{2k+1}).  A sample column c is then covered exactly when the crossings
// at x <= c have non-zero (odd) winding, provided the row's crossings are
// balanced.  Closed subpaths always give balanced rows; fills with an open
// 2-point subpath are routed to k_exact.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "fill.cuh"
#include "host_pool.h"
#include "edges.cuh"
#include "spline.cuh"
#include "raster_px.cuh"
#include "stroke_gpu.cuh"

namespace z2dg {

// ------------------------------------------------------------ kernels
// The sequential walk of fill_plotter.plot over one fill's nodes, one warp
// per fill: the warp stages 32 nodes at a time in shared memory, lane 0
// walks them, and the warp writes their NodeInfo back.
constexpr int kScanWarps = 4;
struct ScanStage {
    double x[32], y[32];    // node end point (curve: p[4], p[5])
    double sx[32], sy[32];  // NodeInfo fields the walk sets
    double ex[32], ey[32];
    int32_t tag[32], n_emit[32], n_added[32], off[32];
};

__global__ void __launch_bounds__(32 * kScanWarps) k_fill_scan(const z2d_node *__restrict__ nodes,
                                                               const FillCmd *__restrict__ fills,
                                                               NodeInfo *__restrict__ info, FillState *__restrict__ st,
                                                               int32_t n_fills, int32_t *__restrict__ counters,
                                                               int32_t *__restrict__ status,
                                                               const int32_t *__restrict__ stroke_edges,
                                                               const int32_t *__restrict__ poly_edges) {
    __shared__ ScanStage stages[kScanWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int32_t f = blockIdx.x * kScanWarps + w;
    if (f >= n_fills) return;  // uniform across the warp
    ScanStage &S = stages[w];
    const int32_t node_off = fills[f].node_off, n_nodes = fills[f].n_nodes;
    const double tol = fills[f].tol;
    double fx = 0, fy = 0, lx = 0, ly = 0;
    int32_t count = 0;  // PointBuffer.len, saturating at 3
    int32_t off = 0;
    if (fills[f].stroke >= 0) {  // a device-stroked polygon: its edge count is known
        off = stroke_edges[fills[f].stroke];
        if (off < 0) {
            if (lane == 0) atomicExch(status, Z2D_ERR_INVALID_ARGUMENT);
            off = 0;
        }
    } else if (fills[f].poly >= 0) {  // a host-built polygon: one edge per point
        off = poly_edges[fills[f].poly];
    }
    int32_t flags = 0;
    for (int32_t base = 0; base < n_nodes; base += 32) {
        const int32_t j = base + lane;
        const bool valid = j < n_nodes;
        NodeInfo inf{};
        if (valid) {
            const z2d_node nd = nodes[node_off + j];
            inf = info[node_off + j];
            S.tag[lane] = nd.tag;
            S.x[lane] = nd.tag == Z2D_CURVE_TO ? nd.p[4] : nd.p[0];
            S.y[lane] = nd.tag == Z2D_CURVE_TO ? nd.p[5] : nd.p[1];
            S.n_emit[lane] = inf.n_emit;
            S.n_added[lane] = inf.n_added;
            S.sx[lane] = inf.sx;
            S.sy[lane] = inf.sy;
            S.ex[lane] = inf.ex;
            S.ey[lane] = inf.ey;
        }
        __syncwarp();
        if (lane == 0) {
            const int32_t m = min(32, n_nodes - base);
            for (int32_t k = 0; k < m; k++) {
                S.off[k] = off;
                int32_t ne;
                const double px = S.x[k], py = S.y[k];
                switch (S.tag[k]) {
                    case Z2D_MOVE_TO:
                        ne = 0;
                        if (base + k == n_nodes - 1) break;  // trailing move_to (fill_plotter.zig:38-40)
                        fx = lx = px;
                        fy = ly = py;
                        count = 1;
                        break;
                    case Z2D_LINE_TO:
                        S.sx[k] = lx;
                        S.sy[k] = ly;
                        ne = 1;
                        if (!pt_eq(lx, ly, px, py)) count = min(count + 1, 3);
                        lx = px;
                        ly = py;
                        break;
                    case Z2D_CURVE_TO: {
                        S.sx[k] = lx;
                        S.sy[k] = ly;
                        ne = S.n_emit[k];
                        if (ne < 0) {  // start depends on a preceding close_path
                            int32_t cne = 0, cna = 0;
                            double qx = lx, qy = ly;
                            auto cnt = [&](double x, double y) {
                                cne++;
                                if (!pt_eq(x, y, qx, qy)) cna++;
                                qx = x;
                                qy = y;
                            };
                            if (!spline_walk(lx, ly, nodes[node_off + base + k].p, tol, cnt))
                                atomicExch(status, Z2D_ERR_INVALID_STATE);
                            ne = cne;
                            S.n_added[k] = cna;
                        }
                        count = min(count + S.n_added[k], 3);
                        lx = px;
                        ly = py;
                        break;
                    }
                    default:  // close_path (fill_plotter.zig:72-92)
                        ne = 0;
                        S.sx[k] = lx;
                        S.sy[k] = ly;
                        S.ex[k] = fx;
                        S.ey[k] = fy;
                        if (count >= 3) {
                            if (!pt_eq(lx, ly, fx, fy)) {
                                ne = 1;
                                lx = fx;
                                ly = fy;
                            }
                        } else if (!pt_eq(lx, ly, fx, fy)) {
                            flags |= FILL_OPEN_CHAIN;  // a lone edge stays unmatched
                        }
                        break;
                }
                S.n_emit[k] = ne;
                off += ne;
            }
        }
        __syncwarp();
        if (valid) {
            inf.edge_off = S.off[lane];
            inf.n_emit = S.n_emit[lane];
            inf.n_added = S.n_added[lane];
            inf.sx = S.sx[lane];
            inf.sy = S.sy[lane];
            inf.ex = S.ex[lane];
            inf.ey = S.ey[lane];
            info[node_off + j] = inf;
        }
        __syncwarp();
    }
    if (lane == 0) {
        st[f].n_edges = off;
        st[f].edge_base = atomicAdd(&counters[CNT_EDGES], off);
        st[f].flags = flags;
        st[f].ext[0] = ~0ull;  // min slots start at the largest key
        st[f].ext[1] = 0ull;
        st[f].ext[2] = ~0ull;
        st[f].ext[3] = 0ull;
    }
}


// ------------------------------------------- warp-cooperative flattening
// One warp per curve.  The subdivision tree of Spline.decomposeInto is first
// expanded breadth-first into an ordered frontier of up to kFrontier
// subcurves (z2d's depth-first order is the frontier order), then lane l
// walks frontier items l and l+32 depth-first.  Warp scans give each lane
// the number of points emitted before it and the point emitted just before
// its first one, so edges land where the sequential walk would put them.
constexpr int kFrontier = 64;
constexpr int kFlattenWarps = 4;

struct WarpFrontier {
    Knots k[kFrontier];
    uint8_t leaf[kFrontier];  // 1: error below tolerance already established
};

// Expands the frontier of the curve from (ax, ay) through p[0..5].
__device__ int frontier_expand(double ax, double ay, const double *p, const Tol &tol, WarpFrontier &fr, int lane) {
    if (lane == 0) {
        fr.k[0] = Knots{ax, ay, p[0], p[1], p[2], p[3], p[4], p[5]};
        fr.leaf[0] = 0;
    }
    __syncwarp();
    int n = 1;
    for (int round = 0; round < 8 && n < 32; round++) {
        Knots k{};
        bool leaf = true;
        int grow = 0;
        if (lane < n) {
            k = fr.k[lane];
            leaf = fr.leaf[lane] || below_tol(k, tol);
            grow = leaf ? 1 : 2;
        }
        int incl = grow;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        const bool all_leaf = __all_sync(0xffffffffu, leaf);
        __syncwarp();
        if (all_leaf || total > kFrontier) {
            if (lane < n) fr.leaf[lane] = leaf ? 1 : 0;
            __syncwarp();
            break;
        }
        const int pos = incl - grow;
        if (lane < n) {
            if (leaf) {
                fr.k[pos] = k;
                fr.leaf[pos] = 1;
            } else {
                const Knots second = de_casteljau(k);
                fr.k[pos] = k;
                fr.leaf[pos] = 0;
                fr.k[pos + 1] = second;
                fr.leaf[pos + 1] = 0;
            }
        }
        __syncwarp();
        n = total;
    }
    return n;
}

// Depth-first walk of one frontier item (Spline.zig:56-71): leaf(k) for
// every subcurve that decomposeInto stops at, in order.
template <class L>
__device__ __forceinline__ bool walk_leaves(const Knots &k0, bool is_leaf, const Tol &tol, L &&leaf) {
    if (is_leaf) {
        leaf(k0);
        return true;
    }
    Knots stack[kSplineStack];
    int sp = 0;
    stack[sp++] = k0;
    int32_t budget = kSplineMaxSplits;
    while (sp > 0) {
        Knots k = stack[--sp];
        while (true) {
            if (--budget < 0) return false;
            if (below_tol(k, tol)) {
                leaf(k);
                break;
            }
            const Knots second = de_casteljau(k);
            if (sp >= kSplineStack) return false;
            stack[sp++] = second;
        }
    }
    return true;
}

// emit(x, y) for each leaf start that differs from the curve start: the
// lineTo calls of decomposeInto.  The final lineTo(d) is not part of an item.
template <class F>
__device__ __forceinline__ bool walk_item(const Knots &k0, bool is_leaf, double ax, double ay, const Tol &tol, F &&emit) {
    return walk_leaves(k0, is_leaf, tol, [&](const Knots &k) {
        if (!pt_eq(k.ax, k.ay, ax, ay)) emit(k.ax, k.ay);
    });
}

// "Last valid value before this lane" across the warp, seeded with carry.
__device__ __forceinline__ void prev_point_scan(bool has, double lx, double ly, double cx, double cy, int lane,
                                                double &px, double &py) {
    // inclusive "most recent valid" scan, then shift by one lane
    int v = has ? 1 : 0;
    double x = lx, y = ly;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int tv = __shfl_up_sync(0xffffffffu, v, o);
        const double tx = __shfl_up_sync(0xffffffffu, x, o);
        const double ty = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o && !v) {
            v = tv;
            x = tx;
            y = ty;
        }
    }
    const int pv = __shfl_up_sync(0xffffffffu, v, 1);
    const double qx = __shfl_up_sync(0xffffffffu, x, 1);
    const double qy = __shfl_up_sync(0xffffffffu, y, 1);
    if (lane > 0 && pv) {
        px = qx;
        py = qy;
    } else {
        px = cx;
        py = cy;
    }
}

__device__ __forceinline__ int warp_excl_sum(int v, int lane, int &total) {
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    total = __shfl_sync(0xffffffffu, incl, 31);
    return incl - v;
}

// Counts the lineTo calls (n_emit) and the points they add (n_added) of the
// curve from (sx, sy) through p, cooperatively.  Result valid in all lanes.
// Counts the lineTo calls (n_emit) and the points PointBuffer keeps
// (n_added) of one curve, and the leaves of each frontier item
// (item_leaves[0..kFrontier)).  chords is set when the curve's edges are
// exactly its leaves' chords: every leaf start but the first differs from the
// curve start (consecutive leaves share their end points, so the lineTo
// sequence start, a1, a2, ..., d is the chord sequence), and every item has
// fewer than 65536 leaves.
// Each lane also keeps the start points of the leaves it walks, up to
// kScratch of them, interleaved across the warp in `scr` (scr_n counts
// them, beyond kScratch too); n_items and leaves return the frontier size
// and the curve's leaf count.
constexpr int kScratch = 64;
__device__ bool curve_count_warp(double sx, double sy, const double *p, double tol, WarpFrontier &fr, int lane,
                                 int32_t &n_emit, int32_t &n_added, uint16_t *item_leaves, int32_t &chords,
                                 double2 *scr, int32_t &scr_n, int &n_items, int32_t &leaves_out) {
    chords = 0;
    scr_n = 0;
    n_items = 0;
    leaves_out = 0;
    if (pt_eq(sx, sy, p[0], p[1]) && pt_eq(p[2], p[3], p[4], p[5])) {  // Spline.zig:39-42
        n_emit = 1;
        n_added = pt_eq(sx, sy, p[4], p[5]) ? 0 : 1;
        return true;
    }
    const Tol tol2 = make_tol(tol);
    const int n = frontier_expand(sx, sy, p, tol2, fr, lane);
    n_items = n;
    bool ok = true, small = true;
    int32_t emit_tot = 0, add_tot = 0, leaf_tot = 0;
    double carry_x = sx, carry_y = sy;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        int32_t cnt = 0, internal = 0, leaves = 0;
        double fx = 0, fy = 0, lx = 0, ly = 0;
        if (i < n) {
            ok &= walk_leaves(fr.k[i], fr.leaf[i] != 0, tol2, [&](const Knots &k) {
                leaves++;
                if (scr_n < kScratch) scr[scr_n * 32 + lane] = make_double2(k.ax, k.ay);
                scr_n++;
                if (pt_eq(k.ax, k.ay, sx, sy)) return;  // decomposeInto plots no point equal to the start
                const double x = k.ax, y = k.ay;
                if (cnt == 0) {
                    fx = x;
                    fy = y;
                } else if (!pt_eq(x, y, lx, ly)) {
                    internal++;
                }
                lx = x;
                ly = y;
                cnt++;
            });
            small &= leaves < 65536;
            item_leaves[i] = (uint16_t)leaves;
        }
        int lt = 0;
        warp_excl_sum(leaves, lane, lt);
        leaf_tot += lt;
        double px, py;
        prev_point_scan(cnt > 0, lx, ly, carry_x, carry_y, lane, px, py);
        const int32_t first_add = (cnt > 0 && !pt_eq(fx, fy, px, py)) ? 1 : 0;
        int rt = 0;
        warp_excl_sum(cnt, lane, rt);
        emit_tot += rt;
        int at = 0;
        warp_excl_sum(internal + first_add, lane, at);
        add_tot += at;
        // carry: the last point emitted so far
        const unsigned m = __ballot_sync(0xffffffffu, cnt > 0);
        if (m) {
            const int src = 31 - __clz(m);
            carry_x = __shfl_sync(0xffffffffu, lx, src);
            carry_y = __shfl_sync(0xffffffffu, ly, src);
        }
    }
    // final lineTo(d)
    chords = (__all_sync(0xffffffffu, small) && leaf_tot == emit_tot + 1) ? 1 : 0;
    leaves_out = leaf_tot;
    emit_tot += 1;
    add_tot += pt_eq(p[4], p[5], carry_x, carry_y) ? 0 : 1;
    n_emit = emit_tot;
    n_added = add_tot;
    return __all_sync(0xffffffffu, ok);
}

// Appends idx to a device list (one atomic per warp); all lanes call it.
__device__ __forceinline__ void queue_push(bool push, int32_t idx, int32_t *list, int32_t *count, int lane) {
    const unsigned all = 0xffffffffu;
    const unsigned m = __ballot_sync(all, push);
    if (!m) return;
    int32_t base = 0;
    if (lane == 0) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(all, base, 0);
    if (push) list[base + __popc(m & ((1u << lane) - 1u))] = idx;
}

// The node kernels take 32 consecutive nodes per warp: every lane handles
// its own line, move and close_path node and queues its curve, if it has
// one; the curve kernels then subdivide one queued curve per warp.
__global__ void __launch_bounds__(32 * kFlattenWarps) k_node_count_w(const z2d_node *__restrict__ nodes,
                                                                     const int32_t *__restrict__ node_fill,
                                                                     const FillCmd *__restrict__ fills,
                                                                     NodeInfo *__restrict__ info, int32_t n_nodes,
                                                                     int32_t *__restrict__ curves,
                                                                     int32_t *__restrict__ counters) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int32_t base = (blockIdx.x * kFlattenWarps + w) * 32; base < n_nodes;
         base += gridDim.x * kFlattenWarps * 32) {
        const int32_t i = base + lane;
        NodeInfo inf{};
        bool curve = false;
        if (i < n_nodes) {
            const int32_t f = node_fill[i];
            if (f >= 0) {  // else no fill owns the node
                const z2d_node nd = nodes[i];
                const bool first_of_fill = (i == fills[f].node_off);
                if (nd.tag == Z2D_LINE_TO || nd.tag == Z2D_CURVE_TO) {
                    const z2d_node pv = first_of_fill ? nd : nodes[i - 1];
                    const bool static_start = !first_of_fill && (pv.tag == Z2D_MOVE_TO || pv.tag == Z2D_LINE_TO ||
                                                                 pv.tag == Z2D_CURVE_TO);
                    if (!static_start) {
                        inf.n_emit = -1;  // resolved by k_fill_scan
                    } else if (nd.tag == Z2D_LINE_TO) {
                        const double sx = pv.tag == Z2D_CURVE_TO ? pv.p[4] : pv.p[0];
                        const double sy = pv.tag == Z2D_CURVE_TO ? pv.p[5] : pv.p[1];
                        inf.n_emit = 1;
                        inf.n_added = pt_eq(sx, sy, nd.p[0], nd.p[1]) ? 0 : 1;
                    } else {
                        curve = true;  // k_curve_count_w fills in its info
                    }
                }
            }
        }
        inf.pool = -1;
        if (i < n_nodes && !curve) info[i] = inf;
        queue_push(curve, i, curves, counters + CNT_CURVES, lane);
    }
}

// Besides the counts, a chord curve whose leaves all fit the lanes' scratch
// leaves its polyline (leaf starts, then d) in the curve pool, so that the
// emit pass copies points instead of subdividing the curve again.
__global__ void __launch_bounds__(32 * kFlattenWarps) k_curve_count_w(const z2d_node *__restrict__ nodes,
                                                                      const int32_t *__restrict__ node_fill,
                                                                      const FillCmd *__restrict__ fills,
                                                                      NodeInfo *__restrict__ info,
                                                                      const int32_t *__restrict__ curves,
                                                                      int32_t *__restrict__ counters,
                                                                      uint16_t *__restrict__ item_leaves,
                                                                      int32_t *__restrict__ status,
                                                                      double2 *__restrict__ scratch,
                                                                      double2 *__restrict__ pool, int32_t pool_cap) {
    __shared__ WarpFrontier frs[kFlattenWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned all = 0xffffffffu;
    WarpFrontier &fr = frs[w];
    double2 *scr = scratch + (size_t)(blockIdx.x * kFlattenWarps + w) * (32 * kScratch);
    const int32_t n = counters[CNT_CURVES];
    for (int32_t q = blockIdx.x * kFlattenWarps + w; q < n; q += gridDim.x * kFlattenWarps) {
        const int32_t i = curves[q];
        const z2d_node nd = nodes[i];
        const z2d_node pv = nodes[i - 1];
        const double sx = pv.tag == Z2D_CURVE_TO ? pv.p[4] : pv.p[0];
        const double sy = pv.tag == Z2D_CURVE_TO ? pv.p[5] : pv.p[1];
        NodeInfo inf{};
        int32_t scr_n = 0, leaves = 0;
        int n_items = 0;
        uint16_t *il = item_leaves + (size_t)i * kFrontier;
        const bool ok = curve_count_warp(sx, sy, nd.p, fills[node_fill[i]].tol, fr, lane, inf.n_emit, inf.n_added, il,
                                         inf.chords, scr, scr_n, n_items, leaves);
        if (!ok && lane == 0) atomicExch(status, Z2D_ERR_INVALID_STATE);
        inf.pool = -1;
        if (ok && inf.chords && __all_sync(all, scr_n <= kScratch)) {
            int32_t base = -1;
            if (lane == 0) {
                const unsigned long long b = atomicAdd(reinterpret_cast<unsigned long long *>(&counters[CNT_POOL]),
                                                       (unsigned long long)(leaves + 1));
                base = (b + (unsigned long long)(leaves + 1) <= (unsigned long long)pool_cap) ? (int32_t)b : -1;
            }
            base = __shfl_sync(all, base, 0);
            if (base >= 0) {
                __syncwarp();  // item_leaves of the other lanes are visible
                int32_t off = 0, src = 0;
                for (int b0 = 0; b0 < n_items; b0 += 32) {
                    const int i2 = b0 + lane;
                    const int32_t cnt = i2 < n_items ? (int32_t)il[i2] : 0;
                    int tot = 0;
                    const int32_t at = off + warp_excl_sum(cnt, lane, tot);
                    for (int32_t j = 0; j < cnt; j++) pool[base + at + j] = scr[(src + j) * 32 + lane];
                    src += cnt;
                    off += tot;
                }
                if (lane == 0) pool[base + leaves] = make_double2(nd.p[4], nd.p[5]);
                inf.pool = base;
            }
        }
        if (lane == 0) info[i] = inf;
        __syncwarp();
    }
}

// Emits the edges of one curve with the whole warp.
__device__ __forceinline__ void curve_emit_warp(const FillCmd &F, DEdge *out, const NodeInfo &inf, const double *p,
                                                const uint16_t *il, WarpFrontier &fr, int lane, double &et, double &eb,
                                                double &el, double &er, bool &any) {
    const Tol tol2 = make_tol(F.tol);
    const int n = frontier_expand(inf.sx, inf.sy, p, tol2, fr, lane);
    if (inf.chords) {
        // One walk: the edges are the leaves' chords (a -> d), and the
        // count pass left each frontier item's leaf count.
        int32_t base_off = 0;
        for (int base = 0; base < n; base += 32) {
            const int i2 = base + lane;
            const int32_t cnt = i2 < n ? (int32_t)il[i2] : 0;
            int tot = 0;
            const int off = base_off + warp_excl_sum(cnt, lane, tot);
            if (i2 < n && cnt > 0) {
                int32_t k = off;
                walk_leaves(fr.k[i2], fr.leaf[i2] != 0, tol2, [&](const Knots &kn) {
                    if (k < inf.n_emit) add_edge(F, out + k, kn.ax, kn.ay, kn.dx, kn.dy, et, eb, el, er, any);
                    k++;
                });
            }
            base_off += tot;
        }
        return;
    }
    int32_t base_off = 0;
    double carry_x = inf.sx, carry_y = inf.sy;
    for (int base = 0; base < n; base += 32) {
        const int i2 = base + lane;
        int32_t cnt = 0;
        double lx = 0, ly = 0;
        if (i2 < n)
            walk_item(fr.k[i2], fr.leaf[i2] != 0, inf.sx, inf.sy, tol2, [&](double x, double y) {
                cnt++;
                lx = x;
                ly = y;
            });
        double px, py;
        prev_point_scan(cnt > 0, lx, ly, carry_x, carry_y, lane, px, py);
        int tot = 0;
        const int off = base_off + warp_excl_sum(cnt, lane, tot);
        if (i2 < n && cnt > 0) {
            int32_t k = off;
            walk_item(fr.k[i2], fr.leaf[i2] != 0, inf.sx, inf.sy, tol2, [&](double x, double y) {
                if (k < inf.n_emit) add_edge(F, out + k, px, py, x, y, et, eb, el, er, any);
                k++;
                px = x;
                py = y;
            });
        }
        const unsigned m = __ballot_sync(0xffffffffu, cnt > 0);
        if (m) {
            const int src = 31 - __clz(m);
            carry_x = __shfl_sync(0xffffffffu, lx, src);
            carry_y = __shfl_sync(0xffffffffu, ly, src);
        }
        base_off += tot;
    }
    if (lane == 0 && base_off < inf.n_emit)  // final lineTo(d)
        add_edge(F, out + base_off, carry_x, carry_y, p[4], p[5], et, eb, el, er, any);
}

__global__ void __launch_bounds__(32 * kFlattenWarps) k_node_emit_w(const z2d_node *__restrict__ nodes,
                                                                    const int32_t *__restrict__ node_fill,
                                                                    const FillCmd *__restrict__ fills,
                                                                    const NodeInfo *__restrict__ info,
                                                                    FillState *__restrict__ st, DEdge *__restrict__ edges,
                                                                    int32_t n_nodes, int32_t *__restrict__ curves,
                                                                    int32_t *__restrict__ counters) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int32_t base = (blockIdx.x * kFlattenWarps + w) * 32; base < n_nodes;
         base += gridDim.x * kFlattenWarps * 32) {
        const int32_t i = base + lane;
        int32_t f = -1;
        bool curve = false;
        double et = 0, eb = 0, el = 0, er = 0;
        bool any = false;
        if (i < n_nodes) {
            const NodeInfo inf = info[i];
            if (inf.n_emit > 0) {
                const z2d_node nd = nodes[i];
                f = node_fill[i];
                const FillCmd &F = fills[f];
                DEdge *out = edges + st[f].edge_base + inf.edge_off;
                const bool straight = nd.tag == Z2D_CURVE_TO && pt_eq(inf.sx, inf.sy, nd.p[0], nd.p[1]) &&
                                      pt_eq(nd.p[2], nd.p[3], nd.p[4], nd.p[5]);
                if (nd.tag == Z2D_LINE_TO) add_edge(F, out, inf.sx, inf.sy, nd.p[0], nd.p[1], et, eb, el, er, any);
                else if (nd.tag == Z2D_CLOSE_PATH) add_edge(F, out, inf.sx, inf.sy, inf.ex, inf.ey, et, eb, el, er, any);
                else if (straight) add_edge(F, out, inf.sx, inf.sy, nd.p[4], nd.p[5], et, eb, el, er, any);
                else curve = true;  // k_curve_emit_w emits it
            }
        }
        queue_push(curve, i, curves, counters + CNT_CURVES_EMIT, lane);
        merge_extents(st, f, any, et, eb, el, er);
    }
}

__global__ void __launch_bounds__(32 * kFlattenWarps) k_curve_emit_w(const z2d_node *__restrict__ nodes,
                                                                     const int32_t *__restrict__ node_fill,
                                                                     const FillCmd *__restrict__ fills,
                                                                     const NodeInfo *__restrict__ info,
                                                                     FillState *__restrict__ st,
                                                                     DEdge *__restrict__ edges,
                                                                     const int32_t *__restrict__ curves,
                                                                     const int32_t *__restrict__ counters,
                                                                     const uint16_t *__restrict__ item_leaves,
                                                                     const double2 *__restrict__ pool) {
    __shared__ WarpFrontier frs[kFlattenWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    WarpFrontier &fr = frs[w];
    const int32_t n = counters[CNT_CURVES_EMIT];
    for (int32_t q = blockIdx.x * kFlattenWarps + w; q < n; q += gridDim.x * kFlattenWarps) {
        const int32_t i = curves[q];
        const NodeInfo inf = info[i];
        const int32_t f = node_fill[i];
        const FillCmd &F = fills[f];
        DEdge *out = edges + st[f].edge_base + inf.edge_off;
        double et = 0, eb = 0, el = 0, er = 0;
        bool any = false;
        if (inf.pool >= 0) {  // the count pass kept the polyline: edge k joins points k and k + 1
            const double2 *P = pool + inf.pool;
            for (int32_t k = lane; k < inf.n_emit; k += 32) {
                const double2 a = P[k], b = P[k + 1];
                add_edge(F, out + k, a.x, a.y, b.x, b.y, et, eb, el, er, any);
            }
        } else {
            const z2d_node nd = nodes[i];
            curve_emit_warp(F, out, inf, nd.p, item_leaves + (size_t)i * kFrontier, fr, lane, et, eb, el, er, any);
        }
        merge_extents(st, f, any, et, eb, el, er);
        __syncwarp();
    }
}

__device__ __forceinline__ int32_t clampi(int32_t v, int32_t lo, int32_t hi) { return max(lo, min(v, hi)); }

__global__ void k_fill_setup(const FillCmd *__restrict__ fills, FillState *__restrict__ st, int32_t n_fills,
                             DevJob *__restrict__ jobs, int32_t *__restrict__ counters, RasterFill *__restrict__ rf) {
    const int32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_fills) return;
    const FillCmd F = fills[f];
    DevJob &J = jobs[F.job];
    const int32_t sw = J.sfc.w, sh = J.sfc.h;
    FillState S = st[f];
    S.active = 0;
    if (!S.has_edges) {  // inBox of the empty polygon is false
        st[f] = S;
        return;
    }
    const double et = dkey_inv(S.ext[0]), eb = dkey_inv(S.ext[1]), el = dkey_inv(S.ext[2]), er = dkey_inv(S.ext[3]);
    const double sc = F.scale;
    // Polygon.inBox (Polygon.zig:142-201)
    if (er < 0.0 || eb < 0.0) {
        st[f] = S;
        return;
    }
    const int32_t psx = (int32_t)floor(el / sc), psy = (int32_t)floor(et / sc);
    const int32_t pex = (int32_t)ceil(er / sc), pey = (int32_t)ceil(eb / sc);
    const int32_t pw = pex - psx, ph = pey - psy;
    if (pw == 0 || ph == 0 || psx + pw < 0 || psy + ph < 0 || psx >= sw || psy >= sh) {
        st[f] = S;
        return;
    }
    S.active = 1;
    const bool bounded = is_bounded(F.op);
    if (F.aa == Z2D_AA_NONE) {  // direct.run (direct.zig:36-49)
        const int32_t y0 = bounded ? (int32_t)floor(et) : 0;
        const int32_t y1 = bounded ? (int32_t)ceil(eb) : sh - 1;
        S.start_y = clampi(y0, 0, sh - 1);
        S.end_y = clampi(y1, S.start_y, sh - 1);
        // spans are clamped to the surface, not to the extents; crossings
        // lie within one pixel of the x extents
        S.start_x = clampi((int32_t)floor(el) - 1, 0, sw);
        S.end_x = clampi((int32_t)ceil(er) + 2, S.start_x, sw);
        if (!bounded) S.flags |= FILL_EXACT;
    } else if (F.aa == Z2D_AA_SUPERSAMPLE_4X) {
        // supersample.run (supersample.zig:41-84, 172-184): a 4x mask over
        // [bx0, bx1] x [by0, by1] in sample units, downsampled 4x4 -> 1
        // unless it is narrower or lower than 4 samples, then composited at
        // (max(0, x0), max(0, y0)) and clipped to the surface by
        // SurfaceCompositor.run (compositor.zig:313-374).  Downsampled mask
        // pixel (i, j) averages the samples of surface pixel (cx + i, cy + j).
        const int32_t x0 = bounded ? (int32_t)floor(el / 4.0) : 0;
        const int32_t y0 = bounded ? (int32_t)floor(et / 4.0) : 0;
        const int32_t x1 = bounded ? (int32_t)ceil(er / 4.0) : sw;
        const int32_t y1 = bounded ? (int32_t)ceil(eb / 4.0) : sh;
        const int32_t tw = sw * 4, th = sh * 4;
        const int32_t bx0 = clampi(x0 * 4, 0, tw - 1), by0 = clampi(y0 * 4, 0, th - 1);
        const int32_t bx1 = clampi(x1 * 4, bx0, tw - 1), by1 = clampi(y1 * 4, by0, th - 1);
        const int32_t mw = bx1 + 1 - bx0, mh = by1 + 1 - by0;
        const bool down = mw >= 4 && mh >= 4;
        const int32_t rw = down ? mw / 4 : mw, rh = down ? mh / 4 : mh;
        const int32_t cx = max(0, x0), cy = max(0, y0);
        const int32_t w = (rw + cx > sw) ? sw - cx : rw, h = (rh + cy > sh) ? sh - cy : rh;
        if (w <= 0 || h <= 0) {
            S.active = 0;
            st[f] = S;
            return;
        }
        S.start_x = cx;
        S.end_x = cx + w;
        S.start_y = cy;
        S.end_y = cy + h - 1;
        // Without the downsample, nothing is ever painted into the mask: it
        // is 1 sample wide (or high) only when extent_right (or _bottom) is
        // 0 and the polygon lies left of (or above) the surface.
        if (!down) S.flags |= FILL_SS_ZERO;
    } else {  // multisample.run (multisample.zig:46-78)
        S.start_y = clampi((int32_t)floor(et / 4.0), 0, sh - 1);
        S.end_y = clampi((int32_t)ceil(eb / 4.0), S.start_y, sh - 1);
        S.start_x = clampi((int32_t)floor(el / 4.0), 0, sw - 1);
        S.end_x = clampi((int32_t)ceil(er / 4.0), S.start_x, sw);
    }
    if ((S.flags & FILL_OPEN_CHAIN) && !(S.flags & FILL_SS_ZERO)) S.flags |= FILL_EXACT;
    // rows the fill touches: the draw rows, or every row for unbounded
    // operators (their clears reach outside the draw box); a supersample
    // fill touches exactly its composite region
    const bool boxed = bounded || F.aa == Z2D_AA_SUPERSAMPLE_4X;
    const int32_t ty0 = boxed ? S.start_y : 0;
    const int32_t ty1 = boxed ? S.end_y : sh - 1;
    S.band0 = ty0 / kTileRows;
    S.band1 = ty1 / kTileRows;
    S.fb_base = atomicAdd(&counters[CNT_FILL_BANDS], S.band1 - S.band0 + 1);
    if (S.flags & FILL_EXACT) {
        // action mask over the rows the exact rasteriser visits
        S.mask_w = (F.aa == Z2D_AA_NONE) ? sw : (S.end_x - S.start_x);
        S.mask_x0 = (F.aa == Z2D_AA_NONE) ? 0 : S.start_x;
        // mask, then 8-byte aligned work arrays of 4 ints per edge
        // (permutation, crossings, and 2 breakpoints)
        const long long bytes = ((((long long)S.mask_w * (S.end_y - S.start_y + 1) + 7) & ~7ll) + 16ll * S.n_edges + 15) & ~7ll;
        S.mask_base = atomicAdd(reinterpret_cast<unsigned long long *>(&counters[CNT_MASK_LO]), (unsigned long long)bytes);
        atomicAdd(&counters[CNT_EXACT], 1);
    }
    atomicMin(&J.band_lo, S.band0);
    atomicMax(&J.band_hi, S.band1);
    const int32_t cx0 = boxed ? S.start_x : 0, cx1 = boxed ? S.end_x : sw;
    S.cull_x0 = cx0;
    S.cull_x1 = cx1;
    atomicMin(&J.tcol_lo, cx0 / kTileCols);
    atomicMax(&J.tcol_hi, (max(cx1, cx0 + 1) - 1) / kTileCols);
    st[f] = S;
    RasterFill R;
    R.start_x = S.start_x;
    R.end_x = S.end_x;
    R.start_y = S.start_y;
    R.end_y = S.end_y;
    R.meta = ((uint32_t)F.op & RF_OP_MASK) | ((uint32_t)F.aa << RF_AA_SHIFT) |
             (F.rule == Z2D_FILL_EVEN_ODD ? RF_EVEN_ODD : 0u) | ((uint32_t)F.fast_kind << RF_FAST_SHIFT) |
             ((S.flags & FILL_EXACT) ? RF_EXACT : 0u) | ((S.flags & FILL_SS_ZERO) ? RF_SS_ZERO : 0u) |
             (bounded ? RF_BOUNDED : 0u);
    R.px = (F.src.pix.r & 0xFFu) | ((F.src.pix.g & 0xFFu) << 8) | ((F.src.pix.b & 0xFFu) << 16) |
           ((F.src.pix.a & 0xFFu) << 24);
    R._pad[0] = R._pad[1] = 0;
    rf[f] = R;
}

// Band range of an edge's active sample rows within the fill's draw rows.
__device__ __forceinline__ bool edge_bands(const DEdge &e, const FillCmd &F, const FillState &S, int32_t &b0,
                                           int32_t &b1) {
    if (e.dir == 0) return false;
    const int32_t S_ = (int32_t)F.scale;
    const int32_t lo = max(e.rt, S.start_y * S_), hi = min(e.rb, (S.end_y + 1) * S_);
    if (lo >= hi) return false;
    b0 = lo / (kTileRows * S_);
    b1 = (hi - 1) / (kTileRows * S_);
    return true;
}

// Binning visits every (edge, band) pair.  A long edge spans hundreds of
// bands, so a thread per edge would serialise its atomics; instead each warp
// takes 32 edges and walks their pairs 32 at a time, every lane finding the
// edge of its pair by a binary search over the warp's prefix sums.
template <class Visit>
__device__ __forceinline__ void for_edge_bands(const FillCmd *__restrict__ fills, const FillState *__restrict__ st,
                                               const DEdge *__restrict__ edges, const int32_t *__restrict__ edge_fill,
                                               int32_t n_edges, Visit &&visit) {
    const int lane = threadIdx.x & 31;
    const int32_t stride = gridDim.x * blockDim.x;
    for (int32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n_edges; base += stride) {
        const int32_t i = base + lane;
        int32_t nb = 0, fb0 = 0;
        if (i < n_edges) {
            const int32_t f = edge_fill[i];
            if (f >= 0) {
                const FillState &S = st[f];
                int32_t b0, b1;
                if (S.active && !(S.flags & FILL_EXACT) && edge_bands(edges[i], fills[f], S, b0, b1)) {
                    nb = b1 - b0 + 1;
                    fb0 = S.fb_base + (b0 - S.band0);
                }
            }
        }
        int32_t incl = nb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        const int32_t excl = incl - nb;
        const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
        for (int32_t k0 = 0; k0 < total; k0 += 32) {
            const int32_t k = k0 + lane;
            // the last lane whose first pair is <= k owns pair k
            int owner = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int32_t e = __shfl_sync(0xffffffffu, excl, owner + step);
                if (e <= k) owner += step;
            }
            const int32_t o_excl = __shfl_sync(0xffffffffu, excl, owner);
            const int32_t o_fb0 = __shfl_sync(0xffffffffu, fb0, owner);
            if (k < total) visit(base + owner, o_fb0 + (k - o_excl));
        }
    }
}

__global__ void k_bin_count(const FillCmd *__restrict__ fills, const FillState *__restrict__ st,
                            const DEdge *__restrict__ edges, const int32_t *__restrict__ edge_fill, int32_t n_edges,
                            int32_t *__restrict__ fb_count, int32_t *__restrict__ status) {
    for_edge_bands(fills, st, edges, edge_fill, n_edges, [&](int32_t, int32_t fb) {
        if (atomicAdd(&fb_count[fb], 1) >= kMaxBandEdges) atomicExch(status, Z2D_ERR_INVALID_ARGUMENT);
    });
}

__global__ void k_bin_fill(const FillCmd *__restrict__ fills, const FillState *__restrict__ st,
                           const DEdge *__restrict__ edges, const int32_t *__restrict__ edge_fill, int32_t n_edges,
                           int32_t *__restrict__ fb_cursor, int32_t *__restrict__ bins) {
    for_edge_bands(fills, st, edges, edge_fill, n_edges,
                   [&](int32_t edge, int32_t fb) { bins[atomicAdd(&fb_cursor[fb], 1)] = edge; });
}

// Edge -> fill map (edges of one fill are contiguous).
__global__ void k_edge_fill(const FillState *__restrict__ st, int32_t n_fills, int32_t *__restrict__ edge_fill) {
    const int32_t f = blockIdx.x;
    const FillState S = st[f];
    for (int32_t k = threadIdx.x; k < S.n_edges; k += blockDim.x) edge_fill[S.edge_base + k] = f;
}

// Ordered list of the fills touching each band (call order preserved by a
// block-wide stream compaction).
// The job a global index belongs to: the last job whose base is <= i
// (bases ascending; jobs with nothing to draw repeat the next base).
template <class Base>
__device__ __forceinline__ int32_t job_of(const DevJob *__restrict__ jobs, int32_t n_jobs, long long i, Base base) {
    int32_t lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if (base(jobs[mid]) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One CTA per global band: the job's fills touching the band, in call order
// (ordered compaction), with the tile-column range each one can affect and
// the fill's (fill, band) slot of the band.
__global__ void __launch_bounds__(256) k_band_lists(const FillState *__restrict__ st, const DevJob *__restrict__ jobs,
                                                    int32_t n_jobs, int32_t *__restrict__ band_count,
                                                    int4 *__restrict__ band_fills) {
    const int32_t gb = blockIdx.x;
    const int32_t j = job_of(jobs, n_jobs, gb, [](const DevJob &J) { return (long long)J.gband_base; });
    const DevJob J = jobs[j];
    const int32_t lb = gb - J.gband_base;
    const int32_t b = J.band_lo + lb;
    const int32_t nf = J.fill1 - J.fill0;
    __shared__ int32_t warp_tot[8];
    __shared__ int32_t base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const int32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int4 *out = band_fills + J.list_base + (long long)lb * nf;
    for (int32_t f0 = J.fill0; f0 < J.fill1; f0 += blockDim.x) {
        const int32_t f = f0 + threadIdx.x;
        bool hit = false;
        int4 ent = make_int4(f, 0, 0, 0);
        if (f < J.fill1) {
            const FillState &S = st[f];
            hit = S.active && b >= S.band0 && b <= S.band1;
            ent.y = S.cull_x0;
            ent.z = S.cull_x1;
            ent.w = S.fb_base + (b - S.band0);
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) warp_tot[wid] = __popc(m);
        __syncthreads();
        int32_t before = 0, total = 0;
        for (int w = 0; w < 8; w++) {
            if (w < wid) before += warp_tot[w];
            total += warp_tot[w];
        }
        if (hit) out[base + before + __popc(m & ((1u << lane) - 1u))] = ent;
        __syncthreads();
        if (threadIdx.x == 0) base += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) band_count[gb] = base;
}

}  // namespace z2dg

namespace z2dg {

// ----------------------------------------------------------- exact path
// Literal restatement of multisample.run / direct.run's sorted-span loop
// (multisample.zig:115-188, direct.zig:51-126, Polygon.zig:232-353) for one
// fill, one thread, writing a per-pixel action mask.  Used for fills whose
// rows may be unbalanced (open 2-point subpaths) and for unbounded operators
// without anti-aliasing, where z2d's per-span clears depend on span order.
__device__ void sort_insertion(int32_t *perm, int32_t *xv, int32_t n) {
    // std.sort.insertionContext; stable, so it orders ties like the stable
    // sort the CPU oracle uses beyond 24 active edges
    for (int32_t i = 1; i < n; i++)
        for (int32_t j = i; j > 0 && xv[j] < xv[j - 1]; j--) {
            const int32_t te = perm[j]; perm[j] = perm[j - 1]; perm[j - 1] = te;
            const int32_t tx = xv[j]; xv[j] = xv[j - 1]; xv[j - 1] = tx;
        }
}

__device__ void shell_sort_unique(int32_t *a, int32_t &n) {
    for (int32_t gap = n / 2; gap > 0; gap /= 2)
        for (int32_t i = gap; i < n; i++) {
            const int32_t t = a[i];
            int32_t j = i;
            for (; j >= gap && a[j - gap] > t; j -= gap) a[j] = a[j - gap];
            a[j] = t;
        }
    int32_t m = 0;
    for (int32_t i = 0; i < n; i++)
        if (m == 0 || a[i] != a[m - 1]) a[m++] = a[i];
    n = m;
}

__global__ void k_exact(const FillCmd *__restrict__ fills, const FillState *__restrict__ st, const DEdge *__restrict__ edges,
                        int32_t n_fills, const DevJob *__restrict__ jobs, uint8_t *__restrict__ masks) {
    const int32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_fills) return;
    const FillState S = st[f];
    if (!S.active || !(S.flags & FILL_EXACT)) return;
    const FillCmd F = fills[f];
    const int32_t sw = jobs[F.job].sfc.w;
    const DEdge *E = edges + S.edge_base;
    uint8_t *mask = masks + S.mask_base;  // zeroed by the host
    const int32_t mh = S.end_y - S.start_y + 1;
    // work arrays live after the mask, 8-byte aligned
    int32_t *perm = reinterpret_cast<int32_t *>(masks + S.mask_base + (((long long)S.mask_w * mh + 7) & ~7ll));
    int32_t *xv = perm + S.n_edges;
    int32_t *bp = xv + S.n_edges;
    int32_t n = 0;
    for (int32_t i = 0; i < S.n_edges; i++)
        if (E[i].dir != 0) perm[n++] = i;
    int32_t nbp = 0;
    for (int32_t i = 0; i < n; i++) {
        bp[nbp++] = E[perm[i]].rt;
        bp[nbp++] = E[perm[i]].rb;
    }
    shell_sort_unique(bp, nbp);
    int32_t bpi = -1;
    for (int32_t i = 0; i < nbp; i++)
        if (bp[i] >= S.start_y) {
            bpi = i == 0 ? 0 : i - 1;
            break;
        }
    if (bpi < 0) return;
    const bool direct = F.aa == Z2D_AA_NONE;
    const bool bounded = is_bounded(F.op);
    const int32_t sc = direct ? 1 : 4;
    int32_t n_active = 0;
    const int32_t sxs = S.start_x * 4, dws = (S.end_x - S.start_x) * 4;
    for (int32_t y = S.start_y; y <= S.end_y; y++) {
        uint8_t *mrow = mask + (long long)(y - S.start_y) * S.mask_w;
        for (int32_t off = 0; off < sc; off++) {
            const int32_t ys = y * sc + off;
            if (ys >= bp[bpi]) {  // WorkingEdgeSet.rescan (Polygon.zig:275-300)
                int32_t to = 0;
                for (int32_t from = 0; from < n; from++) {
                    const DEdge &e = E[perm[from]];
                    if (e.rt <= ys && ys < e.rb) {
                        if (from != to) {
                            const int32_t t = perm[to]; perm[to] = perm[from]; perm[from] = t;
                        }
                        to++;
                    }
                }
                n_active = to;
                if (bpi < nbp - 1) bpi++;
            }
            const double ym = (double)ys + 0.5;
            for (int32_t k = 0; k < n_active; k++) {
                const DEdge &e = E[perm[k]];
                xv[k] = (int32_t)round(e.x_start + (e.x_inc * (ym - e.top)));
            }
            sort_insertion(perm, xv, n_active);
            int32_t fl = n_active;
            if (F.rule == Z2D_FILL_NON_ZERO) {  // WorkingEdgeSet.filter
                int32_t wn = 0, to = 0;
                for (int32_t from = 0; from < n_active; from++) {
                    xv[to] = xv[from];
                    if (wn == 0) {
                        wn += E[perm[from]].dir;
                        to++;
                    } else {
                        wn += E[perm[from]].dir;
                        if (wn == 0) to++;
                    }
                }
                fl = to;
            }
            if (direct) {
                if (!bounded && fl == 0) {
                    for (int32_t x = 0; x < sw; x++) mrow[x] = kMaskClear;
                    continue;
                }
                for (int32_t p = 0; p < fl / 2; p++) {
                    const int32_t sx = max(0, xv[2 * p]);
                    if (sx >= sw) break;
                    const int32_t ex = clampi(xv[2 * p + 1], sx, sw);
                    if (!bounded)
                        for (int32_t x = 0; x < sx; x++) mrow[x] = kMaskClear;
                    for (int32_t x = sx; x < ex; x++) mrow[x] = (uint8_t)((mrow[x] & kMaskClear) | 1);
                    if (!bounded)
                        for (int32_t x = ex; x < sw; x++) mrow[x] = kMaskClear;
                }
            } else {
                int32_t x_min = 0;
                for (int32_t p = 0; p < fl / 2; p++) {
                    const int32_t sx = max(x_min, xv[2 * p] - sxs);
                    if (sx >= dws) break;
                    const int32_t ex = clampi(xv[2 * p + 1] - sxs, sx, dws);
                    for (int32_t c = sx; c < ex; c++) mrow[c >> 2] = (uint8_t)(mrow[c >> 2] + 1);
                    x_min = ex;
                }
            }
        }
    }
}

// --------------------------------------------------------- compositing
// The supersample mask value of a pixel whose 4x4 sample block has n covered
// samples, as 8-bit alpha: the mask is alpha8, or the surface's own format
// for alpha4/2/1 surfaces (supersample.zig:69-83), each covered sample is
// opaque, and downsampleBuffer averages the 16 (surface.zig:447-469).
__device__ __forceinline__ uint32_t ss_mask8(int n, int fmt) {
    if (fmt >= Z2D_FORMAT_ALPHA4) return scale_alpha(((uint32_t)n * fmt_max(fmt)) / 16u, fmt_bits(fmt), 8);
    return ((uint32_t)n * 255u) / 16u;
}

// One pixel of the supersample batch [dst_in(dst = pattern, src = mask), op]
// (supersample.zig:171-184) as StrideCompositor.runPrecision evaluates it
// (compositor.zig:540-621): the mask reads as alpha-only lanes.
static __device__ __noinline__ I16 apply_ssaa(const FillCmd &F, int32_t x, int32_t y, uint32_t m8, I16 d) {
    if (F.precision == Z2D_PRECISION_INTEGER) {
        const I16 r = int_op(Z2D_OP_DST_IN, src_i16_fast(F.src, x, y, 0), I16{0, 0, 0, m8});
        return int_op_any(F.op, d, r);
    }
    const F4 r = float_op(Z2D_OP_DST_IN, src_f4_fast(F.src, x, y, 0), decode_raw(I16{0, 0, 0, m8}));
    return encode_raw(float_op_any(F.op, decode_raw(d), r));
}

// multisample.run's clears for unbounded operators (multisample.zig:96-110),
// including its quirks: the rows below the draw box are cleared up to the
// surface WIDTH, and the right-hand clear starts at x = 0.
__device__ __forceinline__ bool msaa_unbounded_clear(const FillState &S, int32_t x, int32_t y, int32_t sw) {
    if (y < S.start_y) return true;
    if (y > S.end_y) return y < sw;
    return (S.start_x > 0 && x < S.start_x) || (S.end_x < sw && x < sw - S.end_x);
}

struct RasterArgs {
    DevJob job0;                // the job of a one-surface batch, by value
    const DevJob *jobs;
    const FillCmd *fills;
    const FillState *st;
    const DEdge *edges;
    const int32_t *bins;
    const int32_t *bin_off;
    const int32_t *band_count;  // per global band
    const int4 *band_fills;     // {fill, cull_x0, cull_x1, (fill, band) slot} per band, in call order
    const RasterFill *rfills;
    const uint8_t *masks;
    int32_t n_jobs;
    unsigned long long *queue;  // work-queue counter, zero at launch
    unsigned long long n_items; // tiles (CTA items) or tiles x rows (warp items)
    const int32_t *order;       // tile order of the queue, or null (tile index order)
    int32_t one_per_tile;       // not persistent: CTA i draws the i-th tile of the queue
};

// Winding deltas of one warp: up to 4 sample rows x 1024 sample columns,
// two biased 16-bit counters per word (bias 0x8000; a fill with at most
// kMaxBandEdges edges in a band can never carry a counter across halves).
constexpr int kWordsPerSubRow = 512;
constexpr int kTouchOff = 4 * kWordsPerSubRow;  // then 4 x 32 words: pairs touched per (sample row, lane)
constexpr int kTotOff = kTouchOff + 4 * 32;     // then 4 x 32 words: winding change per (sample row, lane)
constexpr int kWarpWords = kTotOff + 4 * 32;
constexpr uint32_t kBias2 = 0x80008000u;

// Sample column c of a sub-scanline belongs to lane c / per (per = sample
// columns per lane: 32 with 4x sampling, 8 without); the pair holding it is
// stored at ((c % per) / 2) * 32 + lane, so a warp reading pair k of every
// lane touches 32 consecutive words.

// One work item is one pixel row of a tile of 4 rows x 256 pixels: lane l
// owns the row's pixels [8l, 8l+8).  The warp walks the band's fills in call
// order, accumulates the winding deltas of its row's 4 (or 1) sample rows
// from the fill's band edges, prefix-scans them across the warp, turns the
// inside bits into coverage and composites its 8 pixels, which stay in
// registers from the first fill to the last.  `words` is the warp's own
// shared-memory scratch.  MULTI = false draws a one-surface batch from
// A.job0, whose fields are kernel parameters (warp-uniform values that need
// no registers); MULTI = true finds the tile's job in the job table.
template <bool MULTI>
__device__ __forceinline__ void raster_row(const RasterArgs &A, const int32_t tile, const int warp, const int lane,
                                           uint32_t *words) {
    // tile -> (job, band, tile column): jobs hold consecutive tile ranges
    int32_t jb = 0;
    if constexpr (MULTI) jb = job_of(A.jobs, A.n_jobs, tile, [](const DevJob &J) { return (long long)J.tile_base; });
    const DevJob &JB = MULTI ? A.jobs[jb] : A.job0;
    const int32_t local = tile - JB.tile_base, ncols = JB.tcol_hi - JB.tcol_lo + 1;
    const int32_t lb = local / ncols;
    const int32_t b = JB.band_lo + lb;
    const int32_t cnt = A.band_count[JB.gband_base + lb];
    if (cnt == 0) return;
    const int32_t x0 = (JB.tcol_lo + local % ncols) * kTileCols, y = b * kTileRows + warp;
    const int32_t W = JB.sfc.w, H = JB.sfc.h, fmt = JB.sfc.fmt;
    if (y >= H) return;
    const int4 *list = A.band_fills + JB.list_base + (long long)lb * (JB.fill1 - JB.fill0);
    const int32_t px0 = x0 + lane * 8;  // this lane's first pixel

    for (int i = lane; i < kWarpWords; i += 32) words[i] = i < kTouchOff ? kBias2 : 0u;
    uint32_t raw[8];
    uint32_t touched = 0;
    {
        const DevSurface dst = JB.sfc;
#pragma unroll
        for (int q = 0; q < 8; q++) raw[q] = (px0 + q < W) ? load_raw(dst, (size_t)W * y + px0 + q) : 0u;
    }
    __syncwarp();

    // The band's fill list is read 32 entries at a time, one per lane; the
    // fills that overlap this tile are then walked in order from a ballot.
    for (int32_t k0 = 0; k0 < cnt; k0 += 32) {
        int4 ent = make_int4(0, 0, 0, 0);
        const bool valid = k0 + lane < cnt;
        if (valid) ent = list[k0 + lane];
        uint32_t hits = __ballot_sync(0xffffffffu, valid && ent.z > x0 && ent.y < x0 + kTileCols);
        while (hits) {
            const int src = __ffs(hits) - 1;
            const int32_t f = __shfl_sync(0xffffffffu, ent.x, src);
            const int32_t fb = __shfl_sync(0xffffffffu, ent.w, src);
            hits &= hits - 1;
            const int4 ra = __ldg(reinterpret_cast<const int4 *>(A.rfills + f));
            const int4 rb = __ldg(reinterpret_cast<const int4 *>(A.rfills + f) + 1);
            // the band's edge range, loaded alongside the record rather than
            // after the tests on it (fb is a valid slot either way)
            const int32_t e0 = __ldg(A.bin_off + fb), e1 = __ldg(A.bin_off + fb + 1);
            const int32_t start_x = ra.x, end_x = ra.y, start_y = ra.z, end_y = ra.w;
            const uint32_t meta = (uint32_t)rb.x;
            const int32_t aa = (int32_t)((meta >> RF_AA_SHIFT) & 3u);
            const bool bounded = (meta & RF_BOUNDED) != 0;
            const bool ssaa = aa == Z2D_AA_SUPERSAMPLE_4X;
            const bool boxed = bounded || ssaa;  // touches only [start_x, end_x) x [start_y, end_y]
            if (boxed && (end_x <= x0 || start_x >= x0 + kTileCols)) continue;
            const bool direct = aa == Z2D_AA_NONE;
            const bool exact = (meta & RF_EXACT) != 0;
            const bool in_rows = y >= start_y && y <= end_y;
            if (!in_rows && boxed) continue;
            const int32_t sc = direct ? 1 : 4, per = 8 * sc, lg_per = direct ? 3 : 5;
            // coverage of pixel q (0..16) is byte q / 2 of cov_ev (q even)
            // or cov_od (q odd)
            uint32_t cov_ev = 0, cov_od = 0;
            if (!exact && in_rows && !(meta & RF_SS_ZERO)) {
                const int32_t sub0 = y * sc, col0 = x0 * sc, ncol = kTileCols * sc;
                // sample rows stay below 2^22, where sr + 0.5 is exact in f32
                const bool f32_ok = sub0 < (1 << 22);
                const float fsub = (float)sub0 + 0.5f;
                // one edge per lane; crossings at or left of the tile's
                // first sample column all land on column 0, so they are
                // summed across the warp and added once (instead of one
                // atomic per edge on the same word)
                for (int32_t base = e0; base < e1; base += 32) {
                    const int32_t ei = base + lane;
                    int32_t id = 0, dir = 0, lo = 0, hi = 0;
                    float4 ef = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (ei < e1) {
                        id = A.bins[ei];
                        ef = __ldg(reinterpret_cast<const float4 *>(A.edges + id));
                        const int2 er = __ldg(reinterpret_cast<const int2 *>(&A.edges[id].rt));
                        dir = __float_as_int(ef.w);
                        lo = max(er.x, sub0);
                        hi = min(er.y, sub0 + sc);
                    }
                    for (int r = 0; r < sc; r++) {  // uniform across the warp
                        const int32_t sr = sub0 + r;
                        int32_t left = 0;
                        if (sr >= lo && sr < hi) {
                            int32_t X;
                            if (!(f32_ok && crossing_f32(ef.x, ef.y, ef.z, fsub + (float)r, X))) {
                                const DEdge &e = A.edges[id];
                                X = (int32_t)round(e.x_start + (e.x_inc * (((double)sr + 0.5) - e.top)));
                            }
                            const int32_t c = X - col0;
                            if (c <= 0) {
                                left = dir;
                            } else if (c < ncol) {
                                // per is 8 or 32 and c > 0: shifts and masks
                                const int lane_c = c >> lg_per, pair = (c & (per - 1)) >> 1;
                                const uint32_t inc = (c & 1) ? ((uint32_t)dir << 16) : (uint32_t)dir;
                                atomicAdd(&words[r * kWordsPerSubRow + ((pair << 5) | lane_c)], inc);
                                atomicOr(&words[kTouchOff + r * 32 + lane_c], 1u << pair);
                                atomicAdd(&words[kTotOff + r * 32 + lane_c], (uint32_t)dir);
                            }
                        }
                        // column 0 is the low half of lane 0's pair 0; a net
                        // zero changes no winding and needs no visit
                        const int32_t sum = __reduce_add_sync(0xffffffffu, left);
                        if (lane == 0 && sum != 0) {
                            atomicAdd(&words[r * kWordsPerSubRow], (uint32_t)sum);
                            atomicOr(&words[kTouchOff + r * 32], 1u);
                            atomicAdd(&words[kTotOff + r * 32], (uint32_t)sum);
                        }
                    }
                }
                __syncwarp();
                // no crossing in or left of the tile on any sample row: the
                // winding is 0 across the tile, nothing is covered
                uint32_t any_touch = 0;
#pragma unroll
                for (int s = 0; s < 4; s++)
                    if (s < sc) any_touch |= words[kTouchOff + s * 32 + lane];
                if (!__any_sync(0xffffffffu, any_touch != 0)) {
                    if (bounded) continue;  // zero coverage draws nothing
                    goto composite;         // unbounded operators still clear
                }
                {
                const bool eo = (meta & RF_EVEN_ODD) != 0;
                // each lane's winding change per sample row, then the
                // winding at the lane's first column: the exclusive scans of
                // rows (0, 1) and (2, 3) run packed as lo + 65536 hi (every
                // partial sum is bounded by the band's edge count, at most
                // kMaxBandEdges < 2^15 in magnitude, so the halves stay apart)
                // (the crossings also summed each lane's winding change)
                int32_t tot[4] = {0, 0, 0, 0};
#pragma unroll
                for (int s = 0; s < 4; s++) {
                    if (s >= sc) break;
                    tot[s] = (int32_t)words[kTotOff + s * 32 + lane];
                    words[kTotOff + s * 32 + lane] = 0u;
                }
                const int32_t t01 = tot[0] + tot[1] * 65536, t23 = tot[2] + tot[3] * 65536;
                int32_t i01 = t01, i23 = t23;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int32_t u01 = __shfl_up_sync(0xffffffffu, i01, o);
                    const int32_t u23 = __shfl_up_sync(0xffffffffu, i23, o);
                    if (lane >= o) {
                        i01 += u01;
                        i23 += u23;
                    }
                }
                const int32_t x01 = i01 - t01, x23 = i23 - t23;
                int32_t wrow[4];
                wrow[0] = (int32_t)(int16_t)(x01 & 0xFFFF);
                wrow[1] = (x01 - wrow[0]) >> 16;
                wrow[2] = (int32_t)(int16_t)(x23 & 0xFFFF);
                wrow[3] = (x23 - wrow[2]) >> 16;
#pragma unroll
                for (int s = 0; s < 4; s++) {
                    if (s >= sc) break;
                    uint32_t *row = words + s * kWordsPerSubRow;
                    uint32_t *touch = words + kTouchOff + s * 32 + lane;
                    const uint32_t touched = *touch;  // pairs of this lane that received crossings
                    int32_t wnd = wrow[s];
                    // Between touched pairs the winding is constant, so inside
                    // bits are filled a range at a time.
                    bool in = eo ? ((wnd & 1) != 0) : (wnd != 0);
                    uint32_t bits = 0;
                    int pos = 0;
                    for (uint32_t m = touched; m; m &= m - 1) {
                        const int kk = __ffs(m) - 1, s0 = 2 * kk;
                        const int idx = (kk << 5) | lane;
                        const uint32_t v = row[idx];
                        row[idx] = kBias2;
                        if (in) bits |= ((1u << s0) - 1u) & ~((1u << pos) - 1u);
                        wnd += (int32_t)(v & 0xFFFFu) - 0x8000;
                        in = eo ? ((wnd & 1) != 0) : (wnd != 0);
                        bits |= (uint32_t)in << s0;
                        wnd += (int32_t)(v >> 16) - 0x8000;
                        in = eo ? ((wnd & 1) != 0) : (wnd != 0);
                        bits |= (uint32_t)in << (s0 + 1);
                        pos = s0 + 2;
                    }
                    if (in && pos < 32) bits |= ~((1u << pos) - 1u);
                    *touch = 0u;
                    if (direct) {  // one sample row: bit q is pixel q's sample
#pragma unroll
                        for (int q = 0; q < 8; q += 2) {
                            cov_ev |= ((bits >> q) & 1u) << (4 * q);
                            cov_od |= ((bits >> (q + 1)) & 1u) << (4 * q);
                        }
                    } else {  // nibble q holds pixel q's 4 samples of this row
                        uint32_t n = bits - ((bits >> 1) & 0x55555555u);
                        n = (n & 0x33333333u) + ((n >> 2) & 0x33333333u);
                        cov_ev += n & 0x0F0F0F0Fu;
                        cov_od += (n >> 4) & 0x0F0F0F0Fu;
                    }
                }
                __syncwarp();
                }
            }
        composite:
            if (((meta >> RF_FAST_SHIFT) & 3u) == FAST_PIXEL_SRC_OVER && !exact && bounded) {
                // Pixel source, integer src_over: the compositeOpaque /
                // compositeOpacity paths reduce to src_over(d, pixel) at full
                // coverage and src_over(d, dst_in(pixel, opacity)) otherwise.
                // The supersample batch [dst_in(pixel, mask), src_over] is the
                // same with the downsampled mask value as opacity; at zero
                // coverage both leave the pixel as it is.
                // (A bounded fill outside its rows was skipped above.)
                const uint32_t pw = (uint32_t)rb.y;
                const I16 px{pw & 0xFFu, (pw >> 8) & 0xFFu, (pw >> 16) & 0xFFu, pw >> 24};
                const int full = direct ? 1 : 16;
                const int32_t xlo = start_x, xhi = direct ? W : min(end_x, W);
                if (fmt <= Z2D_FORMAT_RGBA) {
                    // Lane k holds the source word for coverage k: the pixel
                    // at k = full, dst_in(pixel, opacity(k)) below it.
                    I16 s = px;
                    if (lane < full) {
                        const uint32_t op8 = ssaa ? ss_mask8(lane, fmt) : (uint32_t)max(lane * 16 - 1, 0);
                        s = I16{(px.r * op8) / 255u, (px.g * op8) / 255u, (px.b * op8) / 255u, (px.a * op8) / 255u};
                    }
                    const uint32_t lut_w = i16_to_word(s, word_order(fmt));
                    const bool has_alpha = fmt == Z2D_FORMAT_RGBA || fmt == Z2D_FORMAT_ARGB;
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const int c = (int)((((q & 1) ? cov_od : cov_ev) >> (8 * (q >> 1))) & 0xFFu);
                        const uint32_t L = __shfl_sync(0xffffffffu, lut_w, c);
                        const int32_t x = px0 + q;
                        // without a branch: the lanes of a warp mostly agree
                        // on composing, and a select costs less than a split
                        const bool on = c != 0 && x >= xlo && x < xhi;
                        const uint32_t nv = word_src_over(raw[q], L, has_alpha);
                        raw[q] = on ? nv : raw[q];
                        touched |= (uint32_t)on << q;
                    }
                    continue;
                }
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    const int32_t x = px0 + q;
                    const int c = (int)((((q & 1) ? cov_od : cov_ev) >> (8 * (q >> 1))) & 0xFFu);
                    if (c == 0 || x < xlo || x >= xhi) continue;
                    I16 s = px;
                    if (c < full) {
                        const uint32_t op8 = ssaa ? ss_mask8(c, fmt) : (uint32_t)(c * 16 - 1);
                        s = I16{(px.r * op8) / 255u, (px.g * op8) / 255u, (px.b * op8) / 255u, (px.a * op8) / 255u};
                    }
                    raw[q] = i16_to_raw(int_op(Z2D_OP_SRC_OVER, raw_to_i16(raw[q], fmt), s), fmt);
                    touched |= 1u << q;
                }
                continue;
            }
            const FillState &S = A.st[f];
            const FillCmd &F = A.fills[f];
            if (ssaa) {
                // every pixel of the composite region runs the batch
                // [dst_in(pattern, mask), op] (supersample.zig:171-184)
#pragma unroll 1
                for (int q = 0; q < 8; q++) {
                    const int32_t x = px0 + q;
                    if (x >= W || x < S.start_x || x >= S.end_x) continue;
                    int c = (int)((((q & 1) ? cov_od : cov_ev) >> (8 * (q >> 1))) & 0xFFu);
                    if (exact && x >= S.mask_x0 && x < S.mask_x0 + S.mask_w)
                        c = A.masks[S.mask_base + (long long)(y - S.start_y) * S.mask_w + (x - S.mask_x0)] & 0x1F;
                    uint32_t rq = raw[0];
#pragma unroll
                    for (int j = 1; j < 8; j++)
                        if (q == j) rq = raw[j];
                    rq = i16_to_raw(apply_ssaa(F, x, y, ss_mask8(c, fmt), raw_to_i16(rq, fmt)), fmt);
#pragma unroll
                    for (int j = 0; j < 8; j++)
                        if (q == j) raw[j] = rq;
                    touched |= 1u << q;
                }
                continue;
            }
#pragma unroll 1
            for (int q = 0; q < 8; q++) {
                const int32_t x = px0 + q;
                if (x >= W) continue;
                // raw[] is read and written with constant indices only, so it
                // stays in registers
                int c = (int)((((q & 1) ? cov_od : cov_ev) >> (8 * (q >> 1))) & 0xFFu);
                uint32_t rq = raw[0];
#pragma unroll
                for (int j = 1; j < 8; j++)
                    if (q == j) rq = raw[j];
                bool clear = false;
                if (exact && in_rows && x >= S.mask_x0 && x < S.mask_x0 + S.mask_w) {
                    const uint8_t m = A.masks[S.mask_base + (long long)(y - S.start_y) * S.mask_w + (x - S.mask_x0)];
                    c = m & 0x1F;
                    if (direct) clear = (m & kMaskClear) != 0;
                }
                if (!direct && !bounded) clear = msaa_unbounded_clear(S, x, y, W);
                const bool in_box = in_rows && (direct ? true : (x >= S.start_x && x < S.end_x));
                if (!clear && !(in_box && c > 0)) continue;
                I16 d = clear ? normalize(I16{0, 0, 0, 0}, fmt) : raw_to_i16(rq, fmt);
                if (in_box && c > 0) d = apply_fill(F, fmt, x, y, c, direct ? 1 : 16, d);
                rq = i16_to_raw(d, fmt);
#pragma unroll
                for (int j = 0; j < 8; j++)
                    if (q == j) raw[j] = rq;
                touched |= 1u << q;
            }
        }
    }
    // the surface pointer is read again here rather than kept in registers
    // through the fill loop
    DevSurface dst;
    dst.data = MULTI ? *reinterpret_cast<uint8_t *const volatile *>(&A.jobs[jb].sfc.data) : A.job0.sfc.data;
    dst.fmt = fmt;
    dst.w = W;
    dst.h = 0;  // unused by the stores
#pragma unroll
    for (int q = 0; q < 8; q++)
        if ((touched >> q) & 1u) store_raw(dst, (size_t)W * y + px0 + q, raw[q]);
}

// Work estimate of each raster tile for the cost-ordered queue: the number
// of fills in its band's list (every one is visited by the tile's rows).
__global__ void k_tile_cost(const DevJob *__restrict__ jobs, int32_t n_jobs, const int32_t *__restrict__ band_count,
                            int32_t n_tiles, int32_t *__restrict__ cost, int32_t *__restrict__ idx) {
    const int32_t t = (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= n_tiles) return;
    const int32_t j = job_of(jobs, n_jobs, t, [](const DevJob &J) { return (long long)J.tile_base; });
    const DevJob J = jobs[j];
    const int32_t ncols = J.tcol_hi - J.tcol_lo + 1;
    cost[t] = band_count[J.gband_base + (t - J.tile_base) / ncols];
    idx[t] = t;
}

// Persistent rasteriser: a grid of resident CTAs that take items from a
// device work queue (one 64-bit counter) until it is empty; tiles are
// queued job after job, or in the order of A.order when given.
//  * CTA_ITEMS: an item is a whole tile; the CTA's four warps draw its four
//    rows and meet at a barrier before the next tile, so the rows share the
//    band's fill list and edges in the SM's L1.
//  * otherwise an item is one (tile, row) pair, numbered tile * 4 + row,
//    taken by a single warp: a warp that finishes a cheap row takes the
//    next item at once instead of holding its CTA until the slowest warp of
//    the tile is done.
template <bool MULTI, bool CTA_ITEMS>
__global__ void __launch_bounds__(kRasterThreads, 6) k_raster(const RasterArgs A) {
    extern __shared__ uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *words = smem + warp * kWarpWords;
    if constexpr (CTA_ITEMS) {
        if (A.one_per_tile) {  // a grid of one CTA per tile, dispatched in queue order
            const int32_t tile = A.order ? A.order[blockIdx.x] : (int32_t)blockIdx.x;
            raster_row<MULTI>(A, tile, warp, lane, words);
            return;
        }
        __shared__ unsigned long long next_tile;
        for (;;) {
            if (threadIdx.x == 0) next_tile = atomicAdd(A.queue, 1ull);
            __syncthreads();
            const unsigned long long t = next_tile;
            __syncthreads();  // every thread has read it before it is replaced
            if (t >= A.n_items) break;
            const int32_t tile = A.order ? A.order[t] : (int32_t)t;
            raster_row<MULTI>(A, tile, warp, lane, words);
        }
    } else {
        for (;;) {
            unsigned long long item = 0;
            if (lane == 0) item = atomicAdd(A.queue, 1ull);
            item = __shfl_sync(0xffffffffu, item, 0);
            if (item >= A.n_items) break;
            const long long t = (long long)(item / kTileRows);
            const int32_t tile = A.order ? A.order[t] : (int32_t)t;
            __syncwarp();  // the previous item's reads of `words` are done before it is reset
            raster_row<MULTI>(A, tile, (int)(item % kTileRows), lane, words);
        }
    }
}

// The fill owning each node: warp f writes f over fill f's node range (the
// ranges are disjoint; fills drawing stroke polygons own no nodes).
__global__ void k_node_owner(const FillCmd *__restrict__ fills, int32_t n_fills, int32_t *__restrict__ node_fill) {
    const int32_t f = (int32_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (f >= n_fills) return;
    const int32_t o = fills[f].node_off, n = fills[f].n_nodes;
    for (int32_t k = lane; k < n; k += 32) node_fill[o + k] = f;
}

// ----------------------------------------------------------- host side
static inline unsigned grid_for(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// k_raster's shared-memory attributes: per device, set once on each.
static int raster_attributes(Ctx &c) {
    static std::atomic<uint64_t> attr_set{0};
    const uint64_t dev_bit = 1ull << (c.device & 63);
    if (attr_set.load(std::memory_order_relaxed) & dev_bit) return Z2D_OK;
    const size_t smem = sizeof(uint32_t) * kWarpWords * kTileRows;
    for (auto k : {k_raster<false, false>, k_raster<true, false>, k_raster<false, true>, k_raster<true, true>}) {
        Z2D_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        Z2D_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    }
    attr_set.fetch_or(dev_bit, std::memory_order_relaxed);
    return Z2D_OK;
}

int run_jobs(Ctx &c, std::vector<DevJob> &jobs, const z2d_node *nodes, int32_t n_nodes, std::vector<FillCmd> &fills,
             const std::vector<DevGradient> &grads,
             const std::vector<int32_t> &grad_of_fill, const StrokeSet *strokes) {
    if (n_nodes < 0) return Z2D_ERR_INVALID_ARGUMENT;
    const int32_t n_fills = (int32_t)fills.size();
    const int32_t n_jobs = (int32_t)jobs.size();
    if (n_fills == 0 || n_nodes == 0 || n_jobs == 0) return Z2D_OK;
    if (!strokes) {  // few short fills: one upload, one launch
        bool done = false;
        const int rc = run_small_jobs(c, jobs, nodes, fills, grads, grad_of_fill, done);
        if (rc || done) return rc;
    }
    for (DevJob &J : jobs) {
        J.band_lo = J.tcol_lo = 0x7FFFFFFF;
        J.band_hi = J.tcol_hi = -1;
        J.gband_base = J.tile_base = 0;
        J.list_base = 0;
    }
    // packed surfaces of an odd length are drawn on padded copies
    PackedPads pads;
    {
        const int rc = pads.begin(c, jobs.size(), [&](size_t j) -> DevSurface & { return jobs[j].sfc; });
        if (rc) return rc;
    }
    // ---- upload: gradients | fills | jobs | counters | strokes | polygons
    // through the pinned staging buffer, then the nodes straight from the
    // caller's memory
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t o_grads = 0;
    const size_t o_ext = al(o_grads + sizeof(DevGradient) * grads.size());  // stop tables of long gradients
    const size_t o_fills = al(o_ext + ext_stops_bytes(grads.data(), grads.size()));
    const size_t o_jobs = al(o_fills + sizeof(FillCmd) * (size_t)n_fills);
    const size_t o_cnt = al(o_jobs + sizeof(DevJob) * (size_t)n_jobs);
    const bool has_strokes = strokes && !strokes->empty();
    const size_t n_sk = has_strokes ? strokes->strokes.size() : 0, n_sb = has_strokes ? strokes->subs.size() : 0;
    const size_t n_tr = has_strokes ? strokes->trig.size() : 0;
    const size_t o_sk = al(o_cnt + sizeof(int32_t) * CNT_COUNT);
    const size_t o_sb = al(o_sk + sizeof(StrokeDev) * n_sk);
    const size_t o_tr = al(o_sb + sizeof(SubpathDev) * n_sb);
    // host-built polygons: per polygon its edge count, per contour its
    // start / size / fill / first edge, then the points
    const size_t n_poly = has_strokes ? strokes->polys.size() : 0;
    std::vector<int32_t> poly_fill(n_poly, -1);
    for (int32_t f = 0; f < n_fills; f++)
        if (fills[f].poly >= 0) poly_fill[(size_t)fills[f].poly] = f;
    long long n_pts = 0, n_ctr = 0;
    for (size_t k = 0; k < n_poly; k++) {
        const long long np = (long long)strokes->polys[k]->points();
        if (np > 0x7FFFFFFFll) {
            set_error("batch too large: more than 2^31 edges in one polygon");
            return Z2D_ERR_INVALID_ARGUMENT;
        }
        n_pts += np;
        n_ctr += (long long)strokes->polys[k]->ends.size();
    }
    if (n_ctr > 0x7FFFFFFFll) {
        set_error("batch too large: more than 2^31 contours");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    const size_t o_pe = al(o_tr + sizeof(double) * n_tr);
    const size_t o_cs = al(o_pe + sizeof(int32_t) * n_poly);
    const size_t o_cn = al(o_cs + sizeof(long long) * (size_t)n_ctr);
    const size_t o_cf = al(o_cn + sizeof(int32_t) * (size_t)n_ctr);
    const size_t o_ce = al(o_cf + sizeof(int32_t) * (size_t)n_ctr);
    const size_t o_pt = al(o_ce + sizeof(int32_t) * (size_t)n_ctr);
    const size_t total = al(o_pt + sizeof(double) * 2 * (size_t)n_pts);
    const size_t o_nodes = total;
    if (c.params.ensure(o_nodes + sizeof(z2d_node) * (size_t)n_nodes) || c.staging.ensure(total))
        return Z2D_ERR_OUT_OF_MEMORY;
    uint8_t *h = c.staging.as<uint8_t>();
    uint8_t *dv = c.params.as<uint8_t>();
    const DevGradient *dgrads = reinterpret_cast<const DevGradient *>(dv + o_grads);
    for (int32_t i = 0; i < n_fills; i++)
        if (grad_of_fill[i] >= 0) fills[i].src.grad = dgrads + grad_of_fill[i];
    // make sure the previous call's kernels no longer read the staging buffer
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    // (the flatten kernels are done with the nodes at the first readback
    // below, so the caller's array is free again when this call returns)
    Z2D_CUDA(cudaMemcpyAsync(dv + o_nodes, nodes, sizeof(z2d_node) * (size_t)n_nodes, cudaMemcpyHostToDevice, c.stream));
    if (!grads.empty()) {
        memcpy(h + o_grads, grads.data(), sizeof(DevGradient) * grads.size());
        put_ext_stops(reinterpret_cast<DevGradient *>(h + o_grads), grads.size(), h + o_ext, dv + o_ext);
    }
    memcpy(h + o_fills, fills.data(), sizeof(FillCmd) * (size_t)n_fills);
    memcpy(h + o_jobs, jobs.data(), sizeof(DevJob) * (size_t)n_jobs);
    int32_t *cnt_h = reinterpret_cast<int32_t *>(h + o_cnt);
    for (int i = 0; i < CNT_COUNT; i++) cnt_h[i] = 0;
    if (has_strokes) {
        memcpy(h + o_sk, strokes->strokes.data(), sizeof(StrokeDev) * n_sk);
        memcpy(h + o_sb, strokes->subs.data(), sizeof(SubpathDev) * n_sb);
        if (n_tr > 0) memcpy(h + o_tr, strokes->trig.data(), sizeof(double) * n_tr);
    }
    if (n_poly > 0) {
        int32_t *pe = reinterpret_cast<int32_t *>(h + o_pe);
        long long *cs = reinterpret_cast<long long *>(h + o_cs);
        int32_t *cn = reinterpret_cast<int32_t *>(h + o_cn), *cf = reinterpret_cast<int32_t *>(h + o_cf);
        int32_t *ce = reinterpret_cast<int32_t *>(h + o_ce);
        std::vector<long long> base(n_poly);
        long long pt = 0, ct = 0;
        for (size_t k = 0; k < n_poly; k++) {
            const stroke::Polygon &P = *strokes->polys[k];
            base[k] = pt;
            pe[k] = (int32_t)P.points();
            uint64_t prev = 0;
            for (uint64_t e : P.ends) {
                cs[ct] = pt + (long long)prev;
                cn[ct] = (int32_t)(e - prev);
                cf[ct] = poly_fill[k];
                ce[ct] = (int32_t)prev;
                prev = e;
                ct++;
            }
            pt += (long long)P.points();
        }
        // the points, polygon by polygon, over host threads
        double *hp = reinterpret_cast<double *>(h + o_pt);
        const size_t nt = std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()),
                                           (size_t)(n_pts >> 20) + 1);
        std::atomic<size_t> next{0};
        auto work = [&] {
            for (size_t k; (k = next.fetch_add(1)) < n_poly;) {
                const stroke::Polygon &P = *strokes->polys[k];
                if (!P.xy.empty()) memcpy(hp + 2 * base[k], P.xy.data(), sizeof(double) * P.xy.size());
            }
        };
        std::vector<std::thread> pool;
        for (size_t t = 1; t < nt; t++) pool.emplace_back(work);
        work();
        for (auto &th : pool) th.join();
    }
    Z2D_CUDA(cudaMemcpyAsync(dv, h, total, cudaMemcpyHostToDevice, c.stream));
    const z2d_node *d_nodes = reinterpret_cast<const z2d_node *>(dv + o_nodes);
    const FillCmd *d_fills = reinterpret_cast<const FillCmd *>(dv + o_fills);
    DevJob *d_jobs = reinterpret_cast<DevJob *>(dv + o_jobs);
    int32_t *d_cnt = reinterpret_cast<int32_t *>(dv + o_cnt);

    // node info, then the per-node leaf counts of the curves' frontier items
    const size_t info_bytes = (sizeof(NodeInfo) * (size_t)n_nodes + 255) & ~(size_t)255;
    const size_t items_bytes = (sizeof(uint16_t) * kFrontier * (size_t)n_nodes + 255) & ~(size_t)255;
    const size_t st_bytes = (sizeof(FillState) * (size_t)n_fills + 255) & ~(size_t)255;
    if (c.node_info.ensure(info_bytes + items_bytes + 3 * sizeof(int32_t) * (size_t)n_nodes) ||
        c.fill_state.ensure(st_bytes + sizeof(RasterFill) * (size_t)n_fills))
        return Z2D_ERR_OUT_OF_MEMORY;
    RasterFill *d_rf = reinterpret_cast<RasterFill *>(c.fill_state.as<uint8_t>() + st_bytes);
    NodeInfo *d_info = c.node_info.as<NodeInfo>();
    uint16_t *d_items = reinterpret_cast<uint16_t *>(c.node_info.as<uint8_t>() + info_bytes);
    int32_t *d_curves = reinterpret_cast<int32_t *>(c.node_info.as<uint8_t>() + info_bytes + items_bytes);  // 2 queues
    int32_t *d_nfill = d_curves + 2 * (size_t)n_nodes;
    FillState *d_st = c.fill_state.as<FillState>();
    Z2D_CUDA(cudaMemsetAsync(d_st, 0, sizeof(FillState) * (size_t)n_fills, c.stream));
    // each node's fill; nodes no fill owns (stroke commands' nodes, gaps) keep -1
    long long owned = 0;
    for (const FillCmd &F : fills) owned += F.n_nodes;
    if (owned < n_nodes) Z2D_CUDA(cudaMemsetAsync(d_nfill, 0xFF, sizeof(int32_t) * (size_t)n_nodes, c.stream));
    k_node_owner<<<grid_for(n_fills, 8), 256, 0, c.stream>>>(d_fills, n_fills, d_nfill);
    c.launches++;

    // ---- flatten
    const unsigned flat_blocks =
        (unsigned)std::min<long long>(grid_for((n_nodes + 31) / 32, kFlattenWarps), (long long)c.sm_count * 64);
    // one warp per queued curve, as many as there could be curves up to the
    // blocks the SMs hold at once: a grid of one wave, so the grid-stride
    // loop over the queue has no partial second wave
    static std::atomic<int> curve_occ{0};
    int curve_res = curve_occ.load(std::memory_order_relaxed);
    if (curve_res <= 0) {
        int a = 0, b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_curve_count_w, 32 * kFlattenWarps, 0) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_curve_emit_w, 32 * kFlattenWarps, 0) != cudaSuccess)
            a = b = 4;
        curve_res = std::max(1, std::min(a, b));
        curve_occ.store(curve_res, std::memory_order_relaxed);
    }
    const unsigned curve_blocks =
        (unsigned)std::min<long long>(grid_for(n_nodes, kFlattenWarps), (long long)c.sm_count * curve_res);
    // per curve warp: kScratch leaf points per lane; then the curve pool
    const size_t scratch_pts = (size_t)curve_blocks * kFlattenWarps * 32 * kScratch;
    // pool capacity: 16 points per node, or what the previous call asked for
    const int32_t pool_cap = (int32_t)std::min<long long>(
        64ll << 20, std::max<long long>({1ll << 20, 16ll * n_nodes, c.pool_demand + c.pool_demand / 4}));
    if (c.curve_pool.ensure(sizeof(double2) * (scratch_pts + (size_t)pool_cap))) return Z2D_ERR_OUT_OF_MEMORY;
    double2 *d_scratch = c.curve_pool.as<double2>();
    double2 *d_pool = d_scratch + scratch_pts;
    cudaEvent_t tf = c.timer_begin(c.t_flatten);
    k_node_count_w<<<flat_blocks, 32 * kFlattenWarps, 0, c.stream>>>(d_nodes, d_nfill, d_fills, d_info, n_nodes,
                                                                    d_curves, d_cnt);
    k_curve_count_w<<<curve_blocks, 32 * kFlattenWarps, 0, c.stream>>>(d_nodes, d_nfill, d_fills, d_info, d_curves,
                                                                      d_cnt, d_items, d_cnt + CNT_STATUS, d_scratch,
                                                                      d_pool, pool_cap);
    StrokeRun srun;
    if (n_sk > 0) {
        srun.nodes = d_nodes;
        srun.strokes = reinterpret_cast<const StrokeDev *>(dv + o_sk);
        srun.subs = reinterpret_cast<const SubpathDev *>(dv + o_sb);
        srun.trig = reinterpret_cast<const double *>(dv + o_tr);
        srun.n_strokes = (int32_t)n_sk;
        srun.n_subs = (int32_t)n_sb;
        srun.n_local = strokes->n_local;
        srun.n_pen = strokes->n_pen;
        const int rc = stroke_count(c, srun, d_cnt + CNT_STATUS);
        if (rc) return rc;
    }
    k_fill_scan<<<grid_for(n_fills, kScanWarps), 32 * kScanWarps, 0, c.stream>>>(
        d_nodes, d_fills, d_info, d_st, n_fills, d_cnt, d_cnt + CNT_STATUS, srun.stroke_edges,
        reinterpret_cast<const int32_t *>(dv + o_pe));
    c.timer_end(c.t_flatten, tf);
    c.launches += 3;
    const size_t rb_jobs_off = al(sizeof(int32_t) * CNT_COUNT + 2 * sizeof(long long));
    const size_t rb_bytes = rb_jobs_off + sizeof(DevJob) * (size_t)n_jobs;
    if (c.readback.ensure(rb_bytes)) return Z2D_ERR_OUT_OF_MEMORY;
    int32_t *rb = c.readback.as<int32_t>();
    long long *rb_tot = reinterpret_cast<long long *>(rb + CNT_COUNT);  // stroke contour totals (8-aligned: CNT_COUNT even)
    DevJob *rb_jobs = reinterpret_cast<DevJob *>(c.readback.as<uint8_t>() + rb_jobs_off);
    Z2D_CUDA(cudaMemcpyAsync(rb, d_cnt, sizeof(int32_t) * CNT_COUNT, cudaMemcpyDeviceToHost, c.stream));
    if (n_sk > 0)
        Z2D_CUDA(cudaMemcpyAsync(rb_tot, stroke_totals_dev(srun), 2 * sizeof(long long), cudaMemcpyDeviceToHost,
                                 c.stream));
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    c.pool_demand = (long long)std::min<unsigned long long>(
        64ull << 20, ((unsigned long long)(uint32_t)rb[CNT_POOL + 1] << 32) | (uint32_t)rb[CNT_POOL]);
    if (rb[CNT_STATUS] != 0) {
        set_error(rb[CNT_STATUS] == Z2D_ERR_INVALID_STATE ? "curve subdivision exceeded its depth bound"
                                                          : "batch too large: more than 2^31 edges in one polygon");
        return rb[CNT_STATUS];
    }
    if (n_sk > 0) {
        srun.n_a = rb_tot[0];
        srun.n_b = rb_tot[1];
    }
    const int32_t n_edges = rb[CNT_EDGES];
    if (n_edges < 0) return Z2D_ERR_OUT_OF_MEMORY;
    if (c.edges.ensure(sizeof(DEdge) * (size_t)std::max(n_edges, 1) + sizeof(int32_t) * (size_t)std::max(n_edges, 1)))
        return Z2D_ERR_OUT_OF_MEMORY;
    DEdge *d_edges = c.edges.as<DEdge>();
    int32_t *d_edge_fill = reinterpret_cast<int32_t *>(d_edges + std::max(n_edges, 1));
    // extents start at +inf/-inf keys: min slots 0xFF.., max slots 0
    tf = c.timer_begin(c.t_flatten);
    k_node_emit_w<<<flat_blocks, 32 * kFlattenWarps, 0, c.stream>>>(d_nodes, d_nfill, d_fills, d_info, d_st, d_edges,
                                                                   n_nodes, d_curves + n_nodes, d_cnt);
    k_curve_emit_w<<<curve_blocks, 32 * kFlattenWarps, 0, c.stream>>>(d_nodes, d_nfill, d_fills, d_info, d_st,
                                                                     d_edges, d_curves + n_nodes, d_cnt, d_items,
                                                                     d_pool);
    if (n_sk > 0) {
        const int rc = stroke_emit(c, srun, d_fills, d_st, d_edges);
        if (rc) return rc;
    }
    if (n_ctr > 0) {
        PolyRun pr;
        pr.pts = reinterpret_cast<const double2 *>(dv + o_pt);
        pr.start = reinterpret_cast<const long long *>(dv + o_cs);
        pr.n = reinterpret_cast<const int32_t *>(dv + o_cn);
        pr.fill = reinterpret_cast<const int32_t *>(dv + o_cf);
        pr.edge_off = reinterpret_cast<const int32_t *>(dv + o_ce);
        pr.n_contours = (int32_t)n_ctr;
        pr.n_points = n_pts;
        const int rc = poly_emit(c, pr, d_fills, d_st, d_edges);
        if (rc) return rc;
    }
    k_edge_fill<<<n_fills, 128, 0, c.stream>>>(d_st, n_fills, d_edge_fill);
    k_fill_setup<<<grid_for(n_fills, 64), 64, 0, c.stream>>>(d_fills, d_st, n_fills, d_jobs, d_cnt, d_rf);
    c.timer_end(c.t_flatten, tf);
    c.launches += 4;
    Z2D_CUDA(cudaMemcpyAsync(rb, d_cnt, sizeof(int32_t) * CNT_COUNT, cudaMemcpyDeviceToHost, c.stream));
    Z2D_CUDA(cudaMemcpyAsync(rb_jobs, d_jobs, sizeof(DevJob) * (size_t)n_jobs, cudaMemcpyDeviceToHost, c.stream));
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    const int32_t n_fb = rb[CNT_FILL_BANDS];
    const long long mask_bytes = (long long)(((unsigned long long)(uint32_t)rb[CNT_MASK_LO + 1] << 32) | (uint32_t)rb[CNT_MASK_LO]);
    const int32_t n_exact = rb[CNT_EXACT];
    // ---- layout: global bands, raster CTAs and band-list slots, job after job
    long long n_gbands = 0, n_tiles = 0, n_slots = 0;
    for (int32_t j = 0; j < n_jobs; j++) {
        DevJob &J = jobs[j];
        J.band_lo = rb_jobs[j].band_lo;
        J.band_hi = rb_jobs[j].band_hi;
        J.tcol_lo = rb_jobs[j].tcol_lo;
        J.tcol_hi = rb_jobs[j].tcol_hi;
        J.gband_base = (int32_t)n_gbands;
        J.tile_base = (int32_t)n_tiles;
        J.list_base = n_slots;
        if (J.band_hi < J.band_lo || J.tcol_hi < J.tcol_lo) {  // nothing is drawn on this surface
            J.band_lo = 0;
            J.band_hi = -1;
            J.tcol_lo = 0;
            J.tcol_hi = -1;
            continue;
        }
        const long long nb = J.band_hi - J.band_lo + 1, nc = J.tcol_hi - J.tcol_lo + 1;
        n_gbands += nb;
        n_tiles += nb * nc;
        n_slots += nb * (J.fill1 - J.fill0);
    }
    if (n_gbands == 0) return pads.finish(c);  // nothing is drawn
    if (n_tiles > 0x7FFFFFFFll || n_gbands > 0x7FFFFFFFll) {
        set_error("batch too large: more than 2^31 tiles");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    memcpy(rb_jobs, jobs.data(), sizeof(DevJob) * (size_t)n_jobs);
    Z2D_CUDA(cudaMemcpyAsync(d_jobs, rb_jobs, sizeof(DevJob) * (size_t)n_jobs, cudaMemcpyHostToDevice, c.stream));

    // ---- bins: counts, exclusive scan, scatter
    if (c.bin_offsets.ensure(sizeof(int32_t) * (2 * (size_t)n_fb + 2))) return Z2D_ERR_OUT_OF_MEMORY;
    int32_t *d_fb_cnt = c.bin_offsets.as<int32_t>();
    int32_t *d_fb_off = d_fb_cnt + (n_fb + 1);
    Z2D_CUDA(cudaMemsetAsync(d_fb_cnt, 0, sizeof(int32_t) * (size_t)(n_fb + 1), c.stream));
    cudaEvent_t tb = c.timer_begin(c.t_bins);
    if (n_edges > 0) {
        k_bin_count<<<grid_for(n_edges, 256), 256, 0, c.stream>>>(d_fills, d_st, d_edges, d_edge_fill, n_edges, d_fb_cnt,
                                                                   d_cnt + CNT_STATUS);
        c.launches++;
    }
    size_t tmp_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, d_fb_cnt, d_fb_off, n_fb + 1, c.stream);
    if (c.scan_tmp.ensure(tmp_bytes + 16)) return Z2D_ERR_OUT_OF_MEMORY;
    Z2D_CUDA(cub::DeviceScan::ExclusiveSum(c.scan_tmp.ptr, tmp_bytes, d_fb_cnt, d_fb_off, n_fb + 1, c.stream));
    c.timer_end(c.t_bins, tb);
    c.launches++;
    Z2D_CUDA(cudaMemcpyAsync(rb, d_fb_off + n_fb, sizeof(int32_t), cudaMemcpyDeviceToHost, c.stream));
    Z2D_CUDA(cudaMemcpyAsync(rb + 1, d_cnt + CNT_STATUS, sizeof(int32_t), cudaMemcpyDeviceToHost, c.stream));
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    const int32_t n_bin_entries = rb[0];
    if (rb[1] != 0) {
        set_error("a fill has more than 32000 edges inside one 4-row band");
        return rb[1];
    }
    if (c.bins.ensure(sizeof(int32_t) * (size_t)std::max(n_bin_entries, 1))) return Z2D_ERR_OUT_OF_MEMORY;
    // scatter with the counts array reused as cursors
    Z2D_CUDA(cudaMemcpyAsync(d_fb_cnt, d_fb_off, sizeof(int32_t) * (size_t)(n_fb + 1), cudaMemcpyDeviceToDevice, c.stream));
    tb = c.timer_begin(c.t_bins);
    if (n_edges > 0 && n_bin_entries > 0) {
        k_bin_fill<<<grid_for(n_edges, 256), 256, 0, c.stream>>>(d_fills, d_st, d_edges, d_edge_fill, n_edges, d_fb_cnt,
                                                                  c.bins.as<int32_t>());
        c.launches++;
    }

    // ---- ordered fill lists per global band
    const size_t count_bytes = ((sizeof(int32_t) * (size_t)n_gbands) + 15) & ~(size_t)15;
    if (c.band_fills.ensure(count_bytes + sizeof(int4) * (size_t)std::max(n_slots, 1ll))) return Z2D_ERR_OUT_OF_MEMORY;
    int32_t *d_band_count = c.band_fills.as<int32_t>();
    int4 *d_band_fills = reinterpret_cast<int4 *>(c.band_fills.as<uint8_t>() + count_bytes);
    k_band_lists<<<(unsigned)n_gbands, 256, 0, c.stream>>>(d_st, d_jobs, n_jobs, d_band_count, d_band_fills);
    c.launches++;

    // ---- exact path
    if (n_exact > 0) {
        // mask plus per-fill work arrays (3 ints per edge, 8-byte aligned)
        const size_t need = (size_t)mask_bytes + 64;
        if (c.masks.ensure(need)) return Z2D_ERR_OUT_OF_MEMORY;
        Z2D_CUDA(cudaMemsetAsync(c.masks.ptr, 0, (size_t)mask_bytes, c.stream));
        k_exact<<<grid_for(n_fills, 32), 32, 0, c.stream>>>(d_fills, d_st, d_edges, n_fills, d_jobs, c.masks.as<uint8_t>());
        c.launches++;
    }
    c.timer_end(c.t_bins, tb);

    // ---- raster
    RasterArgs A;
    A.jobs = d_jobs;
    A.fills = d_fills;
    A.st = d_st;
    A.edges = d_edges;
    A.bins = c.bins.as<int32_t>();
    A.bin_off = d_fb_off;
    A.band_count = d_band_count;
    A.band_fills = d_band_fills;
    A.rfills = d_rf;
    A.masks = c.masks.as<uint8_t>();
    A.n_jobs = n_jobs;
    A.job0 = jobs[0];
    const size_t smem = sizeof(uint32_t) * kWarpWords * kTileRows;
    {
        const int rc = raster_attributes(c);
        if (rc) return rc;
    }
    {
        const int rc = c.await_surface();  // a host surface's upload
        if (rc) return rc;
    }
    // persistent grid: every SM filled to the kernel's residency (or the
    // tuned CTAs per SM), never more CTAs than tiles
    static std::atomic<int> occ_cache[2];
    int occ = occ_cache[n_jobs == 1 ? 0 : 1].load(std::memory_order_relaxed);
    if (occ <= 0) {
        if (n_jobs == 1) Z2D_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<false, false>, kRasterThreads, smem));
        else Z2D_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_raster<true, false>, kRasterThreads, smem));
        occ = std::max(occ, 1);
        occ_cache[n_jobs == 1 ? 0 : 1].store(occ, std::memory_order_relaxed);
    }
    // the schedule: forced on the context, or the tuner's for this kind of pass
    const TuneKey key = tune_key(n_jobs, n_tiles, n_slots, n_gbands);
    c.last_key = key;
    RasterPlan plan{c.raster_ctas_per_sm, c.raster_order, c.raster_cta_items, -1};
    if (!c.raster_forced) {
        c.tune_collect(false);
        plan = tune_pick(key);
    }
    cudaEvent_t tune_t0 = nullptr, tune_t1 = nullptr;
    if (plan.candidate >= 0) {
        if (cudaEventCreate(&tune_t0) != cudaSuccess || cudaEventCreate(&tune_t1) != cudaSuccess) {
            if (tune_t0) cudaEventDestroy(tune_t0);
            tune_t0 = tune_t1 = nullptr;
            plan.candidate = -1;
        } else {
            Z2D_CUDA(cudaEventRecord(tune_t0, c.stream));
        }
    }
    // ctas < 0: one CTA per tile (a tile per item), else a persistent grid
    const int per_sm = plan.ctas > 0 ? std::min(plan.ctas, occ) : occ;
    const bool one_per_tile = plan.ctas < 0;
    const unsigned grid =
        one_per_tile ? (unsigned)n_tiles : (unsigned)std::min<long long>(n_tiles, (long long)c.sm_count * per_sm);
    if (one_per_tile) plan.cta_items = 1;
    A.one_per_tile = one_per_tile ? 1 : 0;
    A.queue = reinterpret_cast<unsigned long long *>(d_cnt + CNT_QUEUE);
    A.n_items = (unsigned long long)n_tiles * (plan.cta_items ? 1 : kTileRows);
    A.order = nullptr;
    if (plan.order == 1 && n_tiles > 1) {
        // longest bands first: tiles sorted by their band's fill count
        const size_t nt = (size_t)n_tiles;
        size_t sort_bytes = 0;
        cub::DeviceRadixSort::SortPairsDescending(nullptr, sort_bytes, (const int32_t *)nullptr, (int32_t *)nullptr,
                                                  (const int32_t *)nullptr, (int32_t *)nullptr, (int)nt, 0, 32,
                                                  c.stream);
        const size_t arr = (sizeof(int32_t) * nt + 255) & ~(size_t)255;
        if (c.tile_order.ensure(4 * arr + sort_bytes)) return Z2D_ERR_OUT_OF_MEMORY;
        uint8_t *b = c.tile_order.as<uint8_t>();
        int32_t *cost = reinterpret_cast<int32_t *>(b), *idx = reinterpret_cast<int32_t *>(b + arr);
        int32_t *cost_s = reinterpret_cast<int32_t *>(b + 2 * arr), *order = reinterpret_cast<int32_t *>(b + 3 * arr);
        k_tile_cost<<<grid_for((long long)nt, 256), 256, 0, c.stream>>>(d_jobs, n_jobs, d_band_count, (int32_t)nt, cost,
                                                                         idx);
        Z2D_CUDA(cub::DeviceRadixSort::SortPairsDescending(b + 4 * arr, sort_bytes, cost, cost_s, idx, order, (int)nt,
                                                           0, 32, c.stream));
        c.launches += 2;
        A.order = order;
    }
    cudaEvent_t t0 = c.timer_begin(c.t_raster);
    if (plan.cta_items) {
        if (n_jobs == 1) k_raster<false, true><<<grid, kRasterThreads, smem, c.stream>>>(A);
        else k_raster<true, true><<<grid, kRasterThreads, smem, c.stream>>>(A);
    } else {
        if (n_jobs == 1) k_raster<false, false><<<grid, kRasterThreads, smem, c.stream>>>(A);
        else k_raster<true, false><<<grid, kRasterThreads, smem, c.stream>>>(A);
    }
    c.timer_end(c.t_raster, t0);
    if (plan.candidate >= 0) {
        Z2D_CUDA(cudaEventRecord(tune_t1, c.stream));
        c.tune_pending.push_back(TunePending{key, plan.candidate, tune_t0, tune_t1});
    }
    c.launches++;
    Z2D_CUDA(cudaGetLastError());
    return pads.finish(c);
}

// ------------------------------------------------------- small fills
// One fill of a short path: everything up to the rasteriser runs on the
// host (a few microseconds for a few hundred edges) and reaches the device
// in one upload, so the call costs one copy and one launch instead of the
// pipeline's launches and size readbacks.  The host steps restate the same
// z2d code as the device kernels, with the same f64 operations in the same
// order (the host is compiled without FP contraction), so the edges, the
// fill's box and the tiles are the device pipeline's; bins list a band's
// edges in any order (the rasteriser's sums do not depend on it).
namespace {

// The host's work grows with the edges (about 20-30 ns each to flatten and
// bin) while the pipeline's cost is mostly fixed (~100 us of launches and
// readbacks for a small call), so the path takes calls whose edge count,
// estimated before and counted while flattening, stays below a budget:
// one surface up to 4,096 edges; several (as in the server's passes under
// load, where the pipeline's fixed cost is shared) up to 1,024 on at most
// 8 surfaces.
constexpr int32_t kSmallMaxNodes = 4096;       // nodes of all the call's fills
constexpr size_t kSmallEdgesOne = 4096;        // edge budget, one surface
constexpr size_t kSmallEdgesMany = 1024;       // edge budget, several surfaces
constexpr size_t kSmallMaxJobs = 8;
constexpr size_t kSmallMaxBins = 1 << 17;      // (edge, band) pairs
constexpr long long kSmallMaxBands = 1 << 16;  // (fill, band) slots and band-list entries
constexpr int kSmallMaxDepth = 40;  // below the device subdivision bound

struct HostFlatten {
    const FillCmd &F;
    std::vector<DEdge> &edges;
    size_t max_edges;
    double et = 0, eb = 0, el = 0, er = 0;
    bool any = false, overflow = false;
    // PointBuffer(1, 3) of fill_plotter: its first and last points and length
    double fx = 0, fy = 0, lx = 0, ly = 0;
    int count = 0;

    // Polygon.addEdge (Polygon.zig:61-109), as add_edge in edges.cuh
    void edge(double x0, double y0, double x1, double y1) {
        if (edges.size() >= max_edges) {
            overflow = true;
            return;
        }
        const double ax = x0 * F.edge_scale, ay = y0 * F.edge_scale, bx = x1 * F.edge_scale, by = y1 * F.edge_scale;
        DEdge e{};
        if (ay < by) {
            e.top = ay;
            e.x_start = ax;
            e.x_inc = (bx - ax) / (by - ay);
            e.dir = -1;
            e.rb = (int32_t)std::round(by);
        } else if (ay > by) {
            e.top = by;
            e.x_start = bx;
            e.x_inc = (ax - bx) / (ay - by);
            e.dir = 1;
            e.rb = (int32_t)std::round(ay);
        } else {
            e.rt = 1;
            e.rb = 0;
            edges.push_back(e);
            return;
        }
        e.rt = (int32_t)std::round(e.top);
        e.fxs = (float)e.x_start;
        e.fxi = (float)e.x_inc;
        e.ftp = (float)e.top;
        const double bot = ay < by ? by : ay;
        const double l = ax < bx ? ax : bx, r = ax < bx ? bx : ax;
        if (!any) {
            et = e.top, eb = bot, el = l, er = r;
            any = true;
        } else {
            if (e.top < et) et = e.top;
            if (bot > eb) eb = bot;
            if (l < el) el = l;
            if (r > er) er = r;
        }
        edges.push_back(e);
    }
    // lineTo through the point buffer (fill_plotter.zig:44-51, 100-118)
    void line_to(double x, double y) {
        if (lx == x && ly == y) return;
        edge(lx, ly, x, y);
        lx = x;
        ly = y;
        count = count < 3 ? count + 1 : 3;
    }
    struct K {
        double ax, ay, bx, by, cx, cy, dx, dy;
    };
    static double error_sq(const K &k) {  // Spline.Knots.errorSq (Spline.zig:83-123)
        double bx = k.bx - k.ax, by = k.by - k.ay, cx = k.cx - k.ax, cy = k.cy - k.ay;
        if (k.ax != k.dx || k.ay != k.dy) {
            const double dx = k.dx - k.ax, dy = k.dy - k.ay;
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
    }
    // Spline.decompose / decomposeInto (Spline.zig:37-79): depth-first, the
    // first half before the second, leaves' start points then d
    bool curve(const double *p) {
        const double ax = lx, ay = ly;
        if (ax == p[0] && ay == p[1] && p[2] == p[4] && p[3] == p[5]) {
            line_to(p[4], p[5]);
            return true;
        }
        const double tol2 = F.tol * F.tol;
        struct Item {
            K k;
            int depth;
        };
        Item stack[kSmallMaxDepth + 2];
        int top = 0;
        stack[top++] = Item{K{ax, ay, p[0], p[1], p[2], p[3], p[4], p[5]}, 0};
        auto half = [](double a, double b) { return a + ((b - a) / 2); };
        while (top > 0) {
            Item it = stack[--top];
            K &k = it.k;
            if (error_sq(k) < tol2) {
                if (!(k.ax == ax && k.ay == ay)) line_to(k.ax, k.ay);
                if (overflow) return true;
                continue;
            }
            if (it.depth >= kSmallMaxDepth) return false;
            // deCasteljau: k becomes the first half, s2 the second
            const double abx = half(k.ax, k.bx), aby = half(k.ay, k.by);
            const double bcx = half(k.bx, k.cx), bcy = half(k.by, k.cy);
            const double cdx = half(k.cx, k.dx), cdy = half(k.cy, k.dy);
            const double abbcx = half(abx, bcx), abbcy = half(aby, bcy);
            const double bccdx = half(bcx, cdx), bccdy = half(bcy, cdy);
            const double fx_ = half(abbcx, bccdx), fy_ = half(abbcy, bccdy);
            const K s2{fx_, fy_, bccdx, bccdy, cdx, cdy, k.dx, k.dy};
            const K s1{k.ax, k.ay, abx, aby, abbcx, abbcy, fx_, fy_};
            stack[top++] = Item{s2, it.depth + 1};
            stack[top++] = Item{s1, it.depth + 1};
        }
        line_to(p[4], p[5]);
        return true;
    }
    // fill_plotter.plot (fill_plotter.zig:21-97); false: not for this path
    bool plot(const z2d_node *nodes, int32_t n, bool &open_chain) {
        for (int32_t i = 0; i < n && !overflow; i++) {
            const z2d_node &nd = nodes[i];
            switch (nd.tag) {
                case Z2D_MOVE_TO:
                    if (i == n - 1) return true;  // the auto-added move_to after close_path
                    fx = lx = nd.p[0];
                    fy = ly = nd.p[1];
                    count = 1;
                    break;
                case Z2D_LINE_TO:
                    if (count == 0) return false;  // InvalidState: the pipeline reports it
                    line_to(nd.p[0], nd.p[1]);
                    break;
                case Z2D_CURVE_TO:
                    if (count == 0) return false;
                    if (!curve(nd.p)) return false;
                    break;
                default:  // close_path
                    if (count >= 3) {
                        if (!(lx == fx && ly == fy)) {
                            edge(lx, ly, fx, fy);
                            lx = fx;
                            ly = fy;
                        }
                    } else if (count > 0 && !(lx == fx && ly == fy)) {
                        open_chain = true;
                    }
                    break;
            }
        }
        return !overflow;
    }
};

// An estimate of a path's edges before flattening it: one per line_to and
// close_path, and for a curve 2^k leaves with k the levels of halving that
// bring the initial knots' errorSq below tol^2 (each halving divides it by
// about 16).
size_t estimate_edges(const z2d_node *nodes, int32_t n, double tol) {
    size_t est = 0;
    double lx = 0, ly = 0;
    const double tol2 = tol * tol;
    for (int32_t i = 0; i < n; i++) {
        const z2d_node &nd = nodes[i];
        if (nd.tag == Z2D_CURVE_TO) {
            const HostFlatten::K k{lx, ly, nd.p[0], nd.p[1], nd.p[2], nd.p[3], nd.p[4], nd.p[5]};
            const double e = HostFlatten::error_sq(k);
            size_t leaves = 1;
            if (e >= tol2) {
                const double lv = std::ceil(std::log2(e / tol2) / 4.0);
                leaves = lv >= 20.0 ? ((size_t)1 << 20) : ((size_t)1 << (size_t)std::max(0.0, lv));
            }
            est += leaves;
            lx = nd.p[4];
            ly = nd.p[5];
        } else {
            est += 1;
            if (nd.tag != Z2D_CLOSE_PATH) {
                lx = nd.p[0];
                ly = nd.p[1];
            }
        }
    }
    return est;
}

}  // namespace

int run_small_jobs(Ctx &c, std::vector<DevJob> &jobs, const z2d_node *nodes, const std::vector<FillCmd> &fills,
                   const std::vector<DevGradient> &grads, const std::vector<int32_t> &grad_of_fill, bool &done) {
    done = false;
    const size_t n_fills = fills.size(), n_jobs = jobs.size();
    if (n_fills == 0 || n_jobs == 0 || n_jobs > kSmallMaxJobs) return Z2D_OK;
    const size_t budget = n_jobs == 1 ? kSmallEdgesOne : kSmallEdgesMany;
    long long total_nodes = 0;
    for (const FillCmd &F : fills) {
        if (F.aa != Z2D_AA_MULTISAMPLE_4X || F.stroke >= 0 || F.poly >= 0 || F.n_nodes <= 0) return Z2D_OK;
        total_nodes += F.n_nodes;
    }
    if (total_nodes > kSmallMaxNodes) return Z2D_OK;
    size_t est = 0;
    for (const FillCmd &F : fills) {
        est += estimate_edges(nodes + F.node_off, F.n_nodes, F.tol);
        if (est > budget) return Z2D_OK;
    }
    for (const DevJob &J : jobs)
        if (fmt_packed(J.sfc.fmt)) return Z2D_OK;
    for (const DevGradient &g : grads)
        if (g.n_stops > kMaxStops) return Z2D_OK;
    // ---- flatten every fill (fill_plotter.plot)
    static thread_local std::vector<DEdge> edges;
    static thread_local std::vector<FillState> st;
    static thread_local std::vector<RasterFill> rf;
    static thread_local std::vector<double> ext;  // et, eb, el, er per fill
    edges.clear();
    st.assign(n_fills, FillState{});
    rf.assign(n_fills, RasterFill{});
    ext.assign(4 * n_fills, 0.0);
    for (size_t f = 0; f < n_fills; f++) {
        const size_t e0 = edges.size();
        HostFlatten H{fills[f], edges, budget};
        bool open_chain = false;
        if (!H.plot(nodes + fills[f].node_off, fills[f].n_nodes, open_chain) || open_chain) return Z2D_OK;
        st[f].edge_base = (int32_t)e0;
        st[f].n_edges = (int32_t)(edges.size() - e0);
        st[f].has_edges = H.any ? 1 : 0;
        ext[4 * f] = H.et, ext[4 * f + 1] = H.eb, ext[4 * f + 2] = H.el, ext[4 * f + 3] = H.er;
    }
    // ---- k_fill_setup per fill: Polygon.inBox, multisample.run's draw box,
    // the bands and tile columns it touches
    auto clampi_h = [](int32_t v, int32_t lo, int32_t hi) { return std::max(lo, std::min(v, hi)); };
    static thread_local std::vector<DevJob> J;
    J = jobs;
    for (DevJob &jb : J) {
        jb.band_lo = jb.tcol_lo = 0x7FFFFFFF;
        jb.band_hi = jb.tcol_hi = -1;
        jb.gband_base = jb.tile_base = 0;
        jb.list_base = 0;
    }
    long long n_fb = 0;
    for (size_t f = 0; f < n_fills; f++) {
        const FillCmd &F = fills[f];
        FillState &S = st[f];
        DevJob &jb = J[(size_t)F.job];
        const int32_t sw = jb.sfc.w, sh = jb.sfc.h;
        const double et = ext[4 * f], eb = ext[4 * f + 1], el = ext[4 * f + 2], er = ext[4 * f + 3];
        if (!S.has_edges || er < 0.0 || eb < 0.0) continue;
        const double sc = F.scale;
        const int32_t psx = (int32_t)std::floor(el / sc), psy = (int32_t)std::floor(et / sc);
        const int32_t pex = (int32_t)std::ceil(er / sc), pey = (int32_t)std::ceil(eb / sc);
        const int32_t pw = pex - psx, ph = pey - psy;
        if (pw == 0 || ph == 0 || psx + pw < 0 || psy + ph < 0 || psx >= sw || psy >= sh) continue;
        S.active = 1;
        S.start_y = clampi_h((int32_t)std::floor(et / 4.0), 0, sh - 1);
        S.end_y = clampi_h((int32_t)std::ceil(eb / 4.0), S.start_y, sh - 1);
        S.start_x = clampi_h((int32_t)std::floor(el / 4.0), 0, sw - 1);
        S.end_x = clampi_h((int32_t)std::ceil(er / 4.0), S.start_x, sw);
        const bool bounded = is_bounded(F.op);
        S.band0 = (bounded ? S.start_y : 0) / kTileRows;
        S.band1 = (bounded ? S.end_y : sh - 1) / kTileRows;
        S.fb_base = (int32_t)n_fb;
        n_fb += S.band1 - S.band0 + 1;
        S.cull_x0 = bounded ? S.start_x : 0;
        S.cull_x1 = bounded ? S.end_x : sw;
        jb.band_lo = std::min(jb.band_lo, S.band0);
        jb.band_hi = std::max(jb.band_hi, S.band1);
        jb.tcol_lo = std::min(jb.tcol_lo, S.cull_x0 / kTileCols);
        jb.tcol_hi = std::max(jb.tcol_hi, (std::max(S.cull_x1, S.cull_x0 + 1) - 1) / kTileCols);
        RasterFill &R = rf[f];
        R.start_x = S.start_x;
        R.end_x = S.end_x;
        R.start_y = S.start_y;
        R.end_y = S.end_y;
        R.meta = ((uint32_t)F.op & RF_OP_MASK) | ((uint32_t)F.aa << RF_AA_SHIFT) |
                 (F.rule == Z2D_FILL_EVEN_ODD ? RF_EVEN_ODD : 0u) | ((uint32_t)F.fast_kind << RF_FAST_SHIFT) |
                 (bounded ? RF_BOUNDED : 0u);
        R.px = (F.src.pix.r & 0xFFu) | ((F.src.pix.g & 0xFFu) << 8) | ((F.src.pix.b & 0xFFu) << 16) |
               ((F.src.pix.a & 0xFFu) << 24);
    }
    done = true;
    if (n_fb == 0) return Z2D_OK;  // nothing is drawn
    if (n_fb > kSmallMaxBands) {
        done = false;
        return Z2D_OK;
    }
    // ---- layout: global bands, tiles and band-list storage, job after job
    long long n_gbands = 0, n_tiles = 0, n_slots = 0;
    for (DevJob &jb : J) {
        jb.gband_base = (int32_t)n_gbands;
        jb.tile_base = (int32_t)n_tiles;
        jb.list_base = n_slots;
        if (jb.band_hi < jb.band_lo || jb.tcol_hi < jb.tcol_lo) {
            jb.band_lo = 0;
            jb.band_hi = -1;
            jb.tcol_lo = 0;
            jb.tcol_hi = -1;
            continue;
        }
        const long long nb = jb.band_hi - jb.band_lo + 1, nc = jb.tcol_hi - jb.tcol_lo + 1;
        n_gbands += nb;
        n_tiles += nb * nc;
        n_slots += nb * (jb.fill1 - jb.fill0);
    }
    if (n_slots > kSmallMaxBands || n_tiles > 0x7FFFFFFF) {
        done = false;
        return Z2D_OK;
    }
    // ---- bins: each edge in the bands of its active sample rows (edge_bands)
    static thread_local std::vector<int32_t> cnt, off, bins, bcount;
    static thread_local std::vector<int4> blist;
    cnt.assign((size_t)n_fb + 1, 0);
    auto for_bands = [&](auto &&visit) {
        for (size_t f = 0; f < n_fills; f++) {
            const FillState &S = st[f];
            if (!S.active) continue;
            const int32_t S_ = (int32_t)fills[f].scale;
            for (int32_t k = 0; k < S.n_edges; k++) {
                const DEdge &e = edges[(size_t)(S.edge_base + k)];
                if (e.dir == 0) continue;
                const int32_t lo = std::max(e.rt, S.start_y * S_), hi = std::min(e.rb, (S.end_y + 1) * S_);
                if (lo >= hi) continue;
                const int32_t b0 = lo / (kTileRows * S_), b1 = (hi - 1) / (kTileRows * S_);
                for (int32_t b = b0; b <= b1; b++) visit(S.fb_base + (b - S.band0), S.edge_base + k);
            }
        }
    };
    size_t n_bins = 0;
    for_bands([&](int32_t fb, int32_t) {
        cnt[(size_t)fb]++;
        n_bins++;
    });
    if (n_bins > kSmallMaxBins) {
        done = false;
        return Z2D_OK;
    }
    for (long long fb = 0; fb < n_fb; fb++)
        if (cnt[(size_t)fb] > kMaxBandEdges) {
            done = false;  // the pipeline reports it
            return Z2D_OK;
        }
    off.assign((size_t)n_fb + 1, 0);
    for (long long fb = 0; fb < n_fb; fb++) off[(size_t)fb + 1] = off[(size_t)fb] + cnt[(size_t)fb];
    bins.assign(std::max<size_t>(n_bins, 1), 0);
    for (long long fb = 0; fb < n_fb; fb++) cnt[(size_t)fb] = off[(size_t)fb];
    for_bands([&](int32_t fb, int32_t e) { bins[(size_t)cnt[(size_t)fb]++] = e; });
    // ---- band lists (k_band_lists): the job's fills touching each band, in order
    bcount.assign(std::max<long long>(n_gbands, 1), 0);
    blist.assign(std::max<long long>(n_slots, 1), make_int4(0, 0, 0, 0));
    for (const DevJob &jb : J) {
        if (jb.band_hi < jb.band_lo) continue;
        const int32_t nf = jb.fill1 - jb.fill0;
        for (int32_t b = jb.band_lo; b <= jb.band_hi; b++) {
            const int32_t lb = b - jb.band_lo;
            int4 *out = blist.data() + jb.list_base + (long long)lb * nf;
            int32_t k = 0;
            for (int32_t f = jb.fill0; f < jb.fill1; f++) {
                const FillState &S = st[(size_t)f];
                if (S.active && b >= S.band0 && b <= S.band1)
                    out[k++] = make_int4(f, S.cull_x0, S.cull_x1, S.fb_base + (b - S.band0));
            }
            bcount[(size_t)(jb.gband_base + lb)] = k;
        }
    }
    // ---- one upload
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t o_jobs = 0, o_fill = al(sizeof(DevJob) * n_jobs);
    const size_t o_st = o_fill + al(sizeof(FillCmd) * n_fills), o_rf = o_st + al(sizeof(FillState) * n_fills);
    const size_t o_edges = o_rf + al(sizeof(RasterFill) * n_fills);
    const size_t o_bins = o_edges + al(sizeof(DEdge) * std::max<size_t>(edges.size(), 1));
    const size_t o_off = o_bins + al(sizeof(int32_t) * bins.size());
    const size_t o_cnt = o_off + al(sizeof(int32_t) * ((size_t)n_fb + 1));
    const size_t o_list = o_cnt + al(sizeof(int32_t) * bcount.size());
    const size_t o_grad = o_list + al(sizeof(int4) * blist.size());
    const size_t total = o_grad + al(sizeof(DevGradient) * std::max<size_t>(grads.size(), 1));
    const int slot = c.small_slot;
    c.small_slot ^= 1;
    HostBuf &hb = c.small_stage[slot];
    if (!c.small_done[slot]) Z2D_CUDA(cudaEventCreateWithFlags(&c.small_done[slot], cudaEventDisableTiming));
    Z2D_CUDA(cudaEventSynchronize(c.small_done[slot]));  // the slot's previous upload has been read
    if (hb.ensure(total) || c.small_params.ensure(total)) return Z2D_ERR_OUT_OF_MEMORY;
    uint8_t *h = hb.as<uint8_t>(), *dv = c.small_params.as<uint8_t>();
    memcpy(h + o_jobs, J.data(), sizeof(DevJob) * n_jobs);
    FillCmd *hf = reinterpret_cast<FillCmd *>(h + o_fill);
    memcpy(hf, fills.data(), sizeof(FillCmd) * n_fills);
    const DevGradient *dgrads = reinterpret_cast<const DevGradient *>(dv + o_grad);
    for (size_t f = 0; f < n_fills; f++)
        if (grad_of_fill[f] >= 0) hf[f].src.grad = dgrads + grad_of_fill[f];
    memcpy(h + o_st, st.data(), sizeof(FillState) * n_fills);
    memcpy(h + o_rf, rf.data(), sizeof(RasterFill) * n_fills);
    if (!edges.empty()) memcpy(h + o_edges, edges.data(), sizeof(DEdge) * edges.size());
    memcpy(h + o_bins, bins.data(), sizeof(int32_t) * bins.size());
    memcpy(h + o_off, off.data(), sizeof(int32_t) * ((size_t)n_fb + 1));
    memcpy(h + o_cnt, bcount.data(), sizeof(int32_t) * bcount.size());
    memcpy(h + o_list, blist.data(), sizeof(int4) * blist.size());
    if (!grads.empty()) memcpy(h + o_grad, grads.data(), sizeof(DevGradient) * grads.size());
    Z2D_CUDA(cudaMemcpyAsync(dv, h, total, cudaMemcpyHostToDevice, c.stream));
    Z2D_CUDA(cudaEventRecord(c.small_done[slot], c.stream));
    if (n_tiles == 0) return Z2D_OK;
    // ---- the rasteriser, one CTA per tile
    RasterArgs A{};
    A.job0 = J[0];
    A.jobs = reinterpret_cast<const DevJob *>(dv + o_jobs);
    A.fills = reinterpret_cast<const FillCmd *>(dv + o_fill);
    A.st = reinterpret_cast<const FillState *>(dv + o_st);
    A.edges = reinterpret_cast<const DEdge *>(dv + o_edges);
    A.bins = reinterpret_cast<const int32_t *>(dv + o_bins);
    A.bin_off = reinterpret_cast<const int32_t *>(dv + o_off);
    A.band_count = reinterpret_cast<const int32_t *>(dv + o_cnt);
    A.band_fills = reinterpret_cast<const int4 *>(dv + o_list);
    A.rfills = reinterpret_cast<const RasterFill *>(dv + o_rf);
    A.masks = nullptr;
    A.n_jobs = (int32_t)n_jobs;
    A.queue = nullptr;
    A.n_items = (unsigned long long)n_tiles;
    A.order = nullptr;
    A.one_per_tile = 1;
    const int rc = raster_attributes(c);
    if (rc) return rc;
    {
        const int rs = c.await_surface();
        if (rs) return rs;
    }
    const size_t smem = sizeof(uint32_t) * kWarpWords * kTileRows;
    cudaEvent_t t0 = c.timer_begin(c.t_raster);
    if (n_jobs == 1) k_raster<false, true><<<(unsigned)n_tiles, kRasterThreads, smem, c.stream>>>(A);
    else k_raster<true, true><<<(unsigned)n_tiles, kRasterThreads, smem, c.stream>>>(A);
    c.timer_end(c.t_raster, t0);
    c.launches++;
    Z2D_CUDA(cudaGetLastError());
    return Z2D_OK;
}

}  // namespace z2dg
