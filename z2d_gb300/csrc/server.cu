// server.cu -- continuous batching in front of z2dgpu_fill_jobs.
//
// Callers submit fill requests from any thread and wait for them by ticket.
// A request draws its fills either on a caller-owned device surface or on a
// surface the server allocates from its device pool (initialised from a
// host copy or cleared, and read back into a caller host buffer when the
// request completes).
//
// The server runs `lanes` workers, each with its own context (stream and
// scratch memory).  A free lane takes the requests queued at that moment
// (after an optional batching window, up to max_batch) and draws them in
// one z2dgpu_fill_jobs pass; while it draws, the other lanes take the
// requests that keep arriving, so several batches are on the GPU at once and
// the host work of one (validation, staging, the pass's size readbacks)
// overlaps the device work of another.
//
// Admission: a request on a pool surface enters a batch only once the pool
// can hold its surface; the pool is one device allocation sized at creation
// from the free HBM the driver reports (cudaMemGetInfo), at most 40 GB.
// Requests are admitted in arrival order (a request that does not fit holds
// back the ones behind it), so large requests are not starved.
//
// Ordering: requests on the same caller-owned surface are drawn in
// submission order: a surface is in at most one batch at a time, and a
// request whose surface is busy holds back the later requests on it.
// Requests are copied at submit time (nodes, commands, patterns, gradients
// and stops, initial pixels), so the caller's buffers may be reused as soon
// as submit returns; caller-owned surfaces and `out` buffers must stay valid
// until the request completes.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "z2d_internal.h"

using Clock = std::chrono::steady_clock;

namespace z2dg {
namespace {

constexpr size_t kPoolAlign = 256;
constexpr unsigned long long kPoolCap = 40ull << 30;  // the pool never exceeds 40 GB

struct Request {
    uint64_t id = 0;
    z2d_surface surface{};
    bool owned = false;         // surface allocated from the pool
    size_t bytes = 0;           // pool block size (the surface rounded up to whole 32-bit words)
    size_t exact = 0;           // the surface's own size in bytes (z2d's layout)
    size_t pool_off = 0;
    std::vector<uint8_t> init;  // initial pixels of a pool surface (empty: cleared)
    void *out = nullptr;        // host buffer receiving a pool surface's pixels
    std::vector<z2d_node> nodes;
    std::vector<z2d_fill_cmd> cmds;
    std::vector<z2d_pattern> patterns;
    std::vector<z2d_gradient> gradients;
    std::vector<z2d_stop> stops;
    int status = -1;  // -1 while pending
    std::string error;
    Clock::time_point t_submit, t_done;
};

// Deep copy of the commands' patterns (and gradient stops) into r.
int copy_request(Request &r, const z2d_node *nodes, size_t n_nodes, const z2d_fill_cmd *cmds, size_t n_cmds) {
    if ((n_nodes > 0 && !nodes) || (n_cmds > 0 && !cmds)) return Z2D_ERR_INVALID_ARGUMENT;
    r.nodes.assign(nodes, nodes + n_nodes);
    r.cmds.assign(cmds, cmds + n_cmds);
    size_t n_grad = 0, n_stops = 0;
    for (size_t i = 0; i < n_cmds; i++) {
        if (!cmds[i].pattern) return Z2D_ERR_INVALID_ARGUMENT;
        const z2d_gradient *g = cmds[i].pattern->gradient;
        if (g) {
            if (g->n_stops < 0 || (g->n_stops > 0 && !g->stops)) return Z2D_ERR_INVALID_ARGUMENT;
            n_grad++;
            n_stops += (size_t)g->n_stops;
        }
    }
    r.patterns.resize(n_cmds);
    r.gradients.resize(n_grad);
    r.stops.resize(n_stops);
    size_t gi = 0, si = 0;
    for (size_t i = 0; i < n_cmds; i++) {
        r.patterns[i] = *cmds[i].pattern;
        const z2d_gradient *g = cmds[i].pattern->gradient;
        if (g) {
            r.gradients[gi] = *g;
            if (g->n_stops > 0) memcpy(&r.stops[si], g->stops, sizeof(z2d_stop) * (size_t)g->n_stops);
            r.gradients[gi].stops = g->n_stops > 0 ? &r.stops[si] : nullptr;
            r.patterns[i].gradient = &r.gradients[gi];
            si += (size_t)g->n_stops;
            gi++;
        }
        r.cmds[i].pattern = &r.patterns[i];
    }
    return Z2D_OK;
}

// First-fit allocator over one device allocation; free blocks are merged
// with their neighbours.  Guarded by the server's mutex.
struct Pool {
    uint8_t *base = nullptr;
    size_t cap = 0, used = 0, peak = 0;
    std::map<size_t, size_t> free_blocks;  // offset -> size

    bool alloc(size_t bytes, size_t &off) {
        bytes = (bytes + kPoolAlign - 1) & ~(kPoolAlign - 1);
        for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
            if (it->second < bytes) continue;
            off = it->first;
            const size_t rest = it->second - bytes;
            free_blocks.erase(it);
            if (rest > 0) free_blocks[off + bytes] = rest;
            used += bytes;
            peak = std::max(peak, used);
            return true;
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + kPoolAlign - 1) & ~(kPoolAlign - 1);
        used -= bytes;
        auto next = free_blocks.lower_bound(off);
        if (next != free_blocks.end() && off + bytes == next->first) {
            bytes += next->second;
            next = free_blocks.erase(next);
        }
        if (next != free_blocks.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += bytes;
                return;
            }
        }
        free_blocks[off] = bytes;
    }
};

// A pool surface's transfer: `bytes` at `dev`, from / to offset `off` of the
// lane's transfer buffer; mode 0 copies in from the buffer, 1 clears, 2
// copies out to the buffer.
struct Xfer {
    uint8_t *dev;
    long long bytes, off;
    int32_t mode, pad_;
};

// One block per transfer; 16-byte vectors where both ends allow them.
__global__ void __launch_bounds__(256) k_xfer(const Xfer *__restrict__ xs, uint8_t *__restrict__ buf) {
    const Xfer x = xs[blockIdx.x];
    uint8_t *const a = x.dev;
    uint8_t *const b = buf + x.off;
    const long long n16 = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) ? 0 : x.bytes / 16;
    for (long long i = threadIdx.x; i < n16; i += blockDim.x) {
        uint4 *pa = reinterpret_cast<uint4 *>(a) + i;
        uint4 *pb = reinterpret_cast<uint4 *>(b) + i;
        if (x.mode == 0) *pa = *pb;
        else if (x.mode == 1) *pa = make_uint4(0, 0, 0, 0);
        else *pb = *pa;
    }
    for (long long i = n16 * 16 + threadIdx.x; i < x.bytes; i += blockDim.x) {
        if (x.mode == 0) a[i] = b[i];
        else if (x.mode == 1) a[i] = 0;
        else b[i] = a[i];
    }
}

}  // namespace
}  // namespace z2dg

using namespace z2dg;

struct z2dgpu_server {
    struct Lane {
        z2dgpu_ctx *ctx = nullptr;
        std::thread th;
        DevBuf xfer_dev;  // transfer descriptors and pool surfaces' pixels
        HostBuf xfer_host;
    };
    int device = 0;
    size_t max_batch = 1;
    std::chrono::microseconds max_wait{0};
    std::vector<std::unique_ptr<Lane>> lanes;
    Pool pool;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::list<std::shared_ptr<Request>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> by_id;
    std::unordered_set<uintptr_t> busy;  // caller-owned surfaces in a batch
    uint64_t next_id = 1;
    bool stopping = false;
    uint64_t n_batches = 0, n_requests = 0, n_deferred = 0;
    int inflight = 0, max_inflight = 0;
    double busy_ms = 0;

    void lane_run(Lane &L);
    std::vector<std::shared_ptr<Request>> take_batch();
    int draw_pass(Lane &L, std::vector<std::shared_ptr<Request>> &batch);
    void draw(Lane &L, std::vector<std::shared_ptr<Request>> &batch);
};

// The requests a lane takes now, in arrival order (caller holds mu).
std::vector<std::shared_ptr<Request>> z2dgpu_server::take_batch() {
    std::vector<std::shared_ptr<Request>> batch;
    std::unordered_set<uintptr_t> held;  // caller-owned surfaces whose next request must wait
    for (auto it = queue.begin(); it != queue.end() && batch.size() < max_batch;) {
        Request &r = **it;
        if (!r.owned) {
            const uintptr_t key = reinterpret_cast<uintptr_t>(r.surface.data);
            if (held.count(key) || busy.count(key)) {
                held.insert(key);
                ++it;
                continue;
            }
            busy.insert(key);
            held.insert(key);  // one request per surface and batch
        } else {
            size_t off;
            if (!pool.alloc(r.bytes, off)) {
                n_deferred++;
                break;  // admission in arrival order
            }
            r.pool_off = off;
            r.surface.data = pool.base + off;
        }
        batch.push_back(*it);
        it = queue.erase(it);
    }
    return batch;
}

// One pass over a batch on a lane: pool surfaces initialised, the fills
// drawn, pool surfaces read back into their callers' buffers.
int z2dgpu_server::draw_pass(Lane &L, std::vector<std::shared_ptr<Request>> &batch) {
    Ctx &c = *L.ctx;
    // a failed pass may have left work queued that reads the transfer buffer
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t n_owned = 0, in_bytes = 0, out_bytes = 0;
    for (auto &r : batch) {
        if (!r->owned) continue;
        n_owned++;
        in_bytes += al(r->init.size());
        if (r->out) out_bytes += al(r->exact);
    }
    const size_t desc_bytes = al(sizeof(Xfer) * 2 * n_owned);
    const size_t data_bytes = std::max(in_bytes, out_bytes);
    if (n_owned > 0) {
        if (L.xfer_dev.ensure(desc_bytes + data_bytes) || L.xfer_host.ensure(desc_bytes + data_bytes))
            return Z2D_ERR_OUT_OF_MEMORY;
        uint8_t *h = L.xfer_host.as<uint8_t>();
        Xfer *xin = reinterpret_cast<Xfer *>(h), *xout = xin + n_owned;
        size_t k = 0, o_in = 0, n_out = 0, o_out = 0;
        for (auto &r : batch) {
            if (!r->owned) continue;
            uint8_t *dev = reinterpret_cast<uint8_t *>(r->surface.data);
            if (!r->init.empty()) {
                memcpy(h + desc_bytes + o_in, r->init.data(), r->init.size());
                xin[k++] = Xfer{dev, (long long)r->init.size(), (long long)o_in, 0, 0};
                o_in += al(r->init.size());
            } else {
                xin[k++] = Xfer{dev, (long long)r->bytes, 0, 1, 0};
            }
            if (r->out) {
                xout[n_out++] = Xfer{dev, (long long)r->exact, (long long)o_out, 2, 0};
                o_out += al(r->exact);
            }
        }
        uint8_t *d = L.xfer_dev.as<uint8_t>();
        Z2D_CUDA(cudaMemcpyAsync(d, h, desc_bytes + in_bytes, cudaMemcpyHostToDevice, c.stream));
        k_xfer<<<(unsigned)n_owned, 256, 0, c.stream>>>(reinterpret_cast<const Xfer *>(d), d + desc_bytes);
        c.launches++;
        Z2D_CUDA(cudaGetLastError());
        // fill_jobs waits for the stream before it reuses its own staging,
        // and the transfer buffer is not touched again before the sync below
    }
    std::vector<z2d_job> jobs(batch.size());
    std::vector<z2d_node> nodes;
    std::vector<z2d_fill_cmd> cmds;
    size_t nn = 0, nc = 0;
    for (auto &r : batch) {
        nn += r->nodes.size();
        nc += r->cmds.size();
    }
    nodes.reserve(nn);
    cmds.reserve(nc);
    for (size_t j = 0; j < batch.size(); j++) {
        Request &r = *batch[j];
        jobs[j].surface = r.surface;
        jobs[j].cmd_offset = cmds.size();
        jobs[j].n_cmds = r.cmds.size();
        const uint64_t base = nodes.size();
        nodes.insert(nodes.end(), r.nodes.begin(), r.nodes.end());
        for (z2d_fill_cmd cm : r.cmds) {
            cm.node_offset += base;
            cmds.push_back(cm);
        }
    }
    int rc = fill_jobs(c, jobs.data(), jobs.size(), nodes.data(), nodes.size(), cmds.data(), cmds.size());
    if (rc) return rc;
    size_t n_out = 0;
    for (auto &r : batch)
        if (r->owned && r->out) n_out++;
    if (n_out > 0) {
        // (the descriptors were uploaded with the initial pixels)
        uint8_t *d = L.xfer_dev.as<uint8_t>();
        const Xfer *dxout = reinterpret_cast<const Xfer *>(d) + n_owned;
        k_xfer<<<(unsigned)n_out, 256, 0, c.stream>>>(dxout, d + desc_bytes);
        c.launches++;
        Z2D_CUDA(cudaGetLastError());
        Z2D_CUDA(cudaMemcpyAsync(L.xfer_host.as<uint8_t>() + desc_bytes, d + desc_bytes, out_bytes,
                                 cudaMemcpyDeviceToHost, c.stream));
    }
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    if (n_out > 0) {
        const uint8_t *h = L.xfer_host.as<uint8_t>() + desc_bytes;
        size_t o = 0;
        for (auto &r : batch) {
            if (!r->owned || !r->out) continue;
            memcpy(r->out, h + o, r->exact);
            o += al(r->exact);
        }
    }
    return Z2D_OK;
}

// Draws a batch; on failure every request is retried alone so that each
// gets its own status.
void z2dgpu_server::draw(Lane &L, std::vector<std::shared_ptr<Request>> &batch) {
    const int rc = draw_pass(L, batch);
    if (rc == Z2D_OK || batch.size() == 1) {
        const std::string err = rc ? last_error() : "";
        const auto now = Clock::now();
        std::lock_guard<std::mutex> lk(mu);
        for (auto &r : batch) {
            r->status = rc;
            r->error = err;
            r->t_done = now;
        }
        return;
    }
    for (auto &r : batch) {
        std::vector<std::shared_ptr<Request>> one{r};
        draw(L, one);
    }
}

void z2dgpu_server::lane_run(Lane &L) {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
        cv_work.wait(lk, [&] { return stopping || !queue.empty(); });
        if (queue.empty()) {
            if (stopping) return;
            continue;
        }
        // batching window: until the batch is full or the oldest request
        // has waited max_wait (a stopping server drains without waiting)
        if (max_wait.count() > 0 && queue.size() < max_batch) {
            const auto deadline = queue.front()->t_submit + max_wait;
            cv_work.wait_until(lk, deadline, [&] { return stopping || queue.size() >= max_batch; });
        }
        std::vector<std::shared_ptr<Request>> batch = take_batch();
        if (batch.empty()) {
            // every queued request waits for a busy surface or for pool
            // space: a completion (or a new request) wakes the lane
            cv_work.wait(lk);
            continue;
        }
        inflight++;
        max_inflight = std::max(max_inflight, inflight);
        lk.unlock();
        const auto t0 = Clock::now();
        draw(L, batch);
        // nothing of the batch may still run once its pool blocks and
        // surfaces are handed to other lanes (a failed pass returns early)
        cudaStreamSynchronize(L.ctx->stream);
        const double ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
        lk.lock();
        inflight--;
        for (auto &r : batch) {
            if (r->owned) pool.release(r->pool_off, r->bytes);
            else busy.erase(reinterpret_cast<uintptr_t>(r->surface.data));
        }
        n_batches++;
        n_requests += batch.size();
        busy_ms += ms;
        cv_done.notify_all();
        cv_work.notify_all();  // freed surfaces and pool space may admit queued requests
    }
}

static int submit_request(z2dgpu_server *s, std::shared_ptr<Request> r, uint64_t *ticket) {
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping) return Z2D_ERR_INVALID_STATE;
        r->id = s->next_id++;
        r->t_submit = Clock::now();
        s->by_id[r->id] = r;
        s->queue.push_back(r);
        *ticket = r->id;
    }
    s->cv_work.notify_one();
    return Z2D_OK;
}

extern "C" {

Z2D_API int z2dgpu_server_create2(z2dgpu_server **out, int device, const z2dgpu_server_opts *opts) {
    if (!out || !opts || opts->max_batch_jobs < 1 || opts->max_wait_us < 0 || opts->lanes < 1 || opts->lanes > 16 ||
        opts->pool_bytes < 0)
        return Z2D_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    auto *s = new z2dgpu_server();
    s->device = device;
    s->max_batch = (size_t)opts->max_batch_jobs;
    s->max_wait = std::chrono::microseconds(opts->max_wait_us);
    int prev = 0;
    cudaGetDevice(&prev);
    int rc = Z2D_OK;
    if (cudaSetDevice(device) != cudaSuccess) rc = Z2D_ERR_INVALID_ARGUMENT;
    if (rc == Z2D_OK && opts->pool_bytes > 0) {
        // the pool: what was asked, at most 40 GB, and no more than the free
        // HBM less a reserve of 1/8 of it for the lanes' scratch and others
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "cudaMemGetInfo");
        } else {
            unsigned long long want = std::min<unsigned long long>((unsigned long long)opts->pool_bytes, kPoolCap);
            want = std::min<unsigned long long>(want, (unsigned long long)(free_b - free_b / 8));
            want &= ~(unsigned long long)(kPoolAlign - 1);
            void *p = nullptr;
            if (want == 0 || cudaMalloc(&p, (size_t)want) != cudaSuccess) {
                set_error("server: the surface pool does not fit in free device memory");
                rc = Z2D_ERR_OUT_OF_MEMORY;
            } else {
                s->pool.base = static_cast<uint8_t *>(p);
                s->pool.cap = (size_t)want;
                s->pool.free_blocks[0] = (size_t)want;
            }
        }
    }
    for (int k = 0; rc == Z2D_OK && k < opts->lanes; k++) {
        auto L = std::make_unique<z2dgpu_server::Lane>();
        rc = z2dgpu_ctx_create(&L->ctx, device, nullptr);
        if (rc == Z2D_OK) s->lanes.push_back(std::move(L));
    }
    if (rc != Z2D_OK) {
        for (auto &L : s->lanes) z2dgpu_ctx_destroy(L->ctx);
        if (s->pool.base) cudaFree(s->pool.base);
        cudaSetDevice(prev);
        delete s;
        return rc;
    }
    cudaSetDevice(prev);
    for (auto &L : s->lanes) {
        z2dgpu_server::Lane *lp = L.get();
        L->th = std::thread([s, lp] { s->lane_run(*lp); });
    }
    *out = s;
    return Z2D_OK;
}

Z2D_API int z2dgpu_server_create(z2dgpu_server **out, int device, int32_t max_batch_jobs, int32_t max_wait_us) {
    const z2dgpu_server_opts o{max_batch_jobs, max_wait_us, 2, 0};
    return z2dgpu_server_create2(out, device, &o);
}

Z2D_API int z2dgpu_server_submit(z2dgpu_server *s, const z2d_surface *surface, const z2d_node *nodes, size_t n_nodes,
                                 const z2d_fill_cmd *cmds, size_t n_cmds, uint64_t *ticket) {
    if (!s || !surface || !ticket) return Z2D_ERR_INVALID_ARGUMENT;
    if (surface->location != Z2D_MEM_DEVICE) {
        set_error("server: surfaces must be in device memory");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    auto r = std::make_shared<Request>();
    r->surface = *surface;
    const int rc = copy_request(*r, nodes, n_nodes, cmds, n_cmds);
    if (rc) {
        set_error("server: malformed request");
        return rc;
    }
    return submit_request(s, r, ticket);
}

Z2D_API int z2dgpu_server_submit_new(z2dgpu_server *s, int32_t format, int32_t width, int32_t height, const void *init,
                                     void *out, const z2d_node *nodes, size_t n_nodes, const z2d_fill_cmd *cmds,
                                     size_t n_cmds, uint64_t *ticket) {
    if (!s || !ticket) return Z2D_ERR_INVALID_ARGUMENT;
    if (format < Z2D_FORMAT_ARGB || format > Z2D_FORMAT_ALPHA1) {
        set_error("server: bad surface format");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    if (width < 1 || height < 1) {
        set_error(width < 1 ? "InvalidWidth" : "InvalidHeight");
        return Z2D_ERR_INVALID_DIMENSIONS;
    }
    if (!s->pool.base) {
        set_error("server: created without a surface pool");
        return Z2D_ERR_INVALID_STATE;
    }
    auto r = std::make_shared<Request>();
    const size_t bytes = ((size_t)width * (size_t)height * (size_t)fmt_bits(format) + 7) / 8;
    // packed formats are updated with 32-bit word operations: whole words
    r->bytes = (bytes + 3) & ~(size_t)3;
    r->exact = bytes;
    if (r->bytes > s->pool.cap) {
        set_error("server: the surface is larger than the whole pool");
        return Z2D_ERR_OUT_OF_MEMORY;
    }
    r->owned = true;
    r->surface = z2d_surface{format, width, height, Z2D_MEM_DEVICE, nullptr};
    if (init) r->init.assign(static_cast<const uint8_t *>(init), static_cast<const uint8_t *>(init) + bytes);
    r->out = out;
    const int rc = copy_request(*r, nodes, n_nodes, cmds, n_cmds);
    if (rc) {
        set_error("server: malformed request");
        return rc;
    }
    return submit_request(s, r, ticket);
}

Z2D_API int z2dgpu_server_wait(z2dgpu_server *s, uint64_t ticket, int32_t timeout_ms, double *latency_us) {
    if (!s) return Z2D_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->by_id.find(ticket);
    if (it == s->by_id.end()) {
        set_error("server: unknown ticket");
        return Z2D_ERR_INVALID_ARGUMENT;
    }
    std::shared_ptr<Request> r = it->second;
    auto done = [&] { return r->status >= 0; };
    if (timeout_ms < 0) s->cv_done.wait(lk, done);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) return Z2D_ERR_TIMEOUT;
    s->by_id.erase(ticket);
    if (latency_us) *latency_us = std::chrono::duration<double, std::micro>(r->t_done - r->t_submit).count();
    if (r->status) set_error(r->error.c_str());
    return r->status;
}

Z2D_API int z2dgpu_server_stats(z2dgpu_server *s, uint64_t *batches, uint64_t *requests, double *busy_ms) {
    if (!s) return Z2D_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    if (batches) *batches = s->n_batches;
    if (requests) *requests = s->n_requests;
    if (busy_ms) *busy_ms = s->busy_ms;
    return Z2D_OK;
}

Z2D_API int z2dgpu_server_info(z2dgpu_server *s, z2dgpu_server_stats_t *out) {
    if (!s || !out) return Z2D_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    out->batches = s->n_batches;
    out->requests = s->n_requests;
    out->deferred = s->n_deferred;
    out->busy_ms = s->busy_ms;
    out->lanes = (int32_t)s->lanes.size();
    out->max_inflight = s->max_inflight;
    out->pool_bytes = (long long)s->pool.cap;
    out->pool_peak_bytes = (long long)s->pool.peak;
    return Z2D_OK;
}

Z2D_API int z2dgpu_server_destroy(z2dgpu_server *s) {
    if (!s) return Z2D_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (auto &L : s->lanes)
        if (L->th.joinable()) L->th.join();
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    for (auto &L : s->lanes) {
        L->xfer_dev.release();
        L->xfer_host.release();
        z2dgpu_ctx_destroy(L->ctx);
    }
    if (s->pool.base) cudaFree(s->pool.base);
    cudaSetDevice(prev);
    delete s;
    return Z2D_OK;
}

}  // extern "C"
