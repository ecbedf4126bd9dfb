// server.cu -- a request queue in front of z2dgpu_fill_jobs.
//
// Callers submit fill requests (one device surface and its ordered fill
// commands each) from any thread and wait for them by ticket.  One worker
// thread per server owns a context and its stream; it takes the requests
// that arrived within a batching window (or until the batch is full), draws
// them in one z2dgpu_fill_jobs pass and completes them.  Requests are copied
// at submit time (nodes, commands, patterns, gradients and their stops), so
// the caller's buffers may be reused as soon as submit returns; the
// surfaces must stay valid until the request completes.
//
// Ordering: requests on the same surface are drawn in submission order (a
// batch never holds two requests for one surface: the second starts the
// next batch).  Requests on different surfaces are independent.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
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

struct Request {
    uint64_t id = 0;
    z2d_surface surface{};
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

}  // namespace
}  // namespace z2dg

using namespace z2dg;

struct z2dgpu_server {
    z2dgpu_ctx *ctx = nullptr;
    int device = 0;
    size_t max_batch = 1;
    std::chrono::microseconds max_wait{0};
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> by_id;
    uint64_t next_id = 1;
    bool stopping = false;
    uint64_t n_batches = 0, n_requests = 0;
    double busy_ms = 0;

    void run();
    void draw(std::vector<std::shared_ptr<Request>> &batch);
};

// Draws a batch; on failure every request is retried alone so that each
// gets its own status.
void z2dgpu_server::draw(std::vector<std::shared_ptr<Request>> &batch) {
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
        for (z2d_fill_cmd c : r.cmds) {
            c.node_offset += base;
            cmds.push_back(c);
        }
    }
    int rc = fill_jobs(*ctx, jobs.data(), jobs.size(), nodes.data(), nodes.size(), cmds.data(), cmds.size());
    if (rc == Z2D_OK) {
        const cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamSynchronize");
    }
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
        draw(one);
    }
}

void z2dgpu_server::run() {
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
        const auto deadline = queue.front()->t_submit + max_wait;
        cv_work.wait_until(lk, deadline, [&] { return stopping || queue.size() >= max_batch; });
        std::vector<std::shared_ptr<Request>> batch;
        std::unordered_set<uintptr_t> surfaces;
        while (!queue.empty() && batch.size() < max_batch) {
            const uintptr_t key = reinterpret_cast<uintptr_t>(queue.front()->surface.data);
            if (!surfaces.insert(key).second) break;  // same surface: next batch, in order
            batch.push_back(queue.front());
            queue.pop_front();
        }
        lk.unlock();
        const auto t0 = Clock::now();
        draw(batch);
        const double ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
        lk.lock();
        n_batches++;
        n_requests += batch.size();
        busy_ms += ms;
        cv_done.notify_all();
    }
}

extern "C" {

Z2D_API int z2dgpu_server_create(z2dgpu_server **out, int device, int32_t max_batch_jobs, int32_t max_wait_us) {
    if (!out || max_batch_jobs < 1 || max_wait_us < 0) return Z2D_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    auto *s = new z2dgpu_server();
    const int rc = z2dgpu_ctx_create(&s->ctx, device, nullptr);
    if (rc) {
        delete s;
        return rc;
    }
    s->device = device;
    s->max_batch = (size_t)max_batch_jobs;
    s->max_wait = std::chrono::microseconds(max_wait_us);
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return Z2D_OK;
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

Z2D_API int z2dgpu_server_destroy(z2dgpu_server *s) {
    if (!s) return Z2D_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    z2dgpu_ctx_destroy(s->ctx);
    delete s;
    return Z2D_OK;
}

}  // extern "C"
