// tune.cu -- the autotuner of the persistent rasteriser's schedule.
//
// k_raster runs as a persistent grid that pulls work items from a device
// queue (fill.cu).  Three things shape its schedule: how many CTAs of 4
// warps stay resident per SM (more hide latency, fewer leave each warp more
// L1), the size of an item (a whole tile, whose four rows share the band's
// data in one SM's L1, or a single tile row, which balances better when
// rows differ in cost) and the order of the queue (tile order, or
// longest-band-first, an LPT schedule that keeps the slowest items from
// starting last).  Which is fastest depends on the workload: how many tiles
// a pass has and how many fills a band's list holds.
//
// The fourth candidate shape is no persistence at all: one CTA per tile, as
// many CTAs as tiles, in queue order, scheduled by the hardware.
//
// The tuner keys a pass by (one surface or many, log2 of its tiles, log2 of
// the mean fills per band list).  The first passes of a new key each run a
// different candidate schedule with CUDA events around the raster launch;
// once every candidate has run, the fastest is kept for the key.  Decisions
// are cached in a JSON file (raster_tune.json beside libz2dgpu.so, or the
// path in Z2D_TUNE_FILE) and loaded on first use, so a later process starts
// from them.  Z2D_TUNE=off keeps the default schedule (one CTA per tile, in
// tile order).  Every schedule draws the same pixels: tiles are disjoint and
// each row's fills run in call order whatever the queue order.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "z2d_internal.h"

namespace z2dg {

namespace {

struct Candidate {
    int ctas, order, cta_items;
};
// CTAs per SM: -1 = not persistent (one CTA per tile, dispatched in queue
// order), 0 = as many as fit (6 for k_raster), else that many
constexpr Candidate kCandidates[] = {{-1, 0, 1}, {-1, 1, 1}, {0, 0, 0}, {0, 1, 0},
                                     {0, 0, 1}, {0, 1, 1}, {4, 0, 0}, {2, 1, 0}};
constexpr int kNumCandidates = sizeof(kCandidates) / sizeof(kCandidates[0]);

struct Entry {
    int best = -1;
    double ms[kNumCandidates] = {};
    int n[kNumCandidates] = {};
};

std::mutex g_mu;
std::map<TuneKey, Entry> g_table;
bool g_loaded = false;
int g_mode = -1;  // 1 on, 0 off

std::string tune_path() {
    if (const char *p = std::getenv("Z2D_TUNE_FILE")) return p;
    Dl_info info;
    if (dladdr(reinterpret_cast<void *>(&tune_path), &info) && info.dli_fname) {
        std::string lib = info.dli_fname;
        const size_t slash = lib.find_last_of('/');
        return (slash == std::string::npos ? std::string(".") : lib.substr(0, slash)) + "/raster_tune.json";
    }
    return "raster_tune.json";
}

// {"multi": m, "tiles": t, "load": l, "ctas": c, "order": o, "cta_items": i, "ms": x} per line
void load_locked() {
    g_loaded = true;
    FILE *f = std::fopen(tune_path().c_str(), "r");
    if (!f) return;
    char line[512];
    while (std::fgets(line, sizeof line, f)) {
        TuneKey k{};
        int ctas = 0, order = 0, items = 0;
        double ms = 0;
        if (std::sscanf(line,
                        " {\"multi\": %d, \"tiles\": %d, \"load\": %d, \"ctas\": %d, \"order\": %d, \"cta_items\": %d, "
                        "\"ms\": %lf",
                        &k.multi, &k.tiles, &k.load, &ctas, &order, &items, &ms) != 7)
            continue;
        for (int i = 0; i < kNumCandidates; i++)
            if (kCandidates[i].ctas == ctas && kCandidates[i].order == order && kCandidates[i].cta_items == items)
                g_table[k].best = i;
    }
    std::fclose(f);
}

void save_locked() {
    const std::string path = tune_path();
    const std::string tmp = path + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "w");
    if (!f) return;  // a read-only install keeps its decisions in memory
    for (const auto &kv : g_table) {
        if (kv.second.best < 0) continue;
        const Entry &e = kv.second;
        const Candidate &c = kCandidates[e.best];
        const double ms = e.n[e.best] ? e.ms[e.best] / e.n[e.best] : 0.0;
        std::fprintf(f,
                     "{\"multi\": %d, \"tiles\": %d, \"load\": %d, \"ctas\": %d, \"order\": %d, \"cta_items\": %d, "
                     "\"ms\": %.4f, \"candidates_ms\": [",
                     kv.first.multi, kv.first.tiles, kv.first.load, c.ctas, c.order, c.cta_items, ms);
        for (int i = 0; i < kNumCandidates; i++)  // every candidate's time, for the record (0: not measured here)
            std::fprintf(f, "%s%.4f", i ? ", " : "", e.n[i] ? e.ms[i] / e.n[i] : 0.0);
        std::fprintf(f, "]}\n");
    }
    std::fclose(f);
    std::rename(tmp.c_str(), path.c_str());
}

int mode_locked() {
    if (g_mode < 0) {
        const char *m = std::getenv("Z2D_TUNE");
        g_mode = (m && (std::strcmp(m, "off") == 0 || std::strcmp(m, "0") == 0)) ? 0 : 1;
    }
    return g_mode;
}

}  // namespace

TuneKey tune_key(int32_t n_jobs, long long n_tiles, long long n_slots, long long n_gbands) {
    TuneKey k{};
    k.multi = n_jobs > 1 ? 1 : 0;
    k.tiles = n_tiles > 0 ? (int)std::log2((double)n_tiles) : 0;
    const double load = n_gbands > 0 ? (double)n_slots / (double)n_gbands : 0.0;
    k.load = (int)std::log2(1.0 + load);
    return k;
}

RasterPlan tune_pick(const TuneKey &k) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!mode_locked()) return RasterPlan{-1, 0, 1, -1};
    if (!g_loaded) load_locked();
    Entry &e = g_table[k];
    const auto plan = [](int i, int cand) {
        return RasterPlan{kCandidates[i].ctas, kCandidates[i].order, kCandidates[i].cta_items, cand};
    };
    if (e.best >= 0) return plan(e.best, -1);
    for (int i = 0; i < kNumCandidates; i++)
        if (e.n[i] == 0) return plan(i, i);
    return RasterPlan{-1, 0, 1, -1};
}

void tune_report(const TuneKey &k, int candidate, float ms) {
    if (candidate < 0 || candidate >= kNumCandidates || !(ms > 0.0f)) return;
    std::lock_guard<std::mutex> lk(g_mu);
    Entry &e = g_table[k];
    if (e.best >= 0) return;
    e.ms[candidate] += ms;
    e.n[candidate] += 1;
    for (int i = 0; i < kNumCandidates; i++)
        if (e.n[i] == 0) return;
    int best = 0;
    for (int i = 1; i < kNumCandidates; i++)
        if (e.ms[i] / e.n[i] < e.ms[best] / e.n[best]) best = i;
    e.best = best;
    save_locked();
}

int tune_state(const TuneKey &k, int *ctas, int *order, int *cta_items) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!mode_locked()) return -1;
    if (!g_loaded) load_locked();
    auto it = g_table.find(k);
    if (it == g_table.end() || it->second.best < 0) return 0;
    *ctas = kCandidates[it->second.best].ctas;
    *order = kCandidates[it->second.best].order;
    *cta_items = kCandidates[it->second.best].cta_items;
    return 1;
}

// Collects the timings of earlier passes whose raster launch has finished.
void Ctx::tune_collect(bool wait) {
    for (size_t i = 0; i < tune_pending.size();) {
        TunePending &p = tune_pending[i];
        if (!wait && cudaEventQuery(p.stop) == cudaErrorNotReady) {
            i++;
            continue;
        }
        float ms = 0.0f;
        if (cudaEventSynchronize(p.stop) == cudaSuccess && cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess)
            tune_report(p.key, p.candidate, ms);
        cudaEventDestroy(p.start);
        cudaEventDestroy(p.stop);
        tune_pending[i] = tune_pending.back();
        tune_pending.pop_back();
    }
}

}  // namespace z2dg
