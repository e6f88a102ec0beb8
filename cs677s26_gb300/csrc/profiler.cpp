// Kernel timing registry behind vj_profile_* (no reference counterpart: the
// reference times whole calls with cudaEvents in its compare modes,
// src/main.cu:1157-1188).
#include "profiler.h"

#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.h"

namespace vjgb {
namespace {

struct Rec {
    const char* name;
    cudaEvent_t start, stop;
};

std::atomic<bool> g_on{false};
std::mutex g_mu;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_free;

cudaEvent_t take_event() {
    if (!g_free.empty()) {
        cudaEvent_t e = g_free.back();
        g_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

}  // namespace

bool profiling() { return g_on.load(std::memory_order_relaxed); }

int prof_begin(const char* name, cudaStream_t s) {
    if (!profiling()) return -1;
    std::lock_guard<std::mutex> lk(g_mu);
    Rec r{name, take_event(), take_event()};
    if (!r.start || !r.stop) return -1;
    cudaEventRecord(r.start, s);
    g_recs.push_back(r);
    return static_cast<int>(g_recs.size()) - 1;
}

void prof_end(int slot, cudaStream_t s) {
    if (slot < 0) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (slot < static_cast<int>(g_recs.size())) cudaEventRecord(g_recs[static_cast<size_t>(slot)].stop, s);
}

}  // namespace vjgb

using namespace vjgb;

extern "C" {

int vj_profile_enable(int on) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_on.store(on != 0);
    return ok();
}

int vj_profile_read(vj_profile_entry* out, int capacity, int* count, int reset) {
    if (!count || capacity < 0 || (capacity > 0 && !out)) return set_error(VJ_INVALID_ARG, "vj_profile_read: bad arguments");
    std::lock_guard<std::mutex> lk(g_mu);
    std::map<std::string, std::pair<int64_t, double>> agg;
    for (const Rec& r : g_recs) {
        if (cudaEventSynchronize(r.stop) != cudaSuccess) continue;
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, r.start, r.stop) != cudaSuccess) continue;
        auto& a = agg[r.name];
        a.first += 1;
        a.second += ms;
    }
    int k = 0;
    for (const auto& kv : agg) {
        if (k < capacity) {
            vj_profile_entry& e = out[k];
            std::memset(&e, 0, sizeof(e));
            std::strncpy(e.name, kv.first.c_str(), sizeof(e.name) - 1);
            e.launches = kv.second.first;
            e.total_ms = kv.second.second;
        }
        ++k;
    }
    *count = k;
    if (reset) {
        for (const Rec& r : g_recs) {
            g_free.push_back(r.start);
            g_free.push_back(r.stop);
        }
        g_recs.clear();
    }
    return ok();
}

}  // extern "C"
