// Continuous-batching detection server (vj_server_*).
//
// Threads: the callers of vj_server_submit / vj_server_wait, and one thread
// per worker.  A worker owns a vj_detector and a CUDA stream.  When it is
// free it takes, in arrival order, every queued request that fits its share
// of the HBM budget (and the batch pixel cap, if set) and runs them as one
// vj_detect_batch launch (one
// persistent kernel over all their pyramid levels, grouping included);
// requests that arrive while batches are on the GPU wait for the next free
// worker.  By default every worker's kernel fills the GPU (all resident CTAs
// per SM) and the kernels follow one another on the device through a shared
// launch chain, so a lone request gets the whole GPU, while one worker's host
// work and uploads overlap another's kernel.  A configured blocksPerSM below
// the full residency instead splits the SMs and lets the workers' kernels
// run side by side.
//
// Request images are copied at submit into pinned host buffers drawn from a
// pool, so the worker's upload is a DMA from pinned memory and the caller's
// buffer is free as soon as submit returns.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "common.h"
#include "launch_chain.h"

namespace vjgb {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Pinned host buffers reused across requests, by capacity.
class PinnedPool {
public:
    ~PinnedPool() {
        for (auto& kv : free_) cudaFreeHost(kv.second);
    }
    uint8_t* take(size_t bytes) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            auto it = free_.lower_bound(bytes);
            if (it != free_.end() && it->first <= 2 * bytes + 65536) {
                uint8_t* p = it->second;
                cap_[p] = it->first;
                free_.erase(it);
                return p;
            }
        }
        void* p = nullptr;
        if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) return nullptr;
        std::lock_guard<std::mutex> lk(mu_);
        cap_[static_cast<uint8_t*>(p)] = bytes;
        return static_cast<uint8_t*>(p);
    }
    void give(uint8_t* p) {
        if (!p) return;
        std::lock_guard<std::mutex> lk(mu_);
        auto it = cap_.find(p);
        const size_t c = it == cap_.end() ? 0 : it->second;
        if (it != cap_.end()) cap_.erase(it);
        free_.emplace(c, p);
    }

private:
    std::mutex mu_;
    std::multimap<size_t, uint8_t*> free_;
    std::map<uint8_t*, size_t> cap_;
};

struct Request {
    uint64_t ticket = 0;
    uint8_t* pix = nullptr;  // pinned copy, w x h, stride w
    int w = 0, h = 0;
    int64_t bytes = 0;       // admission estimate
    int64_t pixels = 0;
    Clock::time_point tSubmit, tDone;
    bool done = false;
    int status = VJ_OK;
    std::vector<vj_detection> result;
};

}  // namespace
}  // namespace vjgb

using namespace vjgb;

struct vj_server {
    vj_server_config cfg{};
    int64_t workerBudget = 0;
    std::vector<vj_detector*> dets;
    std::vector<cudaStream_t> streams;
    std::vector<std::thread> threads;
    PinnedPool pool;
    LaunchChain chain;

    std::mutex mu;
    std::condition_variable cvWork;  // workers: queue not empty or stopping
    std::condition_variable cvDone;  // waiters: some request finished
    std::deque<std::shared_ptr<Request>> queue;
    std::map<uint64_t, std::shared_ptr<Request>> live;
    uint64_t nextTicket = 1;
    bool stopping = false;
    int64_t admitted = 0;  // estimates of the requests in flight

    // statistics since the last reset
    int64_t submitted = 0, completed = 0, failed = 0, batches = 0, batchImages = 0, peakAdmitted = 0;
    std::vector<double> latMs;
    bool haveFirst = false;
    Clock::time_point tFirst, tLast;
};

namespace {

void worker_loop(vj_server* S, int wi) {
    vj_detector* det = S->dets[static_cast<size_t>(wi)];
    cudaStream_t stream = S->streams[static_cast<size_t>(wi)];
    const vj_server_config& c = S->cfg;
    std::vector<const uint8_t*> ptrs;
    std::vector<int> ws, hs, counts;
    std::vector<vj_detection> out;
    const int capPer = std::max(1, c.maxDetections);
    for (;;) {
        std::vector<std::shared_ptr<Request>> batch;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cvWork.wait(lk, [&] { return S->stopping || !S->queue.empty(); });
            if (S->queue.empty()) return;  // stopping and drained
            int64_t bytes = 0, pixels = 0;
            while (!S->queue.empty() && static_cast<int>(batch.size()) < c.maxBatchImages) {
                const auto& r = S->queue.front();
                if (!batch.empty() && (bytes + r->bytes > S->workerBudget ||
                                       (c.maxBatchPixels > 0 && pixels + r->pixels > c.maxBatchPixels)))
                    break;
                bytes += r->bytes;
                pixels += r->pixels;
                batch.push_back(r);
                S->queue.pop_front();
            }
            S->admitted += bytes;
            S->peakAdmitted = std::max(S->peakAdmitted, S->admitted);
            if (!S->queue.empty()) S->cvWork.notify_one();
        }
        const int n = static_cast<int>(batch.size());
        ptrs.resize(n);
        ws.resize(n);
        hs.resize(n);
        counts.assign(n, 0);
        for (int i = 0; i < n; ++i) {
            ptrs[i] = batch[i]->pix;
            ws[i] = batch[i]->w;
            hs[i] = batch[i]->h;
        }
        out.resize(static_cast<size_t>(n) * capPer);
        const int st = vj_detect_batch(det, n, ptrs.data(), ws.data(), hs.data(), ws.data(), 0, c.scaleFactor,
                                       c.minNeighbors, c.minObjectSize, c.maxDetections, c.applyGrouping, out.data(),
                                       capPer, counts.data(), stream);
        const auto tDone = Clock::now();
        {
            std::lock_guard<std::mutex> lk(S->mu);
            int64_t bytes = 0;
            for (int i = 0; i < n; ++i) {
                Request& r = *batch[i];
                bytes += r.bytes;
                r.status = st;
                if (st == VJ_OK)
                    r.result.assign(out.begin() + static_cast<size_t>(i) * capPer,
                                    out.begin() + static_cast<size_t>(i) * capPer + counts[i]);
                r.tDone = tDone;
                r.done = true;
                S->pool.give(r.pix);
                r.pix = nullptr;
                if (st == VJ_OK) {
                    ++S->completed;
                    S->latMs.push_back(ms_between(r.tSubmit, tDone));
                } else {
                    ++S->failed;
                }
            }
            S->admitted -= bytes;
            ++S->batches;
            S->batchImages += n;
            S->tLast = tDone;
        }
        S->cvDone.notify_all();
    }
}

double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    // nearest-rank percentile
    size_t k = static_cast<size_t>(p / 100.0 * static_cast<double>(v.size()) + 0.999999);
    k = std::min(std::max<size_t>(k, 1), v.size());
    return v[k - 1];
}

}  // namespace

extern "C" {

int vj_server_create(const vj_server_config* cfg, const vj_haar_feature* features, int64_t featureCount,
                     const vj_stump4* stumps, int64_t stumpCount, const vj_cascade_stage* stages, int64_t stageCount,
                     vj_server** out) {
    if (!cfg || !out) return set_error(VJ_INVALID_ARG, "vj_server_create: null argument");
    *out = nullptr;
    vj_server_config c = *cfg;
    if (c.workers < 1 || c.workers > 16 || c.maxBatchImages < 1 || c.hbmBudgetBytes <= 0 || !(c.scaleFactor > 1.0f) ||
        c.minObjectSize < 1 || c.maxDetections < 1 || c.blocksPerSM < 0 || c.maxBatchPixels < 0)
        return set_error(VJ_INVALID_ARG, "vj_server_create: bad configuration");
    auto S = std::make_unique<vj_server>();
    S->cfg = c;
    S->workerBudget = c.hbmBudgetBytes / c.workers;
    int st = VJ_OK;
    for (int i = 0; i < c.workers && st == VJ_OK; ++i) {
        vj_detector* d = nullptr;
        st = vj_detector_create(c.winW, c.winH, c.maxImageW, c.maxImageH, c.maxDetections, &d);
        if (st != VJ_OK) break;
        S->dets.push_back(d);
        st = vj_detector_set_model(d, features, featureCount, stumps, stumpCount, stages, stageCount);
        if (st != VJ_OK) break;
        vj_detect_config dc{};
        st = vj_detector_get_config(d, &dc);
        if (c.tileRows) dc.tileRows = c.tileRows;
        if (c.tileStumps) dc.tileStumps = c.tileStumps;
        if (st == VJ_OK) st = vj_detector_set_config(d, &dc);
        int fit = 0;
        if (st == VJ_OK) st = vj_detector_occupancy(d, &fit);
        if (st != VJ_OK) break;
        dc.blocksPerSM = c.blocksPerSM > 0 ? c.blocksPerSM : fit;
        st = vj_detector_set_config(d, &dc);
        // full-residency kernels take turns on the device; split ones may overlap
        if (st == VJ_OK && dc.blocksPerSM * c.workers > fit) st = detector_set_launch_chain(d, &S->chain);
        if (st == VJ_OK) st = vj_detector_reserve(d, S->workerBudget);
        if (st != VJ_OK) break;
        cudaStream_t s = nullptr;
        const cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            st = set_error(VJ_CUDA_ERROR, std::string("vj_server_create: stream: ") + cudaGetErrorString(e));
            break;
        }
        S->streams.push_back(s);
    }
    if (st != VJ_OK) {
        for (auto* d : S->dets) vj_detector_destroy(d);
        for (auto s : S->streams) cudaStreamDestroy(s);
        return st;
    }
    vj_server* raw = S.release();
    for (int i = 0; i < c.workers; ++i) raw->threads.emplace_back(worker_loop, raw, i);
    *out = raw;
    return ok();
}

int vj_server_submit(vj_server* s, const uint8_t* image, int w, int h, int stride, uint64_t* ticket) {
    if (!s || !image || !ticket || w <= 0 || h <= 0 || stride < w || w > s->cfg.maxImageW || h > s->cfg.maxImageH)
        return set_error(VJ_INVALID_ARG, "vj_server_submit: bad arguments");
    int64_t bytes = 0;
    int st = vj_detect_estimate_bytes(s->cfg.winW, s->cfg.winH, w, h, s->cfg.scaleFactor, s->cfg.minObjectSize,
                                      s->cfg.maxDetections, &bytes);
    if (st != VJ_OK) return st;
    if (bytes > s->workerBudget)
        return set_error(VJ_OUT_OF_MEMORY, "vj_server_submit: image needs " + std::to_string(bytes) +
                                               " device bytes, more than a worker's budget");
    auto r = std::make_shared<Request>();
    r->pix = s->pool.take(static_cast<size_t>(w) * h);
    if (!r->pix) return set_error(VJ_OUT_OF_MEMORY, "vj_server_submit: pinned buffer");
    for (int y = 0; y < h; ++y)
        std::memcpy(r->pix + static_cast<size_t>(y) * w, image + static_cast<size_t>(y) * stride, static_cast<size_t>(w));
    r->w = w;
    r->h = h;
    r->bytes = bytes;
    r->pixels = static_cast<int64_t>(w) * h;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping) {
            s->pool.give(r->pix);
            return set_error(VJ_RUNTIME_ERROR, "vj_server_submit: server is stopping");
        }
        r->ticket = s->nextTicket++;
        r->tSubmit = Clock::now();
        if (!s->haveFirst) {
            s->haveFirst = true;
            s->tFirst = r->tSubmit;
        }
        ++s->submitted;
        s->live[r->ticket] = r;
        s->queue.push_back(r);
        *ticket = r->ticket;
    }
    s->cvWork.notify_one();
    return ok();
}

int vj_server_poll(vj_server* s, uint64_t ticket, int* done) {
    if (!s || !done) return set_error(VJ_INVALID_ARG, "vj_server_poll: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) return set_error(VJ_INVALID_ARG, "vj_server_poll: unknown ticket");
    *done = it->second->done ? 1 : 0;
    return ok();
}

int vj_server_wait(vj_server* s, uint64_t ticket, int timeoutMs, vj_detection* out, int capacity, int* count) {
    if (!s || !count || capacity < 0 || (capacity > 0 && !out))
        return set_error(VJ_INVALID_ARG, "vj_server_wait: bad arguments");
    *count = 0;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) return set_error(VJ_INVALID_ARG, "vj_server_wait: unknown ticket");
    std::shared_ptr<Request> r = it->second;
    auto ready = [&] { return r->done; };
    if (timeoutMs < 0) {
        s->cvDone.wait(lk, ready);
    } else if (!s->cvDone.wait_for(lk, std::chrono::milliseconds(timeoutMs), ready)) {
        return set_error(VJ_RUNTIME_ERROR, "vj_server_wait: timed out");
    }
    s->live.erase(ticket);
    if (r->status != VJ_OK) return set_error(r->status, "vj_server_wait: the request's batch failed");
    const int k = std::min(static_cast<int>(r->result.size()), capacity);
    if (k > 0) std::memcpy(out, r->result.data(), sizeof(vj_detection) * k);
    *count = k;
    return ok();
}

int vj_server_get_stats(vj_server* s, vj_server_stats* out) {
    if (!s || !out) return set_error(VJ_INVALID_ARG, "vj_server_get_stats: null argument");
    std::vector<double> lat;
    vj_server_stats o{};
    {
        std::lock_guard<std::mutex> lk(s->mu);
        lat = s->latMs;
        o.submitted = s->submitted;
        o.completed = s->completed;
        o.failed = s->failed;
        o.batches = s->batches;
        o.meanBatchImages = s->batches ? static_cast<double>(s->batchImages) / static_cast<double>(s->batches) : 0.0;
        o.elapsedS = s->haveFirst && s->completed ? ms_between(s->tFirst, s->tLast) * 1e-3 : 0.0;
        o.peakAdmittedBytes = s->peakAdmitted;
    }
    double sum = 0.0, mx = 0.0;
    for (double v : lat) {
        sum += v;
        mx = std::max(mx, v);
    }
    o.meanMs = lat.empty() ? 0.0 : sum / static_cast<double>(lat.size());
    o.maxMs = mx;
    o.p50Ms = percentile(lat, 50.0);
    o.p99Ms = percentile(lat, 99.0);
    o.p999Ms = percentile(lat, 99.9);
    o.imagesPerS = o.elapsedS > 0.0 ? static_cast<double>(o.completed) / o.elapsedS : 0.0;
    int64_t dev = 0;
    for (auto* d : s->dets) {
        int64_t b = 0;
        if (vj_detector_device_bytes(d, &b) == VJ_OK) dev += b;
    }
    o.deviceBytes = dev;
    *out = o;
    return ok();
}

int vj_server_reset_stats(vj_server* s) {
    if (!s) return set_error(VJ_INVALID_ARG, "vj_server_reset_stats: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    s->submitted = s->completed = s->failed = s->batches = s->batchImages = 0;
    s->peakAdmitted = s->admitted;
    s->latMs.clear();
    s->haveFirst = false;
    return ok();
}

int vj_server_destroy(vj_server* s) {
    if (!s) return ok();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cvWork.notify_all();
    for (auto& t : s->threads) t.join();
    for (auto* d : s->dets) vj_detector_destroy(d);
    for (auto st : s->streams) cudaStreamDestroy(st);
    if (s->chain.last) cudaEventDestroy(s->chain.last);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto& kv : s->live)
            if (kv.second->pix) s->pool.give(kv.second->pix);
        s->live.clear();
    }
    delete s;
    return ok();
}

}  // extern "C"
